"""The threshold-pair search, mirroring the reference's ``src/dto``.

optimize            src/dto/optimize_main.rs:53-118
process_threshold_pairs  src/dto/process_threshold_pairs.rs:71-131
compute_population_size  src/dto/compute_population_size.rs:66-104
OptimizationResultRecord / OptimizationResult / FeatureSets
                    src/dto/results_objects.rs:7-32

The search runs in libdto.so on the GPU (dto_optimize, dto_grid_dump); this
module only converts between the reference's objects and the C ABI.
"""
import os
import threading

import numpy as np

from .feature_lists import PermutedRankedFeatureList, RankedFeatureList, dense_ids
from .engine import Engine

_state = threading.local()
_lock = threading.Lock()
_default = {}


def default_engine(device=None):
    """Process-wide engine per device (created on first use)."""
    dev = int(os.environ.get("DTO_DEVICE", "0")) if device is None else int(device)
    with _lock:
        eng = _default.get(dev)
        if eng is None:
            eng = Engine(dev)
            _default[dev] = eng
        return eng


class FeatureSets:
    """FeatureSets::None or FeatureSets::Both(set1, set2) (results_objects.rs:26-32)."""

    def __init__(self, set1=None, set2=None):
        self.set1 = set1
        self.set2 = set2

    @classmethod
    def none(cls):
        return cls()

    @classmethod
    def both(cls, set1, set2):
        return cls(set1, set2)

    def is_none(self):
        return self.set1 is None

    def __eq__(self, other):
        return isinstance(other, FeatureSets) and (self.set1, self.set2) == (other.set1, other.set2)


class OptimizationResultRecord:
    """One cell's record (results_objects.rs:7-24)."""

    __slots__ = ("rank1", "rank2", "set1_len", "set2_len", "population_size",
                 "intersection_size", "pvalue", "permuted", "feature_sets")

    def __init__(self, rank1, rank2, set1_len, set2_len, population_size, intersection_size,
                 pvalue, permuted, feature_sets=None):
        def opt_int(v):
            return None if v is None else int(v)
        self.rank1 = opt_int(rank1)
        self.rank2 = opt_int(rank2)
        self.set1_len = opt_int(set1_len)
        self.set2_len = opt_int(set2_len)
        self.population_size = opt_int(population_size)
        self.intersection_size = opt_int(intersection_size)
        self.pvalue = float(pvalue)
        self.permuted = bool(permuted)
        self.feature_sets = feature_sets if feature_sets is not None else FeatureSets.none()

    @classmethod
    def pvalue_only(cls, pvalue, permuted=True):
        """A permuted task's record when only its minimum p-value was gathered
        (run_multi_node with gather="minp"): the other fields are None."""
        return cls(None, None, None, None, None, None, pvalue, permuted)

    @classmethod
    def from_abi(cls, rec, feature_sets=None):
        g = rec.get if isinstance(rec, dict) else (lambda k: rec[k])
        return cls(g("rank1"), g("rank2"), g("set1_len"), g("set2_len"), g("population_size"),
                   g("intersection_size"), g("pvalue"), g("permuted"), feature_sets)

    def as_dict(self):
        return {k: getattr(self, k) for k in self.__slots__ if k != "feature_sets"}

    def __eq__(self, other):
        return isinstance(other, OptimizationResultRecord) and all(
            getattr(self, k) == getattr(other, k) for k in self.__slots__)

    def __repr__(self):
        return "OptimizationResultRecord(%s)" % ", ".join(
            "%s=%r" % (k, v) for k, v in self.as_dict().items())


class OptimizationResult:
    """OptimizationResult::Best(record) or ::Debug(records) (results_objects.rs:26-32)."""

    def __init__(self, best=None, records=None):
        self.best = best
        self.records = records

    @classmethod
    def Best(cls, record):
        return cls(best=record)

    @classmethod
    def Debug(cls, records):
        return cls(records=records)

    def is_best(self):
        return self.best is not None

    def is_debug(self):
        return self.records is not None


class _PairCache:
    """Device pairs keyed by the identity of the two lists and the population."""

    def __init__(self):
        self.key = None
        self.pair = None

    def get(self, engine, list1, list2, population):
        key = (id(engine), id(list1), id(list2), int(population), len(list1), len(list2))
        if self.key != key or self.pair is None:
            r1, f1, r2, f2, nf = dense_ids(list1, list2)
            self.pair = engine.pair(r1, f1, r2, f2, nf, int(population))
            self.key = key
        return self.pair


def _cache():
    c = getattr(_state, "pairs", None)
    if c is None:
        c = _state.pairs = _PairCache()
    return c


def _view_indices(view, n):
    if view is None:
        return None
    if isinstance(view, PermutedRankedFeatureList):
        return view.indices
    return np.asarray(view, np.int32)


def optimize(ranked_feature_list1, ranked_feature_list2, permute, population_size, debug=False,
             *, seed=None, perm_id=1, indices=None, precision="screen", engine=None):
    """optimize_main.rs:53-118: the threshold pair with the smallest upper-tail
    hypergeometric p-value; ties go to the larger overlap, then to the smaller
    (rank1, rank2).

    permute: shuffle both lists (process_threshold_pairs.rs:81-82).  The
    permutation is permutation ``perm_id`` of the Philox stream ``seed`` (a
    fresh random seed when None, like the reference's thread_rng), or the
    explicit ``indices=(idx1, idx2)`` (index arrays of PermutedRankedFeatureList
    views).  debug: return every cell's record (OptimizationResult::Debug).
    """
    eng = engine or default_engine()
    dp = _cache().get(eng, ranked_feature_list1, ranked_feature_list2, population_size)
    idx1 = idx2 = None
    if permute:
        if indices is not None:
            idx1 = _view_indices(indices[0], dp.N1)
            idx2 = _view_indices(indices[1], dp.N2)
        else:
            if seed is None:
                seed = int.from_bytes(os.urandom(8), "little")
            idx1, idx2 = dp.export_permutations(seed, perm_id, 1)
            idx1, idx2 = idx1[0], idx2[0]
    if debug:
        recs = dp.grid_dump(idx1, idx2)
        return OptimizationResult.Debug(_debug_records(ranked_feature_list1, ranked_feature_list2,
                                                       recs, idx1, idx2))
    r = dp.optimize(permute=bool(permute), idx1=idx1, idx2=idx2, precision=precision)
    return OptimizationResult.Best(OptimizationResultRecord.from_abi(r))


def _debug_records(l1, l2, recs, idx1, idx2):
    g1 = l1.genes()
    g2 = l2.genes()
    out = []
    for r in recs:
        n1, n2 = int(r["set1_len"]), int(r["set2_len"])
        s1 = [g1[int(idx1[p]) if idx1 is not None else p] for p in range(n1)]
        s2 = [g2[int(idx2[p]) if idx2 is not None else p] for p in range(n2)]
        out.append(OptimizationResultRecord.from_abi(r, FeatureSets.both(s1, s2)))
    return out


def process_threshold_pairs(ranked_feature_list1, ranked_feature_list2, use_permutation,
                            population_size, debug=False, *, seed=None, indices=None,
                            engine=None):
    """process_threshold_pairs.rs:71-131: one record per cell, threshold 1 major."""
    eng = engine or default_engine()
    dp = _cache().get(eng, ranked_feature_list1, ranked_feature_list2, population_size)
    idx1 = idx2 = None
    if use_permutation:
        if indices is not None:
            idx1, idx2 = _view_indices(indices[0], dp.N1), _view_indices(indices[1], dp.N2)
        else:
            if seed is None:
                seed = int.from_bytes(os.urandom(8), "little")
            a, b = dp.export_permutations(seed, 1, 1)
            idx1, idx2 = a[0], b[0]
    recs = dp.grid_dump(idx1, idx2)
    if debug:
        return _debug_records(ranked_feature_list1, ranked_feature_list2, recs, idx1, idx2)
    return [OptimizationResultRecord.from_abi(r) for r in recs]


class PopulationError(ValueError):
    """The reference panics in compute_population_size; this is raised instead."""


def compute_population_size(ranked_feature_list1, ranked_feature_list2, background=None):
    """compute_population_size.rs:66-104."""
    if background is None:
        inter = ranked_feature_list1.genes().intersect(ranked_feature_list2.genes())
        if len(inter) != len(ranked_feature_list1) or len(inter) != len(ranked_feature_list2):
            raise PopulationError(
                "If no background is provided, the feature lists must have identical genes.")
        return len(inter)
    for lst, name in ((ranked_feature_list1, "first"), (ranked_feature_list2, "second")):
        diff = lst.genes().difference(background, False)
        if len(diff):
            raise PopulationError(
                "The following genes in the %s ranked feature list are not in the background: %r"
                % (name, diff.ids()))
    return len(background.genes())


__all__ = ["optimize", "process_threshold_pairs", "compute_population_size", "OptimizationResult",
           "OptimizationResultRecord", "FeatureSets", "PopulationError", "RankedFeatureList",
           "default_engine"]
