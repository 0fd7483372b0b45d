"""Data model mirroring the reference's ``src/collections`` (host side).

Feature and FeatureList hold string ids (src/collections/feature.rs:24-77,
src/collections/feature_list.rs:32-421); RankedFeatureList keeps the stable
sort by rank and the threshold grid (src/collections/ranked.rs:176-191,
359-375, 527-542); PermutedRankedFeatureList is a permuted view given by an
index array (src/collections/permuted.rs:30-101).  The threshold grid comes
from libdto.so (dto_generate_thresholds), so host and device use one
definition.  None of this is on the timed path: string ids are mapped to dense
integers before the C ABI.
"""
import ctypes as C

import numpy as np

from ._lib import lib, ptr


class Feature:
    """A feature id (src/collections/feature.rs:24-77)."""

    __slots__ = ("_id",)

    def __init__(self, fid):
        self._id = str(fid)

    @classmethod
    def from_(cls, fid):
        return cls(fid)

    def id(self):
        return self._id

    def __eq__(self, other):
        return isinstance(other, Feature) and other._id == self._id

    def __hash__(self):
        return hash(self._id)

    def __repr__(self):
        return "Feature(%r)" % self._id


class FeatureList:
    """An ordered list of features (src/collections/feature_list.rs)."""

    def __init__(self, genes=None):
        self._genes = [g if isinstance(g, Feature) else Feature(g) for g in (genes or [])]

    @classmethod
    def from_(cls, genes):
        return cls(genes)

    def genes(self):
        return list(self._genes)

    def ids(self):
        return [g.id() for g in self._genes]

    def __len__(self):
        return len(self._genes)

    def __iter__(self):
        return iter(self._genes)

    def __getitem__(self, i):
        return self._genes[i]

    def is_empty(self):
        return not self._genes

    def intersect(self, other):
        """Features present in both lists, in this list's order (feature_list.rs:278-286)."""
        s = set(other.ids())
        return FeatureList([g for g in self._genes if g.id() in s])

    def difference(self, other, _symmetric=False):
        """Features of this list absent from other (feature_list.rs:325-344)."""
        s = set(other.ids())
        return FeatureList([g for g in self._genes if g.id() not in s])

    def check_unique(self):
        """Raise on duplicate ids (feature_list.rs:128-145; the reference never calls it on the
        CLI path, the device boundary rejects duplicates)."""
        seen = set()
        for g in self._genes:
            if g.id() in seen:
                raise ValueError("Duplicate feature found: %s" % g.id())
            seen.add(g.id())


def generate_thresholds(max_rank):
    """T1 = 1, T(k+1) = floor(T(k)*1.01 + 1) while T <= max_rank, the last one not
    clamped to max_rank (src/collections/ranked.rs:359-375)."""
    n = lib().dto_generate_thresholds(int(max_rank), None, 0)
    out = np.zeros(max(n, 1), np.uint32)
    lib().dto_generate_thresholds(int(max_rank), ptr(out), n)
    return out[:n]


class RankedFeatureList:
    """Features stably sorted by rank, with the threshold grid
    (src/collections/ranked.rs:125-191)."""

    def __init__(self):
        self._genes = FeatureList()
        self._ranks = np.zeros(0, np.uint32)
        self._thresholds = np.zeros(0, np.uint32)

    @classmethod
    def from_(cls, genes, ranks):
        genes = genes if isinstance(genes, FeatureList) else FeatureList(genes)
        ranks = np.asarray(ranks, dtype=np.int64)
        if len(genes) != len(ranks):
            raise ValueError("Genes and ranks must have the same length. Got %d genes and %d ranks."
                             % (len(genes), len(ranks)))
        if len(ranks) and (ranks.min() < 0 or ranks.max() > 0xFFFFFFFF):
            raise ValueError("ranks must fit in u32")
        self = cls()
        order = np.argsort(ranks, kind="stable")  # ranked.rs:534 sort_by_key is stable
        self._ranks = ranks[order].astype(np.uint32)
        g = genes.genes()
        self._genes = FeatureList([g[i] for i in order])
        self._thresholds = generate_thresholds(int(self._ranks[-1]) if len(self._ranks) else 0)
        return self

    def genes(self):
        return self._genes

    def ranks(self):
        return self._ranks

    def thresholds(self):
        return self._thresholds

    def __len__(self):
        return len(self._genes)

    def is_empty(self):
        return len(self._genes) == 0

    def get_feature_set_by_threshold(self, threshold):
        """Features with rank <= threshold (ranked.rs:561-568)."""
        n = int(np.searchsorted(self._ranks, threshold, side="right"))
        return [self._genes[i] for i in range(n)]


class PermutedRankedFeatureList:
    """A permuted view: position p shows feature genes[indices[p]] with rank
    ranks[p] (src/collections/permuted.rs:30-101).  The reference shuffles with
    an unseeded thread_rng; here the index array is explicit (or drawn from a
    seeded numpy generator) so a view is reproducible."""

    def __init__(self, original, indices=None, rng=None):
        self.original = original
        if indices is None:
            rng = rng if rng is not None else np.random.default_rng()
            indices = rng.permutation(len(original))
        self.indices = np.asarray(indices, np.int32)
        if sorted(self.indices.tolist()) != list(range(len(original))):
            raise ValueError("indices must be a permutation of 0..len")

    def thresholds(self):
        return self.original.thresholds()

    def ranks(self):
        return self.original.ranks()

    def get_feature_set_by_threshold(self, threshold):
        n = int(np.searchsorted(self.original.ranks(), threshold, side="right"))
        g = self.original.genes()
        return [g[int(self.indices[p])] for p in range(n)]


def dense_ids(list1, list2, background=None):
    """Map the string ids of two ranked lists (and an optional background) to
    dense integers: returns (ranks1, feat1, ranks2, feat2, n_features) with the
    lists in their sorted order."""
    ids = {}
    f1 = np.array([ids.setdefault(g.id(), len(ids)) for g in list1.genes()], np.int32)
    f2 = np.array([ids.setdefault(g.id(), len(ids)) for g in list2.genes()], np.int32)
    if background is not None:
        for g in background.genes():
            ids.setdefault(g.id(), len(ids))
    return list1.ranks(), f1, list2.ranks(), f2, len(ids)
