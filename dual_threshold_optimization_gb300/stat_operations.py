"""Statistics mirroring the reference's ``src/stat_operations``.

hypergeometric_pvalue  src/stat_operations/hypergeometric_pvalue.rs:33-50
                       (evaluated on the GPU with the engine's FP64 tail)
intersect_genes        src/stat_operations/intersect_genes.rs:38-56 (host set utility)
empirical_pvalue       src/stat_operations/empirical_pvalue.rs:109-187
fdr                    src/stat_operations/fdr.rs:29-60
"""
import warnings

import numpy as np

from ._lib import lib


class HypergeometricError(ValueError):
    """The reference panics with "Failed to create hypergeometric distribution"."""


def hypergeometric_pvalue(population_size, successes_in_population, sample_size, observed_overlap,
                          *, engine=None):
    """P(X >= k), X ~ Hypergeometric(N, K, n); k == 0 gives 1.0.  Scalars or
    arrays (broadcast); evaluated on the device."""
    from .dto import default_engine
    N = np.asarray(population_size, np.int64)
    K = np.asarray(successes_in_population, np.int64)
    n = np.asarray(sample_size, np.int64)
    k = np.asarray(observed_overlap, np.int64)
    if np.any(K > N) or np.any(n > N) or np.any(N < 0) or np.any(K < 0) or np.any(n < 0) \
            or np.any(k < 0):
        raise HypergeometricError("Failed to create hypergeometric distribution")
    out = (engine or default_engine()).hypergeom_sf(N, K, n, k)
    return float(out) if np.ndim(out) == 0 else out


def intersect_genes(genes1, genes2):
    """|genes1 ∩ genes2| by id, counting every genes2 member found in genes1
    (intersect_genes.rs:44-55)."""
    ids1 = {g.id() if hasattr(g, "id") else str(g) for g in genes1}
    return sum(1 for g in genes2 if (g.id() if hasattr(g, "id") else str(g)) in ids1)


def fdr(ranked_list_1_len, ranked_list_2_len, overlap_len, population_size, sensitivity=0.8):
    """Expected FDR lower bound (fdr.rs:29-60)."""
    if sensitivity <= 0.0:
        raise ValueError("Sensitivity must be greater than 0.")
    return float(lib().dto_fdr(int(ranked_list_1_len), int(ranked_list_2_len), int(overlap_len),
                               int(population_size), float(sensitivity)))


def _record(result):
    rec = getattr(result, "best", None)
    if rec is None and isinstance(result, dict):
        return result
    return rec.as_dict() if hasattr(rec, "as_dict") else rec


def empirical_pvalue(results):
    """empirical_pvalue.rs:109-187: the fraction of permuted optima with p <= the
    unpermuted optimum's p (1.0 without permutations), plus the FDR at
    sensitivity 0.8.  ``results``: OptimizationResult objects (Best) or dicts
    with the record fields.

    The keys are the reference's (empirical_pvalue.rs:176-186).  When
    ``results`` is a run's output carrying its summary (run.RunResults), three
    more are added: ``logp_err_bound_fp32`` (bound, in nats, on the error of
    the 32-bit screen's log-pmf; 0 for the plain FP64 path),
    ``logp_err_bound_fp64`` (bound on the relative error of an FP64 p-value,
    hence on its log) and ``perms_per_s`` (permutations per second of the run,
    host wall time)."""
    recs = [_record(r) for r in results]
    unperm = [r for r in recs if r is not None and not r["permuted"]]
    perm = [r for r in recs if r is not None and r["permuted"]]
    summary = getattr(results, "summary", None) or {}
    if len(unperm) != 1:
        warnings.warn("Expected exactly one unpermuted result, but found %d." % len(unperm))
    if not unperm:
        raise ValueError("No unpermuted result found in the provided results.")
    u = unperm[0]
    est_fdr = fdr(u["set1_len"], u["set2_len"], u["intersection_size"], u["population_size"], 0.8)
    if "count_le" in summary and "n_perm" in summary:
        # a sharded run (run_multi_node) counted on every rank
        n = int(summary["n_perm"])
        emp = float(summary["count_le"]) / float(n) if n else 1.0
    elif perm:
        pv = np.array([r["pvalue"] for r in perm], np.float64)
        emp = float(np.count_nonzero(pv <= u["pvalue"])) / float(len(pv))
    else:
        emp = 1.0
    out = {
        "rank1": int(u["rank1"]), "rank2": int(u["rank2"]), "set1_len": int(u["set1_len"]),
        "set2_len": int(u["set2_len"]), "population_size": int(u["population_size"]),
        "unpermuted_intersection_size": int(u["intersection_size"]),
        "unpermuted_pvalue": float(u["pvalue"]), "empirical_pvalue": emp, "fdr": est_fdr,
    }
    if summary:
        for k in ("logp_err_bound_fp32", "logp_err_bound_fp64", "perms_per_s"):
            if k in summary:
                out[k] = summary[k]
    return out
