"""ctypes wrapper around the C oracle (test infrastructure only).

Each function names the reference file:line whose behaviour the C code restates
(paths relative to the reference project).  Nothing in the product package
imports this module.
"""
import ctypes as C
import functools

import numpy as np

from . import build as _build


class Record(C.Structure):
    _fields_ = [("rank1", C.c_uint32), ("rank2", C.c_uint32),
                ("set1_len", C.c_int64), ("set2_len", C.c_int64),
                ("intersection_size", C.c_int64), ("pvalue", C.c_double),
                ("i", C.c_int32), ("j", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = C.c_void_p


@functools.lru_cache(maxsize=1)
def lib():
    path = _build.build()
    L = C.CDLL(path)
    L.or_lf_table.argtypes = [C.c_int64, _P, _P]
    L.or_sf64.argtypes = [_P, _P, C.c_int64, C.c_int64, C.c_int64, C.c_int64]
    L.or_sf64.restype = C.c_double
    L.or_logpmf.argtypes = [_P, _P, C.c_int64, C.c_int64, C.c_int64, C.c_int64]
    L.or_logpmf.restype = C.c_double
    L.or_thresholds.argtypes = [C.c_uint32, _P, C.c_int64]
    L.or_thresholds.restype = C.c_int64
    L.or_stable_sort.argtypes = [C.c_int64, _P, _P]
    L.or_optimize.argtypes = [_P, _P, C.c_int64, _P, _P, C.c_int64, C.c_int64, C.c_int64,
                              _P, _P, _P, _P, C.c_int, C.POINTER(Record), _P]
    L.or_optimize.restype = C.c_int
    L.or_fdr.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_double]
    L.or_fdr.restype = C.c_double
    L.or_empirical.argtypes = [C.c_double, _P, C.c_int64]
    L.or_empirical.restype = C.c_double
    L.or_philox4x32_10.argtypes = [_P, _P, _P]
    L.or_shuffle.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, _P]
    L.or_ref_run.argtypes = [_P, _P, C.c_int64, _P, _P, C.c_int64, C.c_int64, _P, _P,
                             _P, _P, C.c_int64, C.c_int64, C.c_int, _P]
    L.or_ref_run.restype = C.c_int64
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


@functools.lru_cache(maxsize=8)
def lf_table(nmax):
    """ln(m!) for m = 0..nmax as (hi, lo) double-double arrays."""
    hi = np.zeros(nmax + 1, np.float64)
    lo = np.zeros(nmax + 1, np.float64)
    lib().or_lf_table(nmax, _ptr(hi), _ptr(lo))
    hi.setflags(write=False)
    lo.setflags(write=False)
    return hi, lo


def sf64(N, K, n, k):
    """P(X >= k), X ~ Hypergeometric(N, K, n) (hypergeometric_pvalue.rs:33-50)."""
    hi, lo = lf_table(max(int(N), 1))
    return lib().or_sf64(_ptr(hi), _ptr(lo), int(N), int(K), int(n), int(k))


def logpmf(N, K, n, k):
    hi, lo = lf_table(max(int(N), 1))
    return lib().or_logpmf(_ptr(hi), _ptr(lo), int(N), int(K), int(n), int(k))


def thresholds(max_rank):
    """ranked.rs:359-375 (last threshold not clamped)."""
    n = lib().or_thresholds(int(max_rank), None, 0)
    out = np.zeros(max(n, 1), np.uint32)
    lib().or_thresholds(int(max_rank), _ptr(out), n)
    return out[:n]


def stable_sort(ranks, items):
    """ranked.rs:527-542: stable sort of (rank, item) by rank."""
    r = np.ascontiguousarray(ranks, dtype=np.uint32).copy()
    f = np.ascontiguousarray(items, dtype=np.int32).copy()
    lib().or_stable_sort(len(r), _ptr(r), _ptr(f))
    return r, f


def optimize(ranks1, feat1, ranks2, feat2, nfeat, population, idx1=None, idx2=None,
             mode="hist", all_records=False):
    """optimize_main.rs:53-118 over process_threshold_pairs.rs:71-131.

    ranks sorted ascending; feat* dense feature ids of the sorted positions;
    idx* the permuted views' index arrays (permuted.rs:34) or None.
    Returns (best_record_dict, all_records ndarray or None).
    """
    r1 = np.ascontiguousarray(ranks1, np.uint32)
    r2 = np.ascontiguousarray(ranks2, np.uint32)
    f1 = np.ascontiguousarray(feat1, np.int32)
    f2 = np.ascontiguousarray(feat2, np.int32)
    i1 = None if idx1 is None else np.ascontiguousarray(idx1, np.int32)
    i2 = None if idx2 is None else np.ascontiguousarray(idx2, np.int32)
    hi, lo = lf_table(max(int(population), 1))
    best = Record()
    allr = None
    if all_records:
        n1 = len(thresholds(int(r1[-1])))
        n2 = len(thresholds(int(r2[-1])))
        allr = (Record * (n1 * n2))()
    rc = lib().or_optimize(_ptr(r1), _ptr(f1), len(r1), _ptr(r2), _ptr(f2), len(r2),
                           int(nfeat), int(population), _ptr(i1), _ptr(i2), _ptr(hi), _ptr(lo),
                           0 if mode == "hist" else 1, C.byref(best),
                           None if allr is None else C.cast(allr, C.c_void_p))
    if rc != 0:
        raise ValueError("oracle: no threshold pairs")
    recs = None
    if allr is not None:
        recs = [allr[q].as_dict() for q in range(len(allr))]
    return best.as_dict(), recs


def fdr(l1, l2, overlap, population, sensitivity=0.8):
    """fdr.rs:29-60."""
    return lib().or_fdr(int(l1), int(l2), int(overlap), int(population), float(sensitivity))


def empirical(p_obs, p_perm):
    """empirical_pvalue.rs:169-173 (count of p_perm <= p_obs over P; 1.0 if P == 0)."""
    a = np.ascontiguousarray(p_perm, np.float64)
    return lib().or_empirical(float(p_obs), _ptr(a), len(a))


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().or_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def shuffle(seed, pair_id, perm_id, list_tag, L):
    """The on-device permutation specification (Rao-Sandelius + Fisher-Yates)."""
    out = np.zeros(max(L, 1), np.int32)
    lib().or_shuffle(int(seed), int(pair_id), int(perm_id), int(list_tag), int(L), _ptr(out))
    return out[:L]


def ref_run(genes1, ranks1, genes2, ranks2, population, idx1s=None, idx2s=None, n_tasks=1,
            row_stride=1, nthreads=1):
    """Reference-algorithm CPU run: string hash-set intersection per cell,
    tasks chunked over threads (single_node.rs:95-133).  Returns
    (records list, cells evaluated)."""
    b1 = [g.encode() for g in genes1]
    b2 = [g.encode() for g in genes2]
    a1 = (C.c_char_p * len(b1))(*b1)
    a2 = (C.c_char_p * len(b2))(*b2)
    r1 = np.ascontiguousarray(ranks1, np.uint32)
    r2 = np.ascontiguousarray(ranks2, np.uint32)
    hi, lo = lf_table(max(int(population), 1))
    i1 = None if idx1s is None else np.ascontiguousarray(idx1s, np.int32)
    i2 = None if idx2s is None else np.ascontiguousarray(idx2s, np.int32)
    out = (Record * max(n_tasks, 1))()
    cells = lib().or_ref_run(C.cast(a1, C.c_void_p), _ptr(r1), len(r1), C.cast(a2, C.c_void_p),
                             _ptr(r2), len(r2), int(population), _ptr(hi), _ptr(lo), _ptr(i1),
                             _ptr(i2), int(n_tasks), int(row_stride), int(nthreads),
                             C.cast(out, C.c_void_p))
    return [out[t].as_dict() for t in range(n_tasks)], cells
