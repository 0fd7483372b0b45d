"""ctypes binding of libdto.so (the C ABI in include/dto.h).

The library is loaded from this package directory.  There is no fallback: if
libdto.so is missing or cannot be loaded, every entry point raises.
"""
import ctypes as C
import functools
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libdto.so")

DTO_OK = 0
DTO_ERR_INVALID = 1
DTO_ERR_OOM = 2
DTO_ERR_TIMEOUT = 3
DTO_ERR_CUDA = 4
DTO_ERR_NOT_FOUND = 5
DTO_ERR_CANCELLED = 6

PRECISION_FP64 = 0
PRECISION_SCREEN = 1

# Every symbol include/dto.h declares.
EXPORTS = (
    "dto_version", "dto_status_string", "dto_ctx_create", "dto_ctx_destroy", "dto_last_error",
    "dto_ctx_stream", "dto_generate_thresholds", "dto_rank_order", "dto_pair_create", "dto_pair_destroy",
    "dto_pair_info", "dto_pair_thresholds", "dto_pair_order", "dto_pair_upload_bytes", "dto_pair_set_stream", "dto_pair_set_ladder",
    "dto_pair_set_level0_quantile", "dto_pair_tune", "dto_run", "dto_run_range", "dto_run_range_noalloc",
    "dto_optimize",
    "dto_grid_dump", "dto_hypergeom_sf", "dto_export_permutations", "dto_fdr",
    "dto_serve_create", "dto_serve_destroy", "dto_serve_submit", "dto_serve_poll", "dto_serve_wait",
    "dto_serve_wait_for", "dto_serve_cancel",
    "dto_serve_last_error", "dto_serve_stats", "dto_run_device_bytes", "dto_batch_run",
)


class DtoResult(C.Structure):
    _fields_ = [("rank1", C.c_uint32), ("rank2", C.c_uint32), ("set1_len", C.c_int64),
                ("set2_len", C.c_int64), ("population_size", C.c_int64),
                ("intersection_size", C.c_int64), ("pvalue", C.c_double),
                ("permuted", C.c_int32), ("i", C.c_int32), ("j", C.c_int32),
                ("status", C.c_int32), ("route", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


RESULT_DTYPE = np.dtype([("rank1", np.uint32), ("rank2", np.uint32), ("set1_len", np.int64),
                         ("set2_len", np.int64), ("population_size", np.int64),
                         ("intersection_size", np.int64), ("pvalue", np.float64),
                         ("permuted", np.int32), ("i", np.int32), ("j", np.int32),
                         ("status", np.int32), ("route", np.int32), ("reserved", np.int32)],
                        align=True)
# The fields that describe a task's optimum: every search path gives the same
# values here; "route" names the path that settled the task.
OPTIMUM_FIELDS = ("rank1", "rank2", "set1_len", "set2_len", "population_size", "intersection_size",
                  "pvalue", "permuted", "i", "j", "status")
ROUTE_NAMES = ("none", "screen", "level0", "level1", "level2", "fallback", "fp64", "unused")
assert RESULT_DTYPE.itemsize == C.sizeof(DtoResult)


class DtoSummary(C.Structure):
    _fields_ = [("n_perm", C.c_int64), ("count_le", C.c_int64), ("empirical_pvalue", C.c_double),
                ("fdr", C.c_double), ("logp_err_bound_screen", C.c_double),
                ("logp_err_bound_fp64", C.c_double), ("n_fallback", C.c_int64),
                ("n_refined", C.c_int64), ("n_stage2", C.c_int64),
                ("device_ms", C.c_double), ("grid_ms", C.c_double), ("perm_ms", C.c_double),
                ("n_launches", C.c_int64), ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
                ("sweep0_ms", C.c_double), ("sweep0_launches", C.c_int64), ("sweep0_tasks", C.c_int64),
                ("n_route", C.c_int64 * 8), ("tail_ms", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "n_route"}
        d["n_route"] = {ROUTE_NAMES[q]: int(self.n_route[q]) for q in range(7)}
        return d


class DtoError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d)" % (message, status))
        self.status = status


_P = C.c_void_p


@functools.lru_cache(maxsize=1)
def lib():
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libdto.so is not built (expected at %s); run "
                           "dual_threshold_optimization_gb300.build.build()" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    L.dto_version.restype = C.c_int
    L.dto_status_string.argtypes = [C.c_int]
    L.dto_status_string.restype = C.c_char_p
    L.dto_ctx_create.argtypes = [C.c_int, C.POINTER(_P)]
    L.dto_ctx_destroy.argtypes = [_P]
    L.dto_last_error.argtypes = [_P]
    L.dto_last_error.restype = C.c_char_p
    L.dto_ctx_stream.argtypes = [_P]
    L.dto_ctx_stream.restype = _P
    L.dto_generate_thresholds.argtypes = [C.c_uint32, _P, C.c_int64]
    L.dto_generate_thresholds.restype = C.c_int64
    L.dto_rank_order.argtypes = [_P, C.c_int64, _P]
    L.dto_rank_order.restype = C.c_int
    L.dto_pair_create.argtypes = [_P, _P, _P, C.c_int64, _P, _P, C.c_int64, C.c_int64, C.c_int64,
                                  C.POINTER(_P)]
    L.dto_pair_destroy.argtypes = [_P]
    L.dto_pair_info.argtypes = [_P, _P, _P, _P]
    L.dto_pair_thresholds.argtypes = [_P, _P, _P]
    L.dto_pair_order.argtypes = [_P, _P, _P]
    L.dto_pair_upload_bytes.argtypes = [_P]
    L.dto_pair_set_stream.argtypes = [_P, C.c_uint32]
    L.dto_pair_set_stream.restype = C.c_int
    L.dto_pair_set_ladder.argtypes = [_P, _P, C.c_int64]
    L.dto_pair_set_ladder.restype = C.c_int
    L.dto_pair_set_level0_quantile.argtypes = [_P, C.c_double]
    L.dto_pair_set_level0_quantile.restype = C.c_int
    L.dto_pair_tune.argtypes = [_P, _P, C.c_int64, C.c_uint64, C.POINTER(C.c_double)]
    L.dto_pair_tune.restype = C.c_int
    L.dto_pair_upload_bytes.restype = C.c_int64
    L.dto_run.argtypes = [_P, _P, C.c_int64, C.c_uint64, _P, C.c_int, C.POINTER(DtoResult), _P,
                          _P, C.POINTER(DtoSummary)]
    L.dto_run_range.argtypes = [_P, _P, C.c_uint32, C.c_int64, C.c_uint64, _P, C.c_int,
                                C.POINTER(DtoResult), _P, _P, C.POINTER(DtoSummary)]
    L.dto_run_range_noalloc.argtypes = [_P, _P, C.c_uint32, C.c_int64, C.c_uint64, _P]
    L.dto_run_range_noalloc.restype = C.c_int
    L.dto_optimize.argtypes = [_P, _P, C.c_int, C.c_uint64, C.c_uint32, _P, _P, C.c_int,
                               C.POINTER(DtoResult)]
    L.dto_grid_dump.argtypes = [_P, _P, _P, _P, _P]
    L.dto_hypergeom_sf.argtypes = [_P, _P, _P, _P, _P, _P, C.c_int64]
    L.dto_export_permutations.argtypes = [_P, _P, C.c_uint64, C.c_uint32, C.c_int64, _P, _P]
    L.dto_fdr.argtypes = [C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_double]
    L.dto_fdr.restype = C.c_double
    L.dto_serve_create.argtypes = [_P, C.c_int, C.c_int64, C.POINTER(_P)]
    L.dto_serve_destroy.argtypes = [_P]
    L.dto_serve_submit.argtypes = [_P, _P, C.c_uint32, C.c_int64, C.c_uint64, C.c_int,
                                   C.POINTER(DtoResult), _P, C.POINTER(DtoSummary), C.POINTER(C.c_int64)]
    L.dto_serve_poll.argtypes = [_P, C.c_int64, C.POINTER(C.c_int)]
    L.dto_serve_wait.argtypes = [_P, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.dto_serve_wait_for.argtypes = [_P, C.c_int64, C.c_double, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
    L.dto_serve_wait_for.restype = C.c_int
    L.dto_serve_cancel.argtypes = [_P, C.c_int64]
    L.dto_serve_cancel.restype = C.c_int
    L.dto_serve_last_error.argtypes = [_P]
    L.dto_serve_last_error.restype = C.c_char_p
    L.dto_serve_stats.argtypes = [_P, _P, _P, _P, _P]
    L.dto_run_device_bytes.argtypes = [_P, C.c_int64]
    L.dto_run_device_bytes.restype = C.c_int64
    L.dto_batch_run.argtypes = [_P, C.c_int, _P, _P, _P, C.c_int, C.c_int, _P, _P, _P]
    for name in EXPORTS:
        getattr(L, name)
    for name in EXPORTS:
        fn = getattr(L, name)
        if fn.restype is C.c_int or name in ("dto_ctx_create", "dto_ctx_destroy", "dto_pair_create",
                                             "dto_pair_destroy", "dto_pair_info",
                                             "dto_pair_thresholds", "dto_pair_order", "dto_run",
                                             "dto_run_range", "dto_optimize", "dto_grid_dump", "dto_hypergeom_sf",
                                             "dto_export_permutations", "dto_serve_create",
                                             "dto_serve_destroy", "dto_serve_submit", "dto_serve_poll",
                                             "dto_serve_wait", "dto_serve_stats", "dto_batch_run"):
            fn.restype = C.c_int
    return L


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def check(status, ctx=None):
    if status != DTO_OK:
        msg = lib().dto_last_error(ctx).decode() if ctx else lib().dto_status_string(status).decode()
        raise DtoError(status, msg or lib().dto_status_string(status).decode())
