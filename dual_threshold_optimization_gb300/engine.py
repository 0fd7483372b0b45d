"""Python handle over the C ABI: a device context and device-resident list pairs.

This is the layer the reference-shaped API (``collections``, ``dto``, ``run``,
``stat_operations``) is built on.  Every compute call goes to libdto.so.
"""
import ctypes as C

import numpy as np

from ._lib import (DtoError, DtoResult, DtoSummary, PRECISION_FP64, PRECISION_SCREEN, RESULT_DTYPE,
                   check, lib, ptr)

_PREC = {"fp64": PRECISION_FP64, "screen": PRECISION_SCREEN, "fp32screen": PRECISION_SCREEN}


def precision_code(precision):
    if isinstance(precision, int):
        return precision
    try:
        return _PREC[precision]
    except KeyError:
        raise ValueError("precision must be one of %s" % sorted(_PREC)) from None


class Engine:
    """One CUDA device: stream, log-factorial tables and scratch (dto_ctx)."""

    def __init__(self, device=0):
        self._ctx = C.c_void_p()
        check(lib().dto_ctx_create(int(device), C.byref(self._ctx)))
        self.device = int(device)

    @property
    def handle(self):
        if not self._ctx:
            raise RuntimeError("engine is closed")
        return self._ctx

    @property
    def stream(self):
        """The context's cudaStream_t as an integer."""
        return lib().dto_ctx_stream(self.handle) or 0

    def close(self):
        if getattr(self, "_ctx", None):
            lib().dto_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def pair(self, ranks1, feat1, ranks2, feat2, n_features, population):
        return DevicePair(self, ranks1, feat1, ranks2, feat2, n_features, population)

    def server(self, lanes=4, mem_budget=0):
        """A request executor on this device (dto_serve_create)."""
        return Server(self, lanes, mem_budget)

    def batch_run(self, pairs, n_perm, seeds, precision="screen", lanes=4, want_minp=True):
        """The permutation null of many pairs at once (dto_batch_run): pair q
        takes n_perm[q] permutations from id 1 of seeds[q].  Returns one
        RunResult per pair."""
        npairs = len(pairs)
        n_perm = np.ascontiguousarray(np.broadcast_to(np.asarray(n_perm, np.int64), (npairs,)))
        seeds = np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, np.uint64), (npairs,)))
        handles = (C.c_void_p * npairs)(*[p.handle.value for p in pairs])
        unp = (DtoResult * npairs)()
        summ = (DtoSummary * npairs)()
        minps = [np.empty(int(n), np.float64) for n in n_perm] if want_minp else None
        mp = (C.c_void_p * npairs)(*[m.ctypes.data for m in minps]) if want_minp else None
        check(lib().dto_batch_run(self.handle, npairs, handles, ptr(n_perm), ptr(seeds),
                                  precision_code(precision), int(lanes), unp, mp, summ), self.handle)
        return [RunResult(unp[q].as_dict(), minps[q] if want_minp else None, None, summ[q].as_dict())
                for q in range(npairs)]

    def hypergeom_sf(self, N, K, n, k):
        """P(X >= k), X ~ Hypergeometric(N, K, n), elementwise, on the device."""
        arrs = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, np.int64), np.broadcast(N, K, n, k).shape))
                for v in (N, K, n, k)]
        flat = [a.reshape(-1).copy() for a in arrs]
        out = np.empty(flat[0].shape[0], np.float64)
        check(lib().dto_hypergeom_sf(self.handle, ptr(flat[0]), ptr(flat[1]), ptr(flat[2]),
                                     ptr(flat[3]), ptr(out), out.shape[0]), self.handle)
        return out.reshape(arrs[0].shape)


class Server:
    """A request executor (dto_server): ``lanes`` permutation nulls run at
    once, admitted in arrival order as lanes and device memory free up."""

    def __init__(self, engine, lanes=4, mem_budget=0):
        self.engine = engine
        self._srv = C.c_void_p()
        check(lib().dto_serve_create(engine.handle, int(lanes), int(mem_budget), C.byref(self._srv)),
              engine.handle)
        self.lanes = int(lanes)

    @property
    def handle(self):
        if not self._srv:
            raise RuntimeError("server is closed")
        return self._srv

    def submit(self, pair, n_perm, seed=0, first=1, precision="screen", want_minp=True):
        job = Job(self, pair, int(n_perm), want_minp)
        st = lib().dto_serve_submit(self.handle, pair.handle, int(first), int(n_perm),
                                    int(seed) & (2**64 - 1), precision_code(precision),
                                    C.byref(job._unp), ptr(job._minp), C.byref(job._summ),
                                    C.byref(job._id))
        if st != 0:
            raise DtoError(st, lib().dto_serve_last_error(self.handle).decode())
        return job

    def stats(self):
        q, r, c, b = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().dto_serve_stats(self.handle, C.byref(q), C.byref(r), C.byref(c), C.byref(b)))
        return {"queued": q.value, "running": r.value, "completed": c.value, "reserved_bytes": b.value}

    def close(self):
        if getattr(self, "_srv", None):
            lib().dto_serve_destroy(self._srv)
            self._srv = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Job:
    """One queued request; its output buffers live here until it is waited for."""

    def __init__(self, server, pair, n_perm, want_minp):
        self.server = server
        self.pair = pair
        self._id = C.c_int64(0)
        self._unp = DtoResult()
        self._summ = DtoSummary()
        self._minp = np.empty(n_perm, np.float64) if want_minp else None
        self._result = None
        self.queue_ms = self.run_ms = None

    def done(self):
        if self._result is not None:
            return True
        d = C.c_int(0)
        check(lib().dto_serve_poll(self.server.handle, self._id.value, C.byref(d)))
        return bool(d.value)

    def wait(self, timeout_ms=None):
        """The request's RunResult.  With timeout_ms, a request not finished
        in time raises DtoError(DTO_ERR_TIMEOUT) and can be waited for again
        or cancelled; a cancelled request raises DtoError(DTO_ERR_CANCELLED)."""
        if self._result is None:
            qm, rm = C.c_double(), C.c_double()
            if timeout_ms is None:
                st = lib().dto_serve_wait(self.server.handle, self._id.value, C.byref(qm), C.byref(rm))
            else:
                st = lib().dto_serve_wait_for(self.server.handle, self._id.value, float(timeout_ms),
                                              C.byref(qm), C.byref(rm))
            if st != 0:
                raise DtoError(st, lib().dto_serve_last_error(self.server.handle).decode())
            self.queue_ms, self.run_ms = qm.value, rm.value
            self._result = RunResult(self._unp.as_dict(), self._minp, None, self._summ.as_dict())
        return self._result

    def cancel(self):
        """dto_serve_cancel: a queued request leaves the queue; a running one
        stops at its next batch boundary."""
        check(lib().dto_serve_cancel(self.server.handle, self._id.value))


class RunResult:
    """Result of DevicePair.run: the unpermuted optimum, the per-permutation
    minimum p-values (and optionally optima) and the summary."""

    def __init__(self, unpermuted, minp, records, summary):
        self.unpermuted = unpermuted
        self.minp = minp
        self.records = records
        self.summary = summary


class DevicePair:
    """Two ranked lists resident on the device (dto_pair)."""

    def __init__(self, engine, ranks1, feat1, ranks2, feat2, n_features, population):
        self.engine = engine
        r1 = np.ascontiguousarray(ranks1, np.uint32)
        r2 = np.ascontiguousarray(ranks2, np.uint32)
        f1 = np.ascontiguousarray(feat1, np.int32)
        f2 = np.ascontiguousarray(feat2, np.int32)
        if r1.shape != f1.shape or r2.shape != f2.shape:
            raise ValueError("ranks and features must have the same length")
        self._pair = C.c_void_p()
        check(lib().dto_pair_create(engine.handle, ptr(r1), ptr(f1), r1.shape[0], ptr(r2), ptr(f2),
                                    r2.shape[0], int(n_features), int(population),
                                    C.byref(self._pair)), engine.handle)
        self.N1, self.N2 = r1.shape[0], r2.shape[0]
        self.population = int(population)
        n1, n2, nc = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().dto_pair_info(self._pair, C.byref(n1), C.byref(n2), C.byref(nc)))
        self.n1, self.n2, self.n_common = n1.value, n2.value, nc.value

    def close(self):
        if getattr(self, "_pair", None):
            lib().dto_pair_destroy(self._pair)
            self._pair = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        if not self._pair:
            raise RuntimeError("pair is closed")
        return self._pair

    def set_stream(self, stream_id):
        """Philox stream id of this pair's permutations (default 0)."""
        check(lib().dto_pair_set_stream(self.handle, int(stream_id)))

    def set_ladder(self, minp):
        """Seed the table ladder of this pair's next long run from a sample of
        minimum p-values (an earlier run's ``minp``); an empty sample forgets
        it.  The ladder decides only which path settles each permutation."""
        a = np.ascontiguousarray(np.asarray(minp, np.float64).reshape(-1))
        check(lib().dto_pair_set_ladder(self.handle, ptr(a) if a.size else None, a.size),
              self.engine.handle)

    def set_level0_quantile(self, q0):
        """The quantile of the minimum p-values that sets this pair's level-0
        table (default 0.85, in [0.5, 0.99]); performance only."""
        check(lib().dto_pair_set_level0_quantile(self.handle, float(q0)), self.engine.handle)

    def tune(self, n_perm, seed=1):
        """Picks this pair's level-0 quantile by timed trial runs of n_perm
        permutations (> 1,024) among 0.80, 0.85 and 0.90, keeps the fastest
        and records it for the pair's shape (dto_pair_tune).  Returns it."""
        best = C.c_double(0.0)
        check(lib().dto_pair_tune(self.engine.handle, self.handle, int(n_perm), int(seed), C.byref(best)),
              self.engine.handle)
        return best.value

    @property
    def upload_bytes(self):
        """Host-to-device bytes dto_pair_create copied for this pair."""
        return int(lib().dto_pair_upload_bytes(self.handle))

    def thresholds(self):
        t1 = np.zeros(self.n1, np.uint32)
        t2 = np.zeros(self.n2, np.uint32)
        check(lib().dto_pair_thresholds(self.handle, ptr(t1), ptr(t2)))
        return t1, t2

    def order(self):
        o1 = np.zeros(self.N1, np.int32)
        o2 = np.zeros(self.N2, np.int32)
        check(lib().dto_pair_order(self.handle, ptr(o1), ptr(o2)))
        return o1, o2

    def run(self, n_perm, seed=0, perm_idx=None, precision="screen", want_minp=True,
            want_records=False, first=1, unpermuted=True):
        """dto_run_range: permutations first .. first + n_perm - 1 of ``seed``
        (or the rows of ``perm_idx``), plus the unpermuted task unless
        ``unpermuted`` is False (then ``RunResult.unpermuted`` is None and the
        summary's count_le is -1)."""
        ctx = self.engine.handle
        n_perm = int(n_perm)
        idx = None
        if perm_idx is not None:
            idx = np.ascontiguousarray(perm_idx, np.int32)
            if idx.shape != (n_perm, self.N1 + self.N2):
                raise ValueError("perm_idx must have shape (n_perm, N1 + N2)")
        unp = DtoResult()
        minp = np.empty(n_perm, np.float64) if want_minp else None
        recs = np.zeros(n_perm, RESULT_DTYPE) if want_records else None
        summ = DtoSummary()
        check(lib().dto_run_range(ctx, self.handle, int(first), n_perm, int(seed) & (2**64 - 1),
                                  ptr(idx), precision_code(precision),
                                  C.byref(unp) if unpermuted else None, ptr(minp),
                                  ptr(recs), C.byref(summ)), ctx)
        return RunResult(unp.as_dict() if unpermuted else None, minp, recs, summ.as_dict())

    def optimize(self, permute=False, seed=0, perm_id=1, idx1=None, idx2=None, precision="screen"):
        ctx = self.engine.handle
        i1 = None if idx1 is None else np.ascontiguousarray(idx1, np.int32)
        i2 = None if idx2 is None else np.ascontiguousarray(idx2, np.int32)
        out = DtoResult()
        check(lib().dto_optimize(ctx, self.handle, int(bool(permute)), int(seed) & (2**64 - 1),
                                 int(perm_id), ptr(i1), ptr(i2), precision_code(precision),
                                 C.byref(out)), ctx)
        return out.as_dict()

    def grid_dump(self, idx1=None, idx2=None):
        ctx = self.engine.handle
        i1 = None if idx1 is None else np.ascontiguousarray(idx1, np.int32)
        i2 = None if idx2 is None else np.ascontiguousarray(idx2, np.int32)
        recs = np.zeros(self.n1 * self.n2, RESULT_DTYPE)
        check(lib().dto_grid_dump(ctx, self.handle, ptr(i1), ptr(i2), ptr(recs)), ctx)
        return recs

    def export_permutations(self, seed, first, count):
        ctx = self.engine.handle
        i1 = np.zeros((count, self.N1), np.int32)
        i2 = np.zeros((count, self.N2), np.int32)
        check(lib().dto_export_permutations(ctx, self.handle, int(seed) & (2**64 - 1), int(first),
                                            int(count), ptr(i1), ptr(i2)), ctx)
        return i1, i2
