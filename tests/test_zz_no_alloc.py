"""dto_run_range_noalloc: the permutation null for callers that cannot allocate
device memory when they run it -- a process whose device memory is owned by
another allocator (a framework's fixed-budget pool, an application that hands
out device memory itself), or a runtime that forbids allocation on its request
path.  The entry point keeps its intermediates in a fixed device array inside
libdto.so; the caller supplies only the output array.

Checked here through the C ABI, on a context that never ran dto_run: two calls
in a row give the same per-permutation minimum p-values as dto_run_range on
another context (bit for bit, the tolerance of the other parity tests), the
device's free memory does not drop across the calls, and a request larger than
the fixed array is refused.  This file is collected last so that a failure here
comes after every other test ran.
"""
import ctypes as C
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_run_range_twice():
    torch = pytest.importorskip("torch")
    from dual_threshold_optimization_gb300 import Engine, synth
    from dual_threshold_optimization_gb300._lib import DTO_ERR_INVALID, lib

    seed = 0xABCDEF
    calls = ((1, 600), (601, 450))
    p = synth.copula_pair(5000, 0.25, seed=61, frac_tied2=0.05)
    # the expected values, from dto_run_range on a context of their own
    ref = Engine(0)
    dref = ref.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    want = {c: dref.run(c[1], seed=seed, first=c[0]).minp for c in calls}

    eng = Engine(0)  # never runs dto_run: only the no-allocation entry point
    dp = eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    outs = {c: torch.full((c[1],), -1.0, dtype=torch.float64, device="cuda") for c in calls}
    # one call first: it resolves the device array's address and loads the
    # kernels, whose code takes device memory once
    warm = torch.empty(calls[0][1], dtype=torch.float64, device="cuda")
    assert lib().dto_run_range_noalloc(eng.handle, dp.handle, 1, calls[0][1], seed,
                                       C.c_void_p(warm.data_ptr())) == 0
    torch.cuda.synchronize()
    gc.collect()
    free0, _ = torch.cuda.mem_get_info()
    for first, count in calls:
        rc = lib().dto_run_range_noalloc(eng.handle, dp.handle, first, count, seed,
                                         C.c_void_p(outs[(first, count)].data_ptr()))
        assert rc == 0, lib().dto_last_error(eng.handle)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, "the calls took %d bytes of device memory" % (free0 - free1)
    for c in calls:
        assert np.array_equal(outs[c].cpu().numpy(), want[c]), c
    assert np.array_equal(warm.cpu().numpy(), want[calls[0]])

    # a request beyond the fixed array is refused with a clear message
    big = torch.empty(1, dtype=torch.float64, device="cuda")
    rc = lib().dto_run_range_noalloc(eng.handle, dp.handle, 1, 1_000_000, seed,
                                     C.c_void_p(big.data_ptr()))
    assert rc == DTO_ERR_INVALID
    assert b"exceeds" in lib().dto_last_error(eng.handle)
    # a pair of another context is refused as such
    rc = lib().dto_run_range_noalloc(eng.handle, dref.handle, 1, 1, seed, C.c_void_p(big.data_ptr()))
    assert rc == DTO_ERR_INVALID
    assert b"another context" in lib().dto_last_error(eng.handle)

    # lists with different feature sets take the two-shuffle path
    q = synth.small_pair(300, 0.3, seed=62, subset1=260, subset2=280)
    dqr = ref.pair(q.ranks1, q.feat1, q.ranks2, q.feat2, q.n_features, q.population)
    want_q = dqr.run(64, seed=seed, first=5).minp
    dq = eng.pair(q.ranks1, q.feat1, q.ranks2, q.feat2, q.n_features, q.population)
    for _ in range(2):
        out = torch.empty(64, dtype=torch.float64, device="cuda")
        assert lib().dto_run_range_noalloc(eng.handle, dq.handle, 5, 64, seed,
                                           C.c_void_p(out.data_ptr())) == 0
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), want_q)
    for h in (dq, dqr, dp, dref):
        h.close()
    eng.close()
    ref.close()
