"""dto_run_range_noalloc: the permutation null for callers that cannot allocate
device memory when they run it (for example while recording a CUDA graph, or
under a memory manager that owns every device allocation).  The entry point
keeps its intermediates in a fixed device array inside libdto.so; the caller
supplies only the output array.

Checked here through the C ABI: two calls in a row give the same per-permutation
minimum p-values as dto_run_range (bit for bit, the tolerance of the other
parity tests), and a request larger than the fixed array is refused.  This file
is collected last so that a failure here comes after every other test ran.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_run_range_twice():
    torch = pytest.importorskip("torch")
    from dual_threshold_optimization_gb300 import Engine, synth
    from dual_threshold_optimization_gb300._lib import DTO_ERR_INVALID, lib

    eng = Engine(0)
    p = synth.copula_pair(5000, 0.25, seed=61, frac_tied2=0.05)
    dp = eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    seed = 0xABCDEF
    for first, count in ((1, 600), (601, 450)):
        want = dp.run(count, seed=seed, first=first).minp
        out = torch.full((count,), -1.0, dtype=torch.float64, device="cuda")
        rc = lib().dto_run_range_noalloc(eng.handle, dp.handle, first, count, seed,
                                         C.c_void_p(out.data_ptr()))
        assert rc == 0, lib().dto_last_error(eng.handle)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got, want), (first, count)

    # a request beyond the fixed array is refused with a clear message
    big = torch.empty(1, dtype=torch.float64, device="cuda")
    rc = lib().dto_run_range_noalloc(eng.handle, dp.handle, 1, 1_000_000, seed,
                                     C.c_void_p(big.data_ptr()))
    assert rc == DTO_ERR_INVALID
    assert b"exceeds" in lib().dto_last_error(eng.handle)

    # lists with different feature sets take the two-shuffle path
    q = synth.small_pair(300, 0.3, seed=62, subset1=260, subset2=280)
    dq = eng.pair(q.ranks1, q.feat1, q.ranks2, q.feat2, q.n_features, q.population)
    want = dq.run(64, seed=seed, first=5).minp
    out = torch.empty(64, dtype=torch.float64, device="cuda")
    assert lib().dto_run_range_noalloc(eng.handle, dq.handle, 5, 64, seed,
                                       C.c_void_p(out.data_ptr())) == 0
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), want)
    dq.close()
    dp.close()
    eng.close()
