"""Many pairs and many requests on one GPU: dto_serve_* and dto_batch_run.

A request's results must not depend on what runs beside it: every request is
run alone through dto_run_range first, then all of them through a server
whose lanes overlap them on the device (some submitted while others run), and
the per-permutation minimum p-values and the unpermuted optimum must agree bit
for bit.
"""
import time

import numpy as np
import pytest

from helpers import optimum

from dual_threshold_optimization_gb300 import synth
from dual_threshold_optimization_gb300._lib import DtoError

pytestmark = pytest.mark.gpu


def _mix(engine):
    specs = [  # (pair, n_perm, seed): table pipeline and exhaustive-only runs, same- and mixed-set lists
        (synth.copula_pair(20000, 0.2, seed=71), 30000, 5),
        (synth.copula_pair(6000, 0.3, seed=72, frac_tied2=0.1), 5000, 6),
        (synth.small_pair(4000, 0.2, seed=73, subset1=3600, subset2=3800), 3000, 7),
        (synth.copula_pair(2500, 0.0, seed=74), 800, 8),
        (synth.background_pair(12000, 9000, 0.1, seed=75), 12000, 9),
        (synth.copula_pair(20000, 0.2, seed=71), 4000, 10),  # same lists again, other seed
    ]
    out = []
    for p, n, s in specs:
        dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
        out.append((dp, n, s))
    return out


def test_requests_same_alone_and_in_the_mix(engine):
    mix = _mix(engine)
    alone = [dp.run(n, seed=s) for dp, n, s in mix]
    with engine.server(lanes=3) as srv:
        jobs = [srv.submit(dp, n, seed=s) for dp, n, s in mix[:3]]
        time.sleep(0.002)  # the rest arrive while the first ones run
        jobs += [srv.submit(dp, n, seed=s) for dp, n, s in mix[3:]]
        res = [j.wait() for j in jobs]
        st = srv.stats()
    assert st["queued"] == 0 and st["running"] == 0 and st["reserved_bytes"] == 0
    for a, r, (dp, n, s) in zip(alone, res, mix):
        assert optimum(r.unpermuted) == optimum(a.unpermuted), (n, s)
        assert np.array_equal(r.minp, a.minp), (n, s)
        assert r.summary["count_le"] == a.summary["count_le"]
        assert r.summary["empirical_pvalue"] == a.summary["empirical_pvalue"]
    for dp, _, _ in mix:
        dp.close()


def test_batch_run_equals_single_runs(engine):
    pairs = [synth.copula_pair(n, r, seed=80 + q) for q, (n, r) in
             enumerate([(2000, 0.1), (9000, 0.3), (15000, 0.0), (3000, 0.4)])]
    dps = [engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population) for p in pairs]
    n_perm = [2500, 4000, 1000, 6000]
    seeds = [11, 12, 13, 14]
    got = engine.batch_run(dps, n_perm, seeds, lanes=2)
    for dp, n, s, g in zip(dps, n_perm, seeds, got):
        a = dp.run(n, seed=s)
        assert optimum(g.unpermuted) == optimum(a.unpermuted)
        assert np.array_equal(g.minp, a.minp)
    for dp in dps:
        dp.close()


def test_batch_waves_with_fallbacks(engine):
    # Pairs whose ladders are too tight leave tasks of a wave's sweep to the
    # exhaustive screen, which reads the labels in the sweep's form: every
    # minimum equals the exhaustive screen's for the same permutation ids
    # (short runs of new pairs, ids 1..1000 and 1001..n).
    specs = [(synth.copula_pair(6000, 0.2, seed=101), 1500, 31),
             (synth.copula_pair(7000, 0.25, seed=102), 1800, 32)]
    refs = []
    for p, n, s in specs:
        parts = []
        for first, count in ((1, 1000), (1001, n - 1000)):
            dq = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
            parts.append(dq.run(count, seed=s, first=first))
            dq.close()
        refs.append((parts[0].unpermuted, np.concatenate([parts[0].minp, parts[1].minp])))
    dps = [engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population) for p, _, _ in specs]
    for dp, (_, n, _), (_, minp) in zip(dps, specs, refs):
        dp.set_ladder(np.sort(minp)[: int(0.3 * n)])
    got = engine.batch_run(dps, [n for _, n, _ in specs], [s for _, _, s in specs])
    # one wave (both grids 16 columns a lane): one sweep launch for the two
    assert sum(g.summary["sweep0_launches"] for g in got) == 1
    for g, (unperm, minp) in zip(got, refs):
        assert g.summary["n_route"]["fallback"] > 0, g.summary["n_route"]
        assert optimum(g.unpermuted) == optimum(unperm)
        assert np.array_equal(g.minp, minp)
    for dp in dps:
        dp.close()


def test_batch_waves_equal_single_runs(engine):
    # Pairs that have run before (so they have a ladder) and short screen
    # runs go through waves: the tasks of several pairs in one multi-pair
    # sweep, grouped by grid width.  Each pair's results equal its own run's
    # bit for bit; the same pair twice (other seeds) shares its table
    # screens; the long run, the run of lists over different features and the
    # short one take a server lane beside the waves.
    specs = [(synth.copula_pair(2000, 0.1, seed=90), 2500, 21),
             (synth.copula_pair(9000, 0.3, seed=91), 4000, 22),
             (synth.copula_pair(15000, 0.0, seed=92), 1500, 23),
             (synth.copula_pair(20000, 0.2, seed=93), 10000, 24),
             (synth.copula_pair(6000, 0.3, seed=94, frac_tied2=0.1), 3000, 25),
             (None, 6000, 26),  # the pair before again
             (synth.copula_pair(12000, 0.2, seed=95), 40000, 27),  # long: a lane
             (synth.small_pair(4000, 0.2, seed=96, subset1=3600, subset2=3800), 3000, 28),  # a lane
             (synth.copula_pair(5000, 0.2, seed=97), 600, 29)]  # short: a lane
    dps = [engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population) if p else None
           for p, _, _ in specs]
    dps[5] = dps[3]
    for dp, (_, n, _) in zip(dps, specs):
        dp.run(n, seed=99)  # each pair's ladder
    n_perm = [n for _, n, _ in specs]
    seeds = [s for _, _, s in specs]
    got = engine.batch_run(dps, n_perm, seeds)
    # six runs in waves: one sweep launch per wave, counted with its first run
    launches = [g.summary["sweep0_launches"] for g in got]
    assert sum(launches[:6]) < 6, launches
    for dp, n, s, g in zip(dps, n_perm, seeds, got):
        a = dp.run(n, seed=s)
        assert optimum(g.unpermuted) == optimum(a.unpermuted), (n, s)
        assert np.array_equal(g.minp, a.minp), (n, s)
        assert g.summary["count_le"] == a.summary["count_le"]
        assert g.summary["empirical_pvalue"] == a.summary["empirical_pvalue"]
        assert sum(g.summary["n_route"].values()) == n + 1
    # a second batch finds the pairs' table screens and ladders
    again = engine.batch_run(dps[:6], n_perm[:6], seeds[:6])
    for g, h in zip(got, again):
        assert np.array_equal(g.minp, h.minp)
    for q, dp in enumerate(dps):
        if q != 5:
            dp.close()


def test_memory_admission_and_errors(engine):
    from dual_threshold_optimization_gb300._lib import lib
    p = synth.copula_pair(8000, 0.2, seed=90)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    need = lib().dto_run_device_bytes(dp.handle, 5000)
    assert need > 0
    # a budget of one request: the requests run one after another, and one
    # larger than the budget still runs (alone)
    with engine.server(lanes=3, mem_budget=need) as srv:
        jobs = [srv.submit(dp, 5000, seed=s) for s in (1, 2, 3)]
        big = srv.submit(dp, 20000, seed=4)
        peak = 0
        while not all(j.done() for j in jobs + [big]):
            peak = max(peak, srv.stats()["running"])
            time.sleep(0.0005)
        res = [j.wait() for j in jobs]
        rb = big.wait()
        assert peak <= 1
        with pytest.raises(DtoError):
            srv.submit(dp, 10, precision=7)
    for s, r in zip((1, 2, 3), res):
        assert np.array_equal(r.minp, dp.run(5000, seed=s).minp)
    assert np.array_equal(rb.minp, dp.run(20000, seed=4).minp)
    dp.close()


def test_bounded_wait_and_cancel(engine):
    # A one-lane server: a long request runs while a short one waits behind it.
    # A wait with a 1 ms limit on the queued request gives up (DTO_ERR_TIMEOUT)
    # and leaves it known; cancelling it takes it out of the queue
    # (DTO_ERR_CANCELLED).  Cancelling the running request stops it at a batch
    # boundary, its kernels drained (or it had finished: its results stand).
    # The server then serves a new request with the same results as a run
    # alone.  Nothing here interrupts a kernel.
    from dual_threshold_optimization_gb300._lib import DTO_ERR_CANCELLED, DTO_ERR_TIMEOUT
    big = synth.copula_pair(20000, 0.2, seed=2)
    dbig = engine.pair(big.ranks1, big.feat1, big.ranks2, big.feat2, big.n_features, big.population)
    p = synth.copula_pair(3000, 0.2, seed=5)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    want = dp.run(3000, seed=9).minp
    with engine.server(lanes=1) as srv:
        running = srv.submit(dbig, 400_000, seed=1)
        queued = srv.submit(dp, 3000, seed=9)
        with pytest.raises(DtoError) as e:
            queued.wait(timeout_ms=1.0)
        assert e.value.status == DTO_ERR_TIMEOUT
        assert srv.stats()["queued"] + srv.stats()["running"] >= 1
        queued.cancel()
        with pytest.raises(DtoError) as e:
            queued.wait()
        assert e.value.status == DTO_ERR_CANCELLED
        running.cancel()
        try:
            running.wait()
        except DtoError as err:
            assert err.status == DTO_ERR_CANCELLED
        again = srv.submit(dp, 3000, seed=9)
        assert np.array_equal(again.wait(timeout_ms=60_000).minp, want)
        assert srv.stats()["queued"] == 0 and srv.stats()["running"] == 0
    dbig.close()
    dp.close()
