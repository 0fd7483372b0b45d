"""GPU parity against the CPU oracle, through the C ABI.

Bar: thresholds, set sizes and overlaps bit-exact; p-values identical bits
(the kernels and the oracle implement the same FP64 specification); both
precision modes give the same argmin.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from dual_threshold_optimization_gb300 import synth
from helpers import optimum, same_records

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")
KEYS = ("rank1", "rank2", "set1_len", "set2_len", "intersection_size", "pvalue")


def sorted_lists(p):
    (r1, f1), (r2, f2) = p.sorted_lists()
    return r1, f1, r2, f2


def assert_same(gpu, ora, what=""):
    for k in KEYS:
        assert gpu[k] == ora[k], "%s: %s gpu=%r oracle=%r" % (what, k, gpu[k], ora[k])


def oracle_best(p, idx1=None, idx2=None, mode="hist"):
    r1, f1, r2, f2 = sorted_lists(p)
    best, _ = O.optimize(r1, f1, r2, f2, p.n_features, p.population, idx1, idx2, mode=mode)
    return best


CASES = [
    ("plain", dict(N=80, rho=0.3, seed=5)),
    ("ties", dict(N=150, rho=0.2, seed=6, frac_tied2=0.3)),
    ("background", dict(N=140, rho=0.4, seed=7, subset1=120, subset2=110)),
    ("tiny", dict(N=7, rho=0.0, seed=8)),
    ("strong", dict(N=300, rho=0.9, seed=9)),
]


@pytest.mark.parametrize("name,kw", CASES)
@pytest.mark.parametrize("precision", ["fp64", "screen"])
def test_unpermuted_and_test_mode_vs_oracle(engine, name, kw, precision):
    p = synth.small_pair(**kw)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    rng = np.random.default_rng(100 + kw["seed"])
    P = 12
    idx = np.zeros((P, dp.N1 + dp.N2), np.int32)
    for b in range(P):
        idx[b, :dp.N1] = rng.permutation(dp.N1)
        idx[b, dp.N1:] = rng.permutation(dp.N2)
    res = dp.run(P, perm_idx=idx, precision=precision, want_records=True)
    ora = oracle_best(p)
    assert_same(res.unpermuted, ora, "unpermuted")
    for b in range(P):
        ob = oracle_best(p, idx[b, :dp.N1], idx[b, dp.N1:])
        assert_same(dict(zip(res.records.dtype.names, res.records[b].tolist())), ob, "perm %d" % b)
        assert res.minp[b] == ob["pvalue"]
    if kw["N"] <= 150:
        # literal per-cell set intersection (intersect_genes.rs) agrees too
        ol = oracle_best(p, idx[0, :dp.N1], idx[0, dp.N1:], mode="literal")
        assert_same(dict(zip(res.records.dtype.names, res.records[0].tolist())), ol, "literal")


def test_reference_test_data_golden(engine):
    g = json.load(open(GOLDEN))
    td = g["test_data"]
    ids = {}
    f1 = [ids.setdefault(n, len(ids)) for n, _ in td["ranklist1"]]
    f2 = [ids.setdefault(n, len(ids)) for n, _ in td["ranklist2"]]
    r1 = [r for _, r in td["ranklist1"]]
    r2 = [r for _, r in td["ranklist2"]]
    dp = engine.pair(r1, f1, r2, f2, len(ids), 30)
    for prec in ("fp64", "screen"):
        res = dp.run(0, precision=prec)
        e = td["expected"]
        u = res.unpermuted
        assert (u["rank1"], u["rank2"], u["set1_len"], u["set2_len"], u["intersection_size"]) == (
            e["rank1"], e["rank2"], e["set1_len"], e["set2_len"], e["unpermuted_intersection_size"])
        assert abs(u["pvalue"] - e["unpermuted_pvalue"]) <= 1e-12 * e["unpermuted_pvalue"]
        assert res.summary["empirical_pvalue"] == 1.0


def test_optimize_10_golden(engine):
    g = json.load(open(GOLDEN))["optimize_10"]
    ids = {}
    f1 = [ids.setdefault(n, len(ids)) for n in g["genes1"]]
    f2 = [ids.setdefault(n, len(ids)) for n in g["genes2"]]
    dp = engine.pair(g["ranks1"], f1, g["ranks2"], f2, len(ids), g["population"])
    r = dp.optimize(permute=False, precision="screen")
    assert (r["rank1"], r["rank2"]) == (g["expected"]["rank1"], g["expected"]["rank2"])
    assert abs(r["pvalue"] - g["expected"]["pvalue"]) <= 1e-12


def test_hypergeom_batch_bit_exact(engine):
    g = json.load(open(GOLDEN))
    rng = np.random.default_rng(3)
    qs = [tuple(c["args"]) for c in g["hypergeometric"]]
    for _ in range(400):
        N = int(rng.integers(1, 30000))
        K = int(rng.integers(0, N + 1))
        n = int(rng.integers(0, N + 1))
        lo, hi = max(0, K + n - N), min(K, n)
        k = int(rng.integers(lo, hi + 1))
        qs.append((N, K, n, k))
    q = np.array(qs, np.int64)
    out = engine.hypergeom_sf(q[:, 0], q[:, 1], q[:, 2], q[:, 3])
    for t, (N, K, n, k) in enumerate(qs):
        assert out[t] == O.sf64(N, K, n, k), (N, K, n, k)
    for t, c in enumerate(g["hypergeometric"]):
        tol = c.get("abs_tol") or 1.3e-11 * c["p"]
        assert abs(out[t] - c["p"]) <= tol


@pytest.mark.parametrize("kw", [dict(N=200, rho=0.2, seed=21),
                                dict(N=180, rho=0.2, seed=22, subset1=150, subset2=170)])
def test_philox_permutations_match_spec_and_test_mode(engine, kw):
    p = synth.small_pair(**kw)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    seed, P = 0x1234_5678_9ABC, 16
    i1, i2 = dp.export_permutations(seed, 1, P)
    same = dp.n_common == dp.N1 == dp.N2
    for b in range(P):
        assert np.array_equal(np.sort(i1[b]), np.arange(dp.N1))
        assert np.array_equal(np.sort(i2[b]), np.arange(dp.N2))
    res_ph = dp.run(P, seed=seed, precision="screen", want_records=True)
    res_tm = dp.run(P, perm_idx=np.concatenate([i1, i2], axis=1), precision="screen", want_records=True)
    assert np.array_equal(res_ph.minp, res_tm.minp)
    assert same_records(res_ph.records, res_tm.records)
    # the device permutations follow the oracle's restatement of the spec
    # (stream id 0 by default)
    for b in range(P):
        assert np.array_equal(O.shuffle(seed, 0, b + 1, 1, dp.N1), i1[b])
        if not same:
            assert np.array_equal(O.shuffle(seed, 0, b + 1, 2, dp.N2), i2[b])
    dp.set_stream(7)
    j1, _ = dp.export_permutations(seed, 1, 1)
    assert np.array_equal(O.shuffle(seed, 7, 1, 1, dp.N1), j1[0])


def test_screen_equals_fp64_medium(engine):
    p = synth.copula_pair(3000, 0.25, seed=31, frac_tied2=0.1)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    a = dp.run(24, seed=99, precision="screen", want_records=True)
    b = dp.run(24, seed=99, precision="fp64", want_records=True)
    assert optimum(a.unpermuted) == optimum(b.unpermuted)
    assert same_records(a.records, b.records)
    # and the oracle agrees on the unpermuted task and one permutation
    assert_same(a.unpermuted, oracle_best(p), "unpermuted")
    i1, i2 = dp.export_permutations(99, 3, 1)
    ob = oracle_best(p, i1[0], i2[0])
    assert_same(dict(zip(a.records.dtype.names, a.records[2].tolist())), ob, "perm 3")


def test_grid_dump_matches_oracle_records(engine):
    p = synth.small_pair(N=60, rho=0.3, seed=41, frac_tied2=0.2)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    recs = dp.grid_dump()
    r1, f1, r2, f2 = sorted_lists(p)
    _, allr = O.optimize(r1, f1, r2, f2, p.n_features, p.population, all_records=True)
    assert len(recs) == len(allr)
    for q, o in enumerate(allr):
        g = dict(zip(recs.dtype.names, recs[q].tolist()))
        assert_same(g, o, "cell %d" % q)


def test_table_screen_equals_fp64_many_permutations(engine):
    # enough permutations that the run switches to the table screen after its
    # first batch; every permutation's optimum must equal the plain FP64 path's
    p = synth.copula_pair(900, 0.2, seed=51, frac_tied2=0.05)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    P = 7400
    a = dp.run(P, seed=123, precision="screen", want_records=True)
    b = dp.run(P, seed=123, precision="fp64", want_records=True)
    assert optimum(a.unpermuted) == optimum(b.unpermuted)
    assert same_records(a.records, b.records)
    assert a.summary["n_fallback"] > 0  # the 85th-percentile level 0 leaves ~15 % to the later levels


@pytest.mark.parametrize("kind", ["same_set", "general"])
def test_pipelined_batches_equal_short_runs(engine, kind):
    # a run long enough for several label batches after the first one
    # (batches in flight, slots reused) must give every permutation the
    # optimum that short runs of the same permutation ids give
    if kind == "same_set":
        p = synth.copula_pair(20000, 0.2, seed=57)
        P = 170000  # 512 + 53,687 x 3 + 8,427 at 40,000 label bytes a permutation: a slot reused
    else:
        p = synth.small_pair(20000, 0.2, seed=58, subset1=19000, subset2=19500)
        P = 15000  # 512 + 6,972 + 6,972 + 544 at 1 GiB of two-list index scratch
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    long_run = dp.run(P, seed=99, precision="screen", want_records=True)
    step = 2000  # at most 2,048: the exhaustive screen alone
    for first in range(1, P + 1, step):
        n = min(step, P + 1 - first)
        short = dp.run(n, seed=99, first=first, precision="screen", want_records=True)
        assert optimum(short.unpermuted) == optimum(long_run.unpermuted)
        assert same_records(short.records, long_run.records[first - 1:first - 1 + n]), first
    s = long_run.summary
    assert s["empirical_pvalue"] == np.mean(long_run.minp <= long_run.unpermuted["pvalue"])
    dp.close()


def test_table_sweep_beyond_16_bit_overlaps(engine):
    # 40,000 shared features: overlaps exceed 0x7FFF, so the table entries
    # wrap in their 16-bit halves (each clamped to its cell's overlap range,
    # the low half's carry taken back by the high one); the optima must
    # equal the exhaustive screen's (runs of
    # at most 2,048 permutations take the exhaustive screen alone)
    p = synth.copula_pair(40000, 0.1, seed=59)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    P = 3000
    long_run = dp.run(P, seed=7, precision="screen", want_records=True)
    assert long_run.summary["n_launches"] > 0
    for first, n in ((1, 1500), (1501, 1500)):
        short = dp.run(n, seed=7, first=first, precision="screen", want_records=True)
        assert optimum(short.unpermuted) == optimum(long_run.unpermuted)
        assert same_records(short.records, long_run.records[first - 1:first - 1 + n])
    dp.close()


@pytest.mark.parametrize("kw", [dict(N=3000, rho=0.2, seed=23),
                                dict(N=3000, rho=0.2, seed=24, subset1=2600, subset2=2800)])
def test_test_mode_through_the_table_sweep(engine, kw):
    # uploaded index arrays through the table sweep (a pair with a ladder):
    # the compose kernel writes their labels in the sweep's form; with a
    # ladder tight enough to leave tasks to the exhaustive screen, every
    # optimum equals the exhaustive screen's for the same permutations
    p = synth.small_pair(**kw)
    dq = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    seed = 0xABCDEF
    ref = dq.run(1000, seed=seed, want_records=True)
    assert set(np.unique(ref.records["route"]).tolist()) == {1}
    i1, i2 = dq.export_permutations(seed, 1, 1000)
    dq.close()
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    dp.set_ladder(np.sort(ref.minp)[:300])
    tm = dp.run(1000, perm_idx=np.concatenate([i1, i2], axis=1), want_records=True)
    routes = set(np.unique(tm.records["route"]).tolist())
    assert 5 in routes and 1 not in routes, routes
    assert optimum(tm.unpermuted) == optimum(ref.unpermuted)
    assert same_records(tm.records, ref.records)
    dp.close()


@pytest.mark.parametrize("N", [3, 7, 8, 9, 17, 33])
def test_philox_permutations_tiny_lists(engine, N):
    # lists shorter than one 16-byte label chunk and grids of one-element rows:
    # the device permutations follow the spec, and the label path (which
    # shuffles only the buckets a row starts inside) gives the optima of the
    # full permutations
    p = synth.small_pair(N=N, rho=0.2, seed=60 + N)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    seed, P = 77, 40
    i1, i2 = dp.export_permutations(seed, 1, P)
    for b in range(P):
        assert np.array_equal(O.shuffle(seed, 0, b + 1, 1, dp.N1), i1[b])
    res_ph = dp.run(P, seed=seed, precision="screen", want_records=True)
    res_tm = dp.run(P, perm_idx=np.concatenate([i1, i2], axis=1), precision="screen", want_records=True)
    assert np.array_equal(res_ph.minp, res_tm.minp)
    assert same_records(res_ph.records, res_tm.records)
    dp.close()


@pytest.mark.parametrize("N", [30000, 40000])
def test_philox_permutations_long_lists_match_spec(engine, N):
    # 30,000 elements: the kernel keeps every Philox word in shared memory;
    # 40,000: it recomputes a word where the shuffle needs it.  Same spec.
    p = synth.copula_pair(N, 0.1, seed=60)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    seed = 0xFEEDFACE
    i1, _ = dp.export_permutations(seed, 11, 3)
    for b in range(3):
        assert np.array_equal(O.shuffle(seed, 0, 11 + b, 1, N), i1[b])
    dp.close()


def test_tuned_level0_quantile_changes_no_result(fresh_engine):
    # dto_pair_tune times 0.80, 0.85 and 0.90 and keeps the fastest; the
    # quantile only moves the level-0 bound, so every optimum stays; a new
    # pair of the same shape starts with the tuned quantile
    from dual_threshold_optimization_gb300._lib import DtoError
    engine = fresh_engine
    p = synth.copula_pair(6000, 0.3, seed=81, frac_tied2=0.1)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    ref = dp.run(3000, seed=5, want_records=True)
    best = dp.tune(3000, seed=100)
    assert best in (0.80, 0.85, 0.90)
    again = dp.run(3000, seed=5, want_records=True)
    assert optimum(again.unpermuted) == optimum(ref.unpermuted)
    assert same_records(again.records, ref.records)
    dq = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    other = dq.run(3000, seed=5, want_records=True)
    assert same_records(other.records, ref.records)
    dp.set_level0_quantile(0.7)
    assert same_records(dp.run(3000, seed=5, want_records=True).records, ref.records)
    with pytest.raises(DtoError):
        dp.set_level0_quantile(0.3)
    with pytest.raises(DtoError):
        dp.tune(500)
    dp.close()
    dq.close()


@pytest.mark.parametrize("N,scale2,C", [(100, 1, 4), (600, 1, 8), (1500, 1, 12), (3000, 1, 16),
                                        (40000, 1, 24), (3000, 100, 28), (3000, 400, 32)])
def test_table_path_and_fallbacks_at_every_grid_width(engine, N, scale2, C):
    # Table runs draw labels in the sweep's form (a count's byte offset in a
    # lane layout that depends on the grid width C); the exhaustive screen
    # turns them back for the tasks no level settles.  A ladder from the
    # lowest 30 % of the minima leaves many tasks to it; every optimum must
    # equal the exhaustive screen's (a new pair's short run).  Sparse list-2
    # ranks give the widest grids.
    p = synth.copula_pair(N, 0.3, seed=90 + N + scale2)
    r2 = p.ranks2 * scale2
    dq = engine.pair(p.ranks1, p.feat1, r2, p.feat2, p.n_features, p.population)
    assert min(c for c in (4, 8, 12, 16, 20, 24, 28, 32) if 32 * c >= dq.n2) == C, dq.n2
    ref = dq.run(1000, seed=31, want_records=True)
    assert set(np.unique(ref.records["route"]).tolist()) == {1}
    dq.close()
    dp = engine.pair(p.ranks1, p.feat1, r2, p.feat2, p.n_features, p.population)
    dp.set_ladder(np.sort(ref.minp)[:300])
    res = dp.run(1000, seed=31, want_records=True)
    routes = set(np.unique(res.records["route"]).tolist())
    assert 5 in routes and 1 not in routes, routes  # fallbacks; no exhaustive first batch
    assert optimum(res.unpermuted) == optimum(ref.unpermuted)
    assert same_records(res.records, ref.records)
    dp.close()


def test_short_runs_of_a_pair_with_a_ladder(fresh_engine):
    # a short screen run (at least 256 permutations) leaves the pair a
    # ladder; the pair's later short runs go through the table sweep (the
    # exhaustive screen only for the unpermuted task) with the optima of the
    # exhaustive screen, which a new pair's first short run still takes
    engine = fresh_engine
    p = synth.copula_pair(6000, 0.3, seed=82, frac_tied2=0.1)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    first = dp.run(1000, seed=5, want_records=True)
    assert set(np.unique(first.records["route"]).tolist()) == {1}
    short = dp.run(1000, seed=6, want_records=True)
    assert 1 not in set(np.unique(short.records["route"]).tolist())
    assert short.summary["n_route"]["screen"] == 1  # the unpermuted task
    dq = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    exhaustive = dq.run(1000, seed=6, want_records=True)
    assert set(np.unique(exhaustive.records["route"]).tolist()) == {1}
    assert optimum(short.unpermuted) == optimum(exhaustive.unpermuted)
    assert same_records(short.records, exhaustive.records)
    assert short.summary["count_le"] == exhaustive.summary["count_le"]
    # under 256 permutations: the exhaustive screen
    tiny = dp.run(200, seed=7, want_records=True)
    assert set(np.unique(tiny.records["route"]).tolist()) == {1}
    dp.close()
    dq.close()


def test_ladder_left_by_a_closed_pair(fresh_engine):
    # a run leaves its ladder for the next reader; the pair closed first, a
    # new pair of its shape still starts from it (no first batch) and gets
    # the same results
    engine = fresh_engine
    p = synth.copula_pair(5000, 0.25, seed=64)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    cold = dp.run(6000, seed=21, want_records=True)
    assert 1 in set(np.unique(cold.records["route"]).tolist())
    dp.close()
    dq = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    warm = dq.run(6000, seed=21, want_records=True)
    assert 1 not in set(np.unique(warm.records["route"]).tolist())
    assert optimum(warm.unpermuted) == optimum(cold.unpermuted)
    assert same_records(warm.records, cold.records)
    # a new quantile applies the ladder the last run left, then rebuilds it
    dq.set_level0_quantile(0.9)
    again = dq.run(6000, seed=21, want_records=True)
    assert same_records(again.records, cold.records)
    dq.close()


def test_warm_ladder_gives_the_same_results(fresh_engine):
    # the first long run of a pair measures its ladder from a first batch; a
    # later run starts from the ladder the earlier run left, and a new pair
    # of the same shape from the context's ladder for that shape: same results
    engine = fresh_engine
    p = synth.copula_pair(5000, 0.25, seed=63, frac_tied2=0.05)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    cold = dp.run(9000, seed=17, want_records=True)
    warm = dp.run(9000, seed=17, want_records=True)
    assert optimum(warm.unpermuted) == optimum(cold.unpermuted)
    assert same_records(warm.records, cold.records)
    assert warm.summary["count_le"] == cold.summary["count_le"]
    other = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    shifted = other.run(4000, seed=17, first=5001, want_records=True)  # the shape's ladder, other ids
    assert same_records(shifted.records, cold.records[5000:9000])
    # warm starts measure no first batch (route 1, the exhaustive screen of
    # the first permutations): the pair's own later run, and the new pair
    # from the ladder its shape's last run left
    for res in (warm, shifted):
        assert 1 not in set(np.unique(res.records["route"]).tolist())
    dp.close()
    other.close()
