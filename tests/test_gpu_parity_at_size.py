"""GPU parity against the CPU oracle at the benchmark sizes, through the C ABI.

The production path of a long run (first batch through the exhaustive screen,
the table ladder's levels 0-2 over pipelined label batches, the exhaustive
screen of what the ladder leaves) is run on the benchmark workloads:

* the headline pair: N = 20,000, copula rho = 0.2, no ties, 100,000 Philox
  permutations (the pair bench.py measures);
* N = 6,000 with ~10 % of list-2 features in tie blocks;
* 25,000-feature rankings restricted to an 18,000-feature background with
  geometric tie blocks (gapped ranks);
* two 20,000-feature lists over different feature sets (two shuffles composed);
* one pair of 60,000 features (700 x 700 thresholds, overlaps beyond 0x7FFF:
  table entries that wrap in their 16-bit halves).

For each run, a sample of permutation ids is taken from every route that
settled tasks (dto_result.route), plus the hardest tasks (largest and smallest
minimum p) and a random sample; their index arrays are exported from the
device and the oracle's optimum of each is compared field by field: thresholds,
set sizes and overlap bit-exact, p-value identical bits (the kernels and the
oracle implement one FP64 specification).  The unpermuted optimum, the
empirical p-value and count_le of the whole run are checked too.  Each pair is
run cold (its first long run measures the ladder) and warm (a later run starts
from the stored ladder).
"""
import zlib

import numpy as np
import pytest

from dual_threshold_optimization_gb300 import synth
from dual_threshold_optimization_gb300._lib import ROUTE_NAMES
from oracle import oracle as O
from oracle.pool import optimize_many

pytestmark = pytest.mark.gpu

SCREEN, LEVEL0, LEVEL1, LEVEL2, FALLBACK = 1, 2, 3, 4, 5
FIELDS = ("rank1", "rank2", "set1_len", "set2_len", "intersection_size", "pvalue", "i", "j")


def _pick(res, rng, per_route, n_random, n_extreme):
    routes = res.records["route"]
    ids = set()
    for r in np.unique(routes):
        where = np.flatnonzero(routes == r)
        ids.update(rng.choice(where, size=min(per_route, len(where)), replace=False).tolist())
    order = np.argsort(res.minp, kind="stable")
    ids.update(order[:n_extreme].tolist())
    ids.update(order[-n_extreme:].tolist())
    ids.update(rng.choice(len(routes), size=min(n_random, len(routes)), replace=False).tolist())
    return sorted(ids)


def _check_run(dp, pair, res, seed, rng, per_route=24, n_random=48, n_extreme=8):
    (r1, f1), (r2, f2) = pair.sorted_lists()
    sorted_pair = (r1, f1, r2, f2, pair.n_features, pair.population)
    ids = _pick(res, rng, per_route, n_random, n_extreme)
    jobs = [(None, None)]
    for b in ids:
        i1, i2 = dp.export_permutations(seed, b + 1, 1)
        jobs.append((i1[0], i2[0]))
    bests = optimize_many(sorted_pair, jobs)
    u = res.unpermuted
    for f in FIELDS:
        assert u[f] == bests[0][f], ("unpermuted", f, u[f], bests[0][f])
    for b, ob in zip(ids, bests[1:]):
        rec = res.records[b]
        for f in FIELDS:
            assert rec[f] == ob[f], ("permutation %d (route %s)" % (b + 1, ROUTE_NAMES[rec["route"]]),
                                     f, rec[f], ob[f])
        assert res.minp[b] == ob["pvalue"]
    s = res.summary
    p_obs = u["pvalue"]
    assert s["count_le"] == int(np.count_nonzero(res.minp <= p_obs))
    assert s["empirical_pvalue"] == O.empirical(p_obs, res.minp)
    assert s["fdr"] == O.fdr(u["set1_len"], u["set2_len"], u["intersection_size"], pair.population)
    routes = res.records["route"]
    counted = {ROUTE_NAMES[q]: int(np.count_nonzero(routes == q)) for q in range(7)}
    counted[ROUTE_NAMES[u["route"]]] += 1
    assert counted == s["n_route"]
    return set(np.unique(routes).tolist()), len(ids)


CASES = [
    # name, pair, permutations, routes a cold run must use
    ("n20000_rho0.2", lambda: synth.copula_pair(20000, 0.2, seed=2), 100_000,
     {SCREEN, LEVEL0, LEVEL1, LEVEL2}),
    ("n6000_ties", synth.config1, 30_000, {SCREEN, LEVEL0, LEVEL1}),
    ("background_18000_of_25000_ties", synth.config4, 60_000, {SCREEN, LEVEL0, LEVEL1}),
    ("different_feature_sets_n20000",
     lambda: synth.small_pair(20000, 0.2, seed=58, subset1=19000, subset2=19500), 15_000,
     {SCREEN, LEVEL0}),
    ("n60000_overlaps_beyond_0x7fff", lambda: synth.copula_pair(60000, 0.15, seed=71), 6_000,
     {SCREEN, LEVEL0}),
]


@pytest.mark.parametrize("name,make,P,must", CASES, ids=[c[0] for c in CASES])
def test_production_path_vs_oracle_at_size(fresh_engine, name, make, P, must):
    engine = fresh_engine
    pair = make()
    dp = engine.pair(pair.ranks1, pair.feat1, pair.ranks2, pair.feat2, pair.n_features,
                     pair.population)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    seed = 0x5EED0000 + P
    cold = dp.run(P, seed=seed, precision="screen", want_records=True)
    seen, n = _check_run(dp, pair, cold, seed, rng)
    assert must <= seen, (name, sorted(ROUTE_NAMES[r] for r in seen))
    warm = dp.run(P, seed=seed + 1, precision="screen", want_records=True)
    assert SCREEN not in set(np.unique(warm.records["route"]).tolist())  # no first batch
    _check_run(dp, pair, warm, seed + 1, rng, per_route=12, n_random=24, n_extreme=4)
    dp.close()


def test_config1_as_stated_vs_oracle(engine):
    # N = 6,000 with ties and the stated 1,000 permutations: every task through
    # the exhaustive screen; a quarter of them checked
    pair = synth.config1()
    dp = engine.pair(pair.ranks1, pair.feat1, pair.ranks2, pair.feat2, pair.n_features,
                     pair.population)
    res = dp.run(1000, seed=11, precision="screen", want_records=True)
    assert set(np.unique(res.records["route"]).tolist()) == {SCREEN}
    _check_run(dp, pair, res, 11, np.random.default_rng(1), per_route=250, n_random=0, n_extreme=4)
    dp.close()


def test_fallback_route_at_size(engine):
    # A ladder seeded from the lower 70 % of an earlier run's minima is too
    # tight for the rest: their permutations fall through all three table
    # levels to the exhaustive screen (route "fallback"), whose optima must
    # equal the oracle's like every other route's.
    pair = synth.copula_pair(20000, 0.2, seed=2)
    dp = engine.pair(pair.ranks1, pair.feat1, pair.ranks2, pair.feat2, pair.n_features,
                     pair.population)
    earlier = dp.run(20000, seed=3)
    dp.set_ladder(np.sort(earlier.minp)[:14000])
    res = dp.run(20000, seed=4, precision="screen", want_records=True)
    routes = res.records["route"]
    assert np.count_nonzero(routes == FALLBACK) > 100, res.summary["n_route"]
    seen, _ = _check_run(dp, pair, res, 4, np.random.default_rng(9), per_route=32)
    assert {LEVEL0, LEVEL1, LEVEL2, FALLBACK} <= seen
    # the ladder decides only the route: a run with the pair's own ladder
    # gives the same optima
    dp.set_ladder([])
    again = dp.run(20000, seed=4, precision="screen", want_records=True)
    for f in FIELDS:
        assert np.array_equal(again.records[f], res.records[f]), f
    dp.close()
