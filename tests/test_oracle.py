"""The CPU oracle pinned against the reference's own goldens and exact values.

No GPU: these tests check the checker.  Goldens: tests/golden/reference_golden.json
(made by tests/golden/make_golden.py from the reference's test_data, README,
unit tests and doctests).
"""
import itertools
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))


def exact_sf(N, K, n, k):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 400
    lo, hi = max(0, K + n - N), min(K, n)
    if k <= lo:
        return mpmath.mpf(1)
    num = sum(mpmath.binomial(K, j) * mpmath.binomial(N - K, n - j) for j in range(k, hi + 1))
    return num / mpmath.binomial(N, n)


def test_philox_known_answers():
    # Random123 known-answer vectors for Philox4x32-10
    assert [int(x) for x in O.philox4x32_10([0, 0, 0, 0], [0, 0])] == \
        [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert [int(x) for x in O.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2)] == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert [int(x) for x in O.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                            [0xa4093822, 0x299f31d0])] == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_log_factorial_table_vs_mpmath():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    hi, lo = O.lf_table(70000)
    for m in (0, 1, 2, 3, 10, 99, 100, 1000, 12345, 20000, 59999, 60000, 70000):
        exact = mpmath.loggamma(m + 1)
        got = mpmath.mpf(float(hi[m])) + mpmath.mpf(float(lo[m]))
        assert abs(got - exact) <= mpmath.mpf(1e-25) * max(1, abs(exact)), m


@pytest.mark.parametrize("case", GOLDEN["hypergeometric"], ids=lambda c: str(c["args"]))
def test_hypergeometric_goldens(case):
    p = O.sf64(*case["args"])
    if "abs_tol" in case:
        assert abs(p - case["p"]) <= case["abs_tol"]
    else:
        # the reference's exact-equality doctests hold statrs 0.17.1's bits, which
        # differ from the exact value by up to 1.2e-11 relative
        assert abs(p - case["p"]) <= 1.3e-11 * case["p"]
    ex = exact_sf(*case["args"])
    assert abs(p - float(ex)) <= 1e-14 * float(ex) + 1e-300


def test_sf64_vs_mpmath_random():
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(300):
        N = int(rng.integers(1, 3000))
        K = int(rng.integers(0, N + 1))
        n = int(rng.integers(0, N + 1))
        lo, hi = max(0, K + n - N), min(K, n)
        k = int(rng.integers(lo, hi + 1))
        p = O.sf64(N, K, n, k)
        ex = float(exact_sf(N, K, n, k))
        if ex > 1e-300:
            worst = max(worst, abs(p - ex) / ex)
    assert worst < 1e-13, worst


def test_sf64_large_n_tails():
    # N = 20,000 cells of the kind the null search sees, including far tails
    for (N, K, n, k) in [(20000, 10000, 10000, 5200), (20000, 10272, 11465, 6593),
                         (20000, 300, 400, 30), (20000, 5, 5, 3), (20000, 19000, 18000, 17200)]:
        p = O.sf64(N, K, n, k)
        ex = float(exact_sf(N, K, n, k))
        assert abs(p - ex) <= 2e-13 * ex, (N, K, n, k, p, ex)


def test_sf64_symmetry_and_edges():
    assert O.sf64(10, 1, 1, 0) == 1.0          # k == 0 (hypergeometric_pvalue.rs:44-46)
    assert O.sf64(30, 24, 13, 7) == 1.0        # k at the bottom of the support
    assert O.sf64(30, 5, 6, 6) == 0.0          # k above min(K, n)
    rng = np.random.default_rng(2)
    for _ in range(200):
        N = int(rng.integers(2, 5000))
        K = int(rng.integers(0, N + 1))
        n = int(rng.integers(0, N + 1))
        k = int(rng.integers(max(0, K + n - N), min(K, n) + 1))
        assert O.sf64(N, K, n, k) == O.sf64(N, n, K, k)


def test_thresholds_series_and_quirk():
    t = O.thresholds(200)
    assert list(t[:3]) == [1, 2, 3]
    assert list(t[97:102]) == [98, 99, 100, 102, 104]
    # ranked.rs:369-374: the last threshold is not clamped to the max rank
    assert O.thresholds(101)[-1] == 100
    assert len(O.thresholds(0)) == 0
    assert len(O.thresholds(20000)) == 589


def _ids(rows, ids):
    return [ids.setdefault(g, len(ids)) for g in rows]


def test_readme_golden_and_literal_mode():
    td = GOLDEN["test_data"]
    ids = {}
    r1, f1 = O.stable_sort([r for _, r in td["ranklist1"]], _ids([g for g, _ in td["ranklist1"]], ids))
    r2, f2 = O.stable_sort([r for _, r in td["ranklist2"]], _ids([g for g, _ in td["ranklist2"]], ids))
    e = td["expected"]
    for mode in ("hist", "literal"):
        b, _ = O.optimize(r1, f1, r2, f2, len(ids), 30, mode=mode)
        assert (b["rank1"], b["rank2"], b["set1_len"], b["set2_len"], b["intersection_size"]) == (
            e["rank1"], e["rank2"], e["set1_len"], e["set2_len"], e["unpermuted_intersection_size"])
        assert abs(b["pvalue"] - e["unpermuted_pvalue"]) <= 1e-14 * e["unpermuted_pvalue"]


def test_optimize_10_golden():
    g = GOLDEN["optimize_10"]
    ids = {}
    r1, f1 = O.stable_sort(g["ranks1"], _ids(g["genes1"], ids))
    r2, f2 = O.stable_sort(g["ranks2"], _ids(g["genes2"], ids))
    b, _ = O.optimize(r1, f1, r2, f2, len(ids), g["population"])
    assert (b["rank1"], b["rank2"]) == (3, 4)
    assert abs(b["pvalue"] - g["expected"]["pvalue"]) <= 1e-12


def test_grid_3x3_has_nine_records():
    g = GOLDEN["grid_3x3"]
    _, recs = O.optimize(g["ranks1"], [0, 1, 2], g["ranks2"], [0, 1, 3], 4, 4, all_records=True)
    assert len(recs) == g["records"]


def random_pair(rng, N, ties=0.0, sub1=None, sub2=None):
    r1 = rng.permutation(N) + 1
    r2 = rng.permutation(N) + 1
    if ties:
        r2 = np.where(rng.random(N) < ties, np.maximum(1, r2 - rng.integers(0, 4, N)), r2)
    f = np.arange(N)
    k1 = np.sort(rng.choice(N, sub1 or N, replace=False))
    k2 = np.sort(rng.choice(N, sub2 or N, replace=False))
    a = O.stable_sort(r1[k1], f[k1])
    b = O.stable_sort(r2[k2], f[k2])
    return a, b


@pytest.mark.parametrize("seed", range(6))
def test_literal_equals_histogram(seed):
    rng = np.random.default_rng(seed)
    N = int(rng.integers(5, 40))
    (r1, f1), (r2, f2) = random_pair(rng, N, ties=0.3 * (seed % 2), sub1=max(2, N - seed),
                                     sub2=max(2, N - 2 * seed))
    for _ in range(3):
        i1 = rng.permutation(len(r1)).astype(np.int32)
        i2 = rng.permutation(len(r2)).astype(np.int32)
        a, ra = O.optimize(r1, f1, r2, f2, N, N, i1, i2, mode="hist", all_records=True)
        b, rb = O.optimize(r1, f1, r2, f2, N, N, i1, i2, mode="literal", all_records=True)
        assert a == b
        assert ra == rb


def test_fdr_and_empirical_goldens():
    for c in GOLDEN["fdr"]:
        assert abs(O.fdr(*c["args"]) - c["value"]) <= c["abs_tol"]
    e = GOLDEN["empirical"]
    assert O.empirical(e["unpermuted"]["pvalue"], e["permuted_pvalues"]) == \
        e["expected"]["empirical_pvalue"]
    u = e["unpermuted"]
    assert O.fdr(u["set1_len"], u["set2_len"], u["intersection_size"], u["population_size"]) == \
        e["expected"]["fdr"]
    assert O.empirical(0.5, []) == 1.0


def test_shuffle_is_a_uniform_permutation():
    # every permutation of 4 elements equally likely (chi-square, 23 dof)
    counts = {}
    n = 12000
    for t in range(1, n + 1):
        s = tuple(O.shuffle(99, 0, t, 1, 4).tolist())
        counts[s] = counts.get(s, 0) + 1
    assert len(counts) == 24
    exp = n / 24.0
    chi2 = sum((c - exp) ** 2 / exp for c in counts.values())
    assert chi2 < 60.0, chi2  # p < 1e-4 under uniformity
    for L in (1, 2, 17, 1023, 1024, 1025, 5000):
        s = O.shuffle(5, 3, 7, 2, L)
        assert sorted(s.tolist()) == list(range(L))


def test_shuffle_position_marginals():
    # element e lands at position p with probability 1/L (L = 64, many draws)
    L, n = 64, 4000
    pos = np.zeros((L, L))
    for t in range(n):
        s = O.shuffle(1234, 1, t + 1, 1, L)
        pos[s, np.arange(L)] += 1
    exp = n / L
    chi2 = ((pos - exp) ** 2 / exp).sum()
    dof = (L - 1) ** 2
    assert abs(chi2 - dof) < 6 * math.sqrt(2 * dof), chi2


def test_shuffle_within_bucket_orders_are_uniform():
    # Lists long enough that buckets hold several elements: recompute each
    # element's bucket from the Philox blocks (8 elements a block, a 16-bit
    # half each, its top 12 bits), check that every bucket holds exactly its
    # elements, and that every bucket of size 3 comes out in each of its 6
    # orders equally often (the Fisher-Yates pass on the bucket's own stream)
    # and every bucket of size 2 swapped half the time.
    L, n = 12288, 40
    seed, pair, tag = 77, 0, 1
    bucket = np.zeros(L, np.uint32)
    c3 = {}
    swaps2 = tot2 = 0
    for t in range(1, n + 1):
        for g in range((L + 7) // 8):
            w = O.philox4x32_10([g, t, pair, 0x10000000 | (tag << 24)], [seed & 0xFFFFFFFF, seed >> 32])
            halves = np.array([(x >> (16 * h)) & 0xFFFF for x in w for h in (0, 1)], np.uint32)
            bucket[8 * g:8 * g + 8] = (halves >> 4)[:min(8, L - 8 * g)]
        s = O.shuffle(seed, pair, t, tag, L)
        starts = np.searchsorted(np.sort(bucket), np.arange(4097))
        for b in range(4096):
            seg = s[starts[b]:starts[b + 1]]
            assert np.all(bucket[seg] == b)
            if len(seg) == 2:
                tot2 += 1
                swaps2 += int(seg[0] > seg[1])
            elif len(seg) == 3:
                key = tuple(np.argsort(np.argsort(seg)).tolist())
                c3[key] = c3.get(key, 0) + 1
    assert abs(swaps2 - tot2 / 2) < 5 * math.sqrt(tot2 / 4), (swaps2, tot2)
    m3 = sum(c3.values())
    exp = m3 / 6.0
    chi2 = sum((c - exp) ** 2 / exp for c in c3.values())
    assert len(c3) == 6 and chi2 < 25.0, (chi2, c3)