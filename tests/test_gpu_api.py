"""The reference-shaped API on the GPU: CLI, optimize, process_threshold_pairs,
run_single_node, hypergeometric_pvalue."""
import json
import os

import numpy as np
import pytest

from dual_threshold_optimization_gb300 import feature_lists as col
from dual_threshold_optimization_gb300 import dto, run, stat_operations

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))


def rlist(genes, ranks):
    return col.RankedFeatureList.from_(col.FeatureList(genes), ranks)


def test_cli_on_reference_test_data(tmp_path, capsys):
    from dual_threshold_optimization_gb300.cli import main
    td = GOLDEN["test_data"]
    for name in ("ranklist1", "ranklist2"):
        (tmp_path / (name + ".csv")).write_text("".join("%s,%d\n" % (g, r) for g, r in td[name]))
    rc = main(["-1", str(tmp_path / "ranklist1.csv"), "-2", str(tmp_path / "ranklist2.csv"),
               "-p", "5", "--seed", "3"])
    assert rc == 0
    out = json.loads(capsys.readouterr().out)
    e = td["expected"]
    for k in ("rank1", "rank2", "set1_len", "set2_len", "population_size",
              "unpermuted_intersection_size"):
        assert out[k] == e[k]
    assert abs(out["unpermuted_pvalue"] - e["unpermuted_pvalue"]) <= 1e-12 * e["unpermuted_pvalue"]
    assert 0.0 <= out["empirical_pvalue"] <= 1.0 and out["fdr"] >= 0.0
    assert list(out) == sorted(out)
    # with the background file: population = |background| = 30 as well
    (tmp_path / "bg.txt").write_text("\n".join(td["background"]) + "\n")
    rc = main(["-1", str(tmp_path / "ranklist1.csv"), "-2", str(tmp_path / "ranklist2.csv"),
               "-b", str(tmp_path / "bg.txt"), "-p", "3", "--seed", "3"])
    assert rc == 0
    assert json.loads(capsys.readouterr().out)["population_size"] == 30


REFERENCE_KEYS = ("empirical_pvalue", "fdr", "population_size", "rank1", "rank2", "set1_len",
                  "set2_len", "unpermuted_intersection_size", "unpermuted_pvalue")
EXTRA_KEYS = ("logp_err_bound_fp32", "logp_err_bound_fp64", "perms_per_s")


def test_cli_output_contract_and_test_mode(tmp_path, capsys):
    # the reference's nine keys, unchanged and in sorted order, plus the three
    # extra keys; --perm-indices runs the uploaded permutations, whose optima
    # equal the oracle's
    from dual_threshold_optimization_gb300 import synth
    from dual_threshold_optimization_gb300.cli import main
    from oracle import oracle as O
    p = synth.copula_pair(400, 0.3, seed=81, frac_tied2=0.1)
    names = p.feature_names()
    for q, (r, f) in enumerate(((p.ranks1, p.feat1), (p.ranks2, p.feat2))):
        (tmp_path / ("l%d.csv" % (q + 1))).write_text("".join("%s,%d\n" % (names[x], y) for x, y in zip(f, r)))
    l1 = col.RankedFeatureList.from_(col.FeatureList([names[f] for f in p.feat1]), p.ranks1)
    l2 = col.RankedFeatureList.from_(col.FeatureList([names[f] for f in p.feat2]), p.ranks2)
    rng = np.random.default_rng(4)
    P = 24
    idx = np.stack([np.concatenate([rng.permutation(400), rng.permutation(400)]) for _ in range(P)])
    np.save(tmp_path / "perms.npy", idx.astype(np.int32))
    rc = main(["-1", str(tmp_path / "l1.csv"), "-2", str(tmp_path / "l2.csv"),
               "--perm-indices", str(tmp_path / "perms.npy")])
    assert rc == 0
    text = capsys.readouterr().out
    out = json.loads(text)
    assert set(out) == set(REFERENCE_KEYS) | set(EXTRA_KEYS)
    assert list(out) == sorted(out)
    ref = [k for k in out if k in REFERENCE_KEYS]
    assert ref == list(REFERENCE_KEYS)
    assert out["logp_err_bound_fp32"] > 0 and 0 < out["logp_err_bound_fp64"] < 1e-12
    assert out["perms_per_s"] > 0
    # the empirical p-value of the uploaded permutations, from the oracle
    r1, f1, r2, f2, nf = col.dense_ids(l1, l2)
    ob, _ = O.optimize(r1, f1, r2, f2, nf, 400)
    pv = [O.optimize(r1, f1, r2, f2, nf, 400, idx[b, :400], idx[b, 400:])[0]["pvalue"] for b in range(P)]
    assert out["unpermuted_pvalue"] == ob["pvalue"]
    assert out["empirical_pvalue"] == O.empirical(ob["pvalue"], pv)
    # text rows work too; a row count that disagrees with -p is an error
    (tmp_path / "perms.txt").write_text("\n".join(",".join(map(str, r)) for r in idx[:5]))
    assert main(["-1", str(tmp_path / "l1.csv"), "-2", str(tmp_path / "l2.csv"),
                 "--perm-indices", str(tmp_path / "perms.txt"), "--precision", "fp64"]) == 0
    o5 = json.loads(capsys.readouterr().out)
    assert o5["empirical_pvalue"] == O.empirical(ob["pvalue"], pv[:5])
    assert o5["logp_err_bound_fp32"] == 0.0
    assert main(["-1", str(tmp_path / "l1.csv"), "-2", str(tmp_path / "l2.csv"), "-p", "7",
                 "--perm-indices", str(tmp_path / "perms.txt")]) == 101
    bad = idx[:2].copy()
    bad[0, 0] = bad[0, 1]
    np.save(tmp_path / "bad.npy", bad.astype(np.int32))
    assert main(["-1", str(tmp_path / "l1.csv"), "-2", str(tmp_path / "l2.csv"),
                 "--perm-indices", str(tmp_path / "bad.npy")]) == 101
    assert "not a permutation" in capsys.readouterr().err


def test_optimize_and_debug():
    g = GOLDEN["optimize_10"]
    l1, l2 = rlist(g["genes1"], g["ranks1"]), rlist(g["genes2"], g["ranks2"])
    r = dto.optimize(l1, l2, False, g["population"], False)
    assert r.is_best() and (r.best.rank1, r.best.rank2) == (3, 4)
    assert abs(r.best.pvalue - g["expected"]["pvalue"]) <= 1e-12
    rp = dto.optimize(l1, l2, True, g["population"], False, seed=1)
    assert rp.is_best() and rp.best.permuted
    # process_threshold_pairs doctest: 3 x 3 grid -> 9 records, with feature sets
    a = rlist(["gene1", "gene2", "gene3"], [1, 2, 3])
    b = rlist(["gene1", "gene2", "gene4"], [1, 2, 3])
    recs = dto.process_threshold_pairs(a, b, True, 4, False, seed=2)
    assert len(recs) == 9 and all(x.pvalue >= 0.0 for x in recs)
    d = dto.optimize(a, b, False, 4, True)
    assert d.is_debug() and len(d.records) == 9
    last = d.records[-1]
    assert [x.id() for x in last.feature_sets.set1] == ["gene1", "gene2", "gene3"]


def test_hypergeometric_pvalue_goldens():
    for c in GOLDEN["hypergeometric"]:
        p = stat_operations.hypergeometric_pvalue(*c["args"])
        tol = c.get("abs_tol") or 1.3e-11 * c["p"]
        assert abs(p - c["p"]) <= tol
    with pytest.raises(stat_operations.HypergeometricError):
        stat_operations.hypergeometric_pvalue(5, 6, 1, 1)


def test_run_single_node_matches_engine():
    from dual_threshold_optimization_gb300 import synth
    p = synth.copula_pair(500, 0.3, seed=8)
    names = p.feature_names()
    l1 = col.RankedFeatureList.from_(col.FeatureList([names[f] for f in p.feat1]), p.ranks1)
    l2 = col.RankedFeatureList.from_(col.FeatureList([names[f] for f in p.feat2]), p.ranks2)
    res = run.run_single_node(run.make_tasks(20), l1, l2, 500, 4, seed=9)
    assert len(res) == 21 and not res[0].best.permuted
    eng = dto.default_engine()
    r1, f1, r2, f2, nf = col.dense_ids(l1, l2)
    dp = eng.pair(r1, f1, r2, f2, nf, 500)
    ref = dp.run(20, seed=9)
    assert [x.best.pvalue for x in res[1:]] == ref.minp.tolist()
    assert res[0].best.pvalue == ref.unpermuted["pvalue"]
    out = stat_operations.empirical_pvalue(res)
    assert out["empirical_pvalue"] == ref.summary["empirical_pvalue"]
    # one-process run_multi_node gives the same records
    mres = run.run_multi_node(run.make_tasks(20), l1, l2, 500, seed=9)
    assert [x.best.pvalue for x in mres] == [x.best.pvalue for x in res]


def test_run_range_splits_reproduce_one_run():
    from dual_threshold_optimization_gb300 import synth
    p = synth.copula_pair(2000, 0.2, seed=12)
    dp = dto.default_engine().pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    whole = dp.run(300, seed=5)
    a = dp.run(120, seed=5, first=1)
    b = dp.run(180, seed=5, first=121)
    assert np.array_equal(np.concatenate([a.minp, b.minp]), whole.minp)


@pytest.mark.parametrize("N", [12380, 12390, 16510, 16520, 24760, 24775, 26875, 26890, 32760, 32780, 49530, 49540, 53755, 53770])
def test_shared_memory_limits_at_list_lengths(engine, N):
    # list lengths around the permutation kernel's shared-memory switches
    # (label staging, kept words): the launches fit and agree with the spec
    from oracle import oracle as O
    from dual_threshold_optimization_gb300 import synth
    p = synth.copula_pair(N, 0.1, seed=91)
    dp = engine.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
    i1, _ = dp.export_permutations(5, 1, 1)
    assert np.array_equal(O.shuffle(5, 0, 1, 1, N), i1[0])
    r = dp.run(40, seed=5)
    assert np.all(np.isfinite(r.minp)) and r.unpermuted["pvalue"] <= 1.0
    dp.close()
