"""Host-side logic of the reference-shaped API (no GPU)."""
import json
import os

import numpy as np
import pytest

from dual_threshold_optimization_gb300 import feature_lists as col
from dual_threshold_optimization_gb300 import dto, read, run, stat_operations

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))


def rlist(genes, ranks):
    return col.RankedFeatureList.from_(col.FeatureList(genes), ranks)


def test_ranked_list_stable_sort_and_thresholds():
    l = rlist(["a", "b", "c", "d"], [3, 1, 3, 2])
    assert l.ranks().tolist() == [1, 2, 3, 3]
    assert l.genes().ids() == ["b", "d", "a", "c"]  # stable: a before c
    assert l.thresholds().tolist() == [1, 2, 3]
    assert [g.id() for g in l.get_feature_set_by_threshold(2)] == ["b", "d"]
    with pytest.raises(ValueError):
        rlist(["a"], [1, 2])


def test_permuted_view():
    l = rlist(["g1", "g2", "g3"], [1, 2, 3])
    v = col.PermutedRankedFeatureList(l, indices=[2, 0, 1])
    assert [g.id() for g in v.get_feature_set_by_threshold(2)] == ["g3", "g1"]
    with pytest.raises(ValueError):
        col.PermutedRankedFeatureList(l, indices=[0, 0, 1])


@pytest.mark.parametrize("case", GOLDEN["population"], ids=lambda c: c["cite"])
def test_compute_population_size_goldens(case):
    l1 = rlist(case["l1"], list(range(1, len(case["l1"]) + 1)))
    l2 = rlist(case["l2"], list(range(1, len(case["l2"]) + 1)))
    bg = col.FeatureList(case["bg"]) if case["bg"] is not None else None
    if "error" in case:
        with pytest.raises(dto.PopulationError) as e:
            dto.compute_population_size(l1, l2, bg)
        assert str(e.value).startswith(case["error"])
    else:
        assert dto.compute_population_size(l1, l2, bg) == case["value"]


def test_empirical_and_fdr_goldens():
    e = GOLDEN["empirical"]
    u = dict(e["unpermuted"], permuted=False)
    recs = [u] + [dict(u, pvalue=p, permuted=True, intersection_size=8) for p in e["permuted_pvalues"]]
    out = stat_operations.empirical_pvalue(recs)
    assert out == e["expected"]
    only = stat_operations.empirical_pvalue([u])
    assert only["empirical_pvalue"] == 1.0
    for c in GOLDEN["fdr"]:
        assert abs(stat_operations.fdr(*c["args"]) - c["value"]) <= c["abs_tol"]
    with pytest.raises(ValueError):
        stat_operations.fdr(1, 1, 1, 1, 0.0)
    with pytest.raises(ValueError):
        stat_operations.empirical_pvalue([dict(u, permuted=True)])


def test_intersect_genes():
    a = [col.Feature(x) for x in ("gene1", "gene2", "gene3")]
    b = [col.Feature(x) for x in ("gene2", "gene3", "gene4")]
    assert stat_operations.intersect_genes(a, b) == 2


def test_readers(tmp_path):
    p = tmp_path / "l.csv"
    p.write_text("gene1,3\ngene2, 1\ngene3,2\n")
    l = read.read_ranked_feature_list_from_csv(str(p))
    assert l.genes().ids() == ["gene2", "gene3", "gene1"]
    bad = tmp_path / "bad.csv"
    bad.write_text("gene1,1,2\n")
    with pytest.raises(read.ReadError, match="Invalid format"):
        read.read_ranked_feature_list_from_csv(str(bad))
    bad.write_text("gene1,x\n")
    with pytest.raises(read.ReadError, match="Invalid rank value"):
        read.read_ranked_feature_list_from_csv(str(bad))
    with pytest.raises(read.ReadError, match="Could not open file"):
        read.read_ranked_feature_list_from_csv(str(tmp_path / "missing.csv"))
    b = tmp_path / "bg.txt"
    b.write_text("gene1\n gene2 \ngene3\n")
    assert read.read_feature_list_from_file(str(b)).ids() == ["gene1", "gene2", "gene3"]


def test_tasks_and_shards():
    t = run.make_tasks(5)
    assert [(x.id, x.permute) for x in t] == [(0, False)] + [(i, True) for i in range(1, 6)]
    for n, w in [(10, 3), (100000, 8), (3, 4), (0, 2)]:
        got = []
        for r in range(w):
            first, count = run.shard_range(n, r, w)
            got.extend(range(first, first + count))
        assert got == list(range(1, n + 1))


def test_cli_parser():
    from dual_threshold_optimization_gb300.cli import build_parser
    a = build_parser().parse_args(["-1", "a.csv", "-2", "b.csv", "-p", "5", "-t", "0", "-m"])
    assert (a.ranked_list1, a.ranked_list2, a.permutations, a.threads, a.multi_node) == \
        ("a.csv", "b.csv", 5, 0, True)
    assert build_parser().parse_args(["-1", "x", "-2", "y"]).permutations == 1000


def test_cli_reports_population_error(tmp_path, capsys):
    from dual_threshold_optimization_gb300.cli import main
    (tmp_path / "a.csv").write_text("g1,1\ng2,2\n")
    (tmp_path / "b.csv").write_text("g1,1\ng3,2\n")
    rc = main(["-1", str(tmp_path / "a.csv"), "-2", str(tmp_path / "b.csv"), "-p", "0"])
    assert rc == 101
    assert "identical genes" in capsys.readouterr().err


def test_synthetic_configs():
    from dual_threshold_optimization_gb300 import synth
    p1 = synth.config1()
    assert len(p1.ranks1) == 6000 and sorted(p1.ranks1.tolist()) == list(range(1, 6001))
    tied = len(p1.ranks2) - len(set(p1.ranks2.tolist()))
    assert 300 < tied < 900  # ~10% of features in tie blocks of size 2-5
    p4 = synth.config4()
    assert len(p4.ranks1) == 18000 and p4.population == 18000 and p4.ranks1.max() > 18000
