"""run_multi_node's sharding, exchange and resume over two gloo ranks on the CPU.

Each rank evaluates its permutation-id range with the CPU oracle standing in
for the GPU (compute=...), so the host logic -- the split of ids, the observed
p broadcast from rank 0, the summed counts, the gather of minimum p-values or
records to rank 0, the checkpoint and resume -- is tested without a GPU.
Failures are made on the host: a rank that raises before the exchange, and
ranks interrupted after their first chunk."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _pair():
    from dual_threshold_optimization_gb300 import synth
    return synth.copula_pair(50, 0.4, seed=3)


def _oracle_compute(p, seed, fail_after=None):
    from oracle import oracle as O
    from dual_threshold_optimization_gb300._lib import RESULT_DTYPE
    (r1, f1), (r2, f2) = p.sorted_lists()
    calls = [0]

    def compute(first, count, unpermuted, want_records):
        if fail_after is not None and calls[0] >= fail_after:
            raise RuntimeError("interrupted after %d chunks" % calls[0])
        calls[0] += 1
        unp = None
        if unpermuted:
            unp, _ = O.optimize(r1, f1, r2, f2, p.n_features, p.population)
            unp["population_size"] = p.population
        recs = np.zeros(count, RESULT_DTYPE)
        for q in range(count):
            i1 = O.shuffle(seed, 0, first + q, 1, len(r1))
            b, _ = O.optimize(r1, f1, r2, f2, p.n_features, p.population, i1, None)
            for k in ("rank1", "rank2", "set1_len", "set2_len", "intersection_size", "pvalue"):
                recs[q][k] = b[k]
            recs[q]["population_size"] = p.population
        return unp, recs["pvalue"].copy(), (recs if want_records else None)
    return compute


def _worker(rank, world, port, n_perm, seed, q, fail_rank, opts=None):
    opts = opts or {}
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from datetime import timedelta
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=20))
    try:
        from dual_threshold_optimization_gb300 import feature_lists as col, run, stat_operations
        p = _pair()
        names = p.feature_names()
        l1 = col.RankedFeatureList.from_(col.FeatureList([names[f] for f in p.feat1]), p.ranks1)
        l2 = col.RankedFeatureList.from_(col.FeatureList([names[f] for f in p.feat2]), p.ranks2)
        if rank == fail_rank:
            raise RuntimeError("rank %d fails before the gather" % rank)
        res = run.run_multi_node(run.make_tasks(n_perm), l1, l2, p.population, seed=seed,
                                 compute=_oracle_compute(p, seed, opts.get("fail_after")),
                                 gather=opts.get("gather", "minp"), checkpoint=opts.get("checkpoint"),
                                 chunk=opts.get("chunk"))
        summ = {k: v for k, v in res.summary.items() if k != "minp"}
        if rank == 0:
            q.put(("ok", [r.best.pvalue for r in res], stat_operations.empirical_pvalue(res), summ, rank))
        else:
            q.put(("ok", list(res), None, summ, rank))
    except Exception as e:  # reported to the parent
        q.put(("err", "%s" % e, rank))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _launch(world, n_perm, seed, fail_rank=-1, opts=None):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_perm, seed, q, fail_rank, opts))
             for r in range(world)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for pr in procs:
        pr.join(timeout=60)
    return out


def _single_process(n_perm, seed):
    from oracle import oracle as O
    p = _pair()
    (r1, f1), (r2, f2) = p.sorted_lists()
    want = [O.optimize(r1, f1, r2, f2, p.n_features, p.population)[0]["pvalue"]]
    for t in range(1, n_perm + 1):
        want.append(O.optimize(r1, f1, r2, f2, p.n_features, p.population,
                               O.shuffle(seed, 0, t, 1, len(r1)), None)[0]["pvalue"])
    return want


@pytest.mark.parametrize("gather", ["minp", "records", "count"])
def test_two_ranks_match_single_process(gather):
    seed, n_perm = 77, 7
    out = _launch(2, n_perm, seed, opts={"gather": gather})
    zero = [o for o in out if o[0] == "ok" and o[4] == 0]
    assert len(zero) == 1, out
    pv, emp, summ = zero[0][1], zero[0][2], zero[0][3]
    want = _single_process(n_perm, seed)
    # same values as one process evaluating every id
    if gather == "count":
        assert pv == want[:1]
    else:
        assert pv == want
    assert summ["n_perm"] == n_perm
    assert summ["count_le"] == sum(1 for x in want[1:] if x <= want[0])
    assert emp["empirical_pvalue"] == summ["count_le"] / n_perm
    others = [o for o in out if o[0] == "ok" and o[4] == 1]
    assert others and others[0][1] == [] and others[0][3]["count_le"] == summ["count_le"]


def test_failed_rank_is_reported_not_hung():
    out = _launch(2, 4, 5, fail_rank=1)
    errs = [o for o in out if o[0] == "err"]
    assert errs, out  # rank 1 raised; rank 0's gather ended with an error


def test_resume_after_interruption(tmp_path):
    # both ranks stop after their first chunk (a host failure, before any
    # exchange); the relaunched job resumes each rank after its saved chunk
    # and ends with the single-process results
    seed, n_perm = 31, 9
    ck = str(tmp_path / "ck")
    out = _launch(2, n_perm, seed, opts={"checkpoint": ck, "chunk": 2, "fail_after": 1})
    assert all(o[0] == "err" and "interrupted" in o[1] for o in out), out
    out = _launch(2, n_perm, seed, opts={"checkpoint": ck, "chunk": 2})
    assert all(o[0] == "ok" for o in out), out
    byrank = {o[4]: o for o in out}
    assert byrank[0][3]["resumed_from"] == 2 and byrank[1][3]["resumed_from"] == 2
    want = _single_process(n_perm, seed)
    assert byrank[0][1] == want
    assert byrank[0][3]["count_le"] == sum(1 for x in want[1:] if x <= want[0])
    # a checkpoint of another run is refused, not reused
    out = _launch(2, n_perm, seed + 1, opts={"checkpoint": ck, "chunk": 2})
    assert all(o[0] == "err" and "another run" in o[1] for o in out), out
