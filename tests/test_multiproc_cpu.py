"""run_multi_node's sharding and gather over two gloo ranks on the CPU.

Each rank evaluates its permutation-id range with the CPU oracle standing in
for the GPU (compute=...), so the host logic -- the split of ids, the gather to
rank 0, the empirical p-value there -- is tested without a GPU.  A rank that
fails is made on the host (an exception before the gather)."""
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


def _oracle_compute(p, seed):
    from oracle import oracle as O
    from dual_threshold_optimization_gb300._lib import RESULT_DTYPE
    (r1, f1), (r2, f2) = p.sorted_lists()

    def compute(first, count):
        unp, _ = O.optimize(r1, f1, r2, f2, p.n_features, p.population)
        recs = np.zeros(count, RESULT_DTYPE)
        for q in range(count):
            i1 = O.shuffle(seed, 0, first + q, 1, len(r1))
            b, _ = O.optimize(r1, f1, r2, f2, p.n_features, p.population, i1, None)
            for k in ("rank1", "rank2", "set1_len", "set2_len", "intersection_size", "pvalue"):
                recs[q][k] = b[k]
            recs[q]["population_size"] = p.population
        unp["population_size"] = p.population
        return unp, recs
    return compute


def _worker(rank, world, port, n_perm, seed, q, fail_rank):
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
                                 compute=_oracle_compute(p, seed))
        if rank == 0:
            q.put(("ok", [r.best.pvalue for r in res], stat_operations.empirical_pvalue(res)))
        else:
            q.put(("ok", res, None))
    except Exception as e:  # reported to the parent
        q.put(("err", "%s" % e, rank))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _launch(world, n_perm, seed, fail_rank=-1):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_perm, seed, q, fail_rank))
             for r in range(world)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for pr in procs:
        pr.join(timeout=60)
    return out


def test_two_ranks_match_single_process():
    seed, n_perm = 77, 7
    out = _launch(2, n_perm, seed)
    zero = [o for o in out if o[0] == "ok" and o[2] is not None]
    assert len(zero) == 1
    pv = zero[0][1]
    assert len(pv) == n_perm + 1
    # same values as one process evaluating every id
    from oracle import oracle as O
    p = _pair()
    (r1, f1), (r2, f2) = p.sorted_lists()
    want = [O.optimize(r1, f1, r2, f2, p.n_features, p.population)[0]["pvalue"]]
    for t in range(1, n_perm + 1):
        want.append(O.optimize(r1, f1, r2, f2, p.n_features, p.population,
                               O.shuffle(seed, 0, t, 1, len(r1)), None)[0]["pvalue"])
    assert pv == want
    others = [o for o in out if o[0] == "ok" and o[2] is None]
    assert others and others[0][1] == []


def test_failed_rank_is_reported_not_hung():
    out = _launch(2, 4, 5, fail_rank=1)
    errs = [o for o in out if o[0] == "err"]
    assert errs, out  # rank 1 raised; rank 0's gather ended with an error
