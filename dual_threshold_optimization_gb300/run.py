"""Task drivers mirroring the reference's ``src/run``.

Task              src/run/task.rs:3-9
run_single_node   src/run/single_node.rs:83-137 -- the reference spreads tasks over
                  std::thread chunks; here all permuted tasks go to the GPU in one
                  dto_run call (the unpermuted task rides in the first batch).
run_multi_node    src/run/multi_node.rs:47-162 -- the reference scatters task chunks
                  over MPI ranks.  Here each process (one per GPU) takes a contiguous
                  range of permutation ids; permutation t is a function of
                  (seed, pair, t) only, so results do not depend on the sharding.
                  Rank 0 gathers the per-permutation minimum p-values over a
                  torch.distributed process group (gloo, host tensors) and returns
                  every result; the other ranks return [].
"""
import os
import time

import numpy as np

from .feature_lists import dense_ids
from .dto import OptimizationResult, OptimizationResultRecord, default_engine


class Task:
    """task.rs:3-9."""

    __slots__ = ("id", "permute")

    def __init__(self, id, permute):  # noqa: A002 - mirrors the reference's field name
        self.id = int(id)
        self.permute = bool(permute)

    def __repr__(self):
        return "Task(id=%d, permute=%s)" % (self.id, self.permute)


def make_tasks(permutations):
    """main.rs:122-126: task 0 unpermuted, tasks 1..=P permuted."""
    return [Task(0, False)] + [Task(i, True) for i in range(1, permutations + 1)]


class RunResults(list):
    """The per-task OptimizationResults of a run, in task order (what the
    reference's run_single_node returns), plus ``summary``: the run's error
    bounds and throughput, which empirical_pvalue adds to its output
    (logp_err_bound_fp32, logp_err_bound_fp64, perms_per_s)."""

    def __init__(self, items=(), summary=None):
        super().__init__(items)
        self.summary = summary or {}


def run_summary(summary, n_perm, seconds):
    """The extra output keys of a run from its dto_summary."""
    return {"logp_err_bound_fp32": float(summary["logp_err_bound_screen"]),
            "logp_err_bound_fp64": float(summary["logp_err_bound_fp64"]),
            "perms_per_s": (n_perm / seconds) if seconds > 0 else None,
            "n_perm": int(n_perm), "seconds": float(seconds)}


def _records_to_results(recs, permuted):
    out = []
    for r in recs:
        d = {k: r[k] for k in r.dtype.names}
        d["permuted"] = permuted
        out.append(OptimizationResult.Best(OptimizationResultRecord.from_abi(d)))
    return out


def _seed_or_random(seed):
    if seed is None:
        return int.from_bytes(os.urandom(8), "little")
    return int(seed)


def run_single_node(tasks, ranked_feature_list1, ranked_feature_list2, population_size,
                    num_threads=1, *, seed=None, precision="screen", engine=None, perm_indices=None):
    """Run every task; returns one OptimizationResult per task, in task order
    (a RunResults list carrying the run's summary).

    num_threads is accepted for the reference's signature; the GPU path ignores
    it (the reference treats 0 as 1, main.rs:73-76).  Permuted task t uses
    permutation id t of the Philox stream ``seed``, or, in test mode, row t - 1
    of ``perm_indices`` ([P][N1 + N2]: the permuted views' index arrays of
    both lists, src/collections/permuted.rs:34).
    """
    eng = engine or default_engine()
    r1, f1, r2, f2, nf = dense_ids(ranked_feature_list1, ranked_feature_list2)
    dp = eng.pair(r1, f1, r2, f2, nf, population_size)
    seed = _seed_or_random(seed)
    perm_ids = sorted(t.id for t in tasks if t.permute)
    out = {}
    t0 = time.perf_counter()
    if perm_ids:
        lo, hi = perm_ids[0], perm_ids[-1]
        if lo < 1:
            raise ValueError("permuted task ids must be >= 1")
        idx = None
        if perm_indices is not None:
            idx = np.ascontiguousarray(perm_indices, np.int32)
            if idx.ndim != 2 or idx.shape[0] < hi or idx.shape[1] != dp.N1 + dp.N2:
                raise ValueError("perm_indices must have shape (P, N1 + N2) with P >= %d rows of %d"
                                 % (hi, dp.N1 + dp.N2))
            idx = idx[:hi]
        res = dp.run(hi, seed=seed, perm_idx=idx, precision=precision, want_records=True)
        unperm = res.unpermuted
        for t in tasks:
            if t.permute:
                d = {k: res.records[t.id - 1][k] for k in res.records.dtype.names}
                d["permuted"] = True
                out[t.id] = OptimizationResult.Best(OptimizationResultRecord.from_abi(d))
    else:
        res = dp.run(0, precision=precision)
        unperm = res.unpermuted
    seconds = time.perf_counter() - t0
    for t in tasks:
        if not t.permute:
            d = dict(unperm)
            d["permuted"] = False
            out[t.id] = OptimizationResult.Best(OptimizationResultRecord.from_abi(d))
    dp.close()
    return RunResults([out[t.id] for t in tasks], run_summary(res.summary, len(perm_ids), seconds))


def shard_range(n_perm, rank, world):
    """Contiguous permutation ids [first, last] (1-based) of one rank."""
    base, extra = divmod(n_perm, world)
    first = rank * base + min(rank, extra) + 1
    count = base + (1 if rank < extra else 0)
    return first, count


def run_multi_node(tasks, ranked_feature_list1, ranked_feature_list2, population_size,
                   num_threads=1, *, seed, precision="screen", group=None, engine=None,
                   compute=None):
    """Sharded replicas over torch.distributed ranks (one GPU each).

    ``seed`` must be the same on every rank.  ``compute(first, count)`` may
    replace the GPU call (tests use the CPU oracle); it returns
    (unpermuted_record_dict_or_None, records structured array).
    """
    import torch
    import torch.distributed as dist

    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    n_perm = sum(1 for t in tasks if t.permute)
    first, count = shard_range(n_perm, rank, world)
    if compute is None:
        eng = engine or default_engine(int(os.environ.get("LOCAL_RANK", "0")))
        r1, f1, r2, f2, nf = dense_ids(ranked_feature_list1, ranked_feature_list2)
        dp = eng.pair(r1, f1, r2, f2, nf, population_size)

        def compute(first, count):
            res = dp.run(count, seed=seed, precision=precision, want_records=True, first=first)
            return res.unpermuted, res.records

    unperm, recs = compute(first, count)
    fields = ("rank1", "rank2", "set1_len", "set2_len", "population_size", "intersection_size")
    local = np.zeros((count, len(fields) + 1), np.float64)
    if count:
        for q, f in enumerate(fields):
            local[:, q] = recs[f]
        local[:, -1] = recs["pvalue"]
    # gather on the host (gloo): sizes first, then the padded rows
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    if world > 1:
        dist.all_gather(sizes, torch.tensor([count], dtype=torch.int64), group=group)
    else:
        sizes = [torch.tensor([count])]
    maxc = max(int(s.item()) for s in sizes)
    buf = torch.zeros((maxc, local.shape[1]), dtype=torch.float64)
    buf[:count] = torch.from_numpy(local)
    if world > 1:
        gathered = [torch.zeros_like(buf) for _ in range(world)]
        dist.all_gather(gathered, buf, group=group)
    else:
        gathered = [buf]
    if rank != 0:
        return []
    results = [OptimizationResult.Best(OptimizationResultRecord.from_abi(dict(unperm, permuted=False)))]
    for r, g in enumerate(gathered):
        c = int(sizes[r].item())
        for row in g[:c].numpy():
            d = {f: int(row[q]) for q, f in enumerate(fields)}
            d["pvalue"] = float(row[-1])
            d["permuted"] = True
            results.append(OptimizationResult.Best(OptimizationResultRecord.from_abi(d)))
    return results
