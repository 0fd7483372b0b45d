"""Task drivers mirroring the reference's ``src/run``.

Task              src/run/task.rs:3-9
run_single_node   src/run/single_node.rs:83-137 -- the reference spreads tasks over
                  std::thread chunks; here all permuted tasks go to the GPU in one
                  dto_run call (the unpermuted task rides in the first batch).
run_multi_node    src/run/multi_node.rs:47-162 -- the reference scatters task chunks
                  over MPI ranks.  Here each process (one per GPU) takes a contiguous
                  range of permutation ids; permutation t is a function of
                  (seed, pair, t) only, so results do not depend on the sharding.
                  Rank 0 runs the unpermuted task and broadcasts its p-value; the
                  ranks' counts of permutations at or below it are summed, and the
                  minimum p-values (8 bytes a permutation) are gathered to rank 0
                  over a torch.distributed process group (gloo, host tensors).
                  Each rank can keep its progress in a checkpoint directory and
                  resume from it.
"""
import hashlib
import json
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


class Checkpoint:
    """Progress of one rank's share of a sharded null, kept on disk so that a
    restarted job resumes where the rank stopped (the reference's MPI run,
    src/run/multi_node.rs:47-162, has no resume).

    ``<dir>/rank<r>.json`` holds what identifies the run (seed, the pair's
    Philox stream, the shard, the pair's digest, the precision) and how many of
    the rank's ids are done; ``<dir>/rank<r>.minp.npy`` their minimum
    p-values (8 bytes each), ``rank<r>.records.npy`` the records when they are
    gathered.  A permutation is a function of (seed, stream, id) only, so the
    ids not yet done give the same results after a restart.  The state file is
    replaced atomically after each chunk.
    """

    def __init__(self, directory, rank, key, count, records):
        from numpy.lib.format import open_memmap
        from ._lib import RESULT_DTYPE
        os.makedirs(directory, exist_ok=True)
        self.path = os.path.join(directory, "rank%d.json" % rank)
        self.key = key
        state = None
        if os.path.exists(self.path):
            with open(self.path) as fh:
                state = json.load(fh)
            if state.get("key") != key:
                raise ValueError("checkpoint %s belongs to another run (%r, not %r)"
                                 % (self.path, state.get("key"), key))
        mp = os.path.join(directory, "rank%d.minp.npy" % rank)
        rp = os.path.join(directory, "rank%d.records.npy" % rank)
        fresh = state is None
        self.minp = open_memmap(mp, mode="w+" if fresh else "r+", dtype=np.float64, shape=(count,))
        self.records = None
        if records:
            self.records = open_memmap(rp, mode="w+" if fresh or not os.path.exists(rp) else "r+",
                                       dtype=RESULT_DTYPE, shape=(count,))
        self.done = 0 if fresh else int(state["done"])
        self.unpermuted = None if fresh else state.get("unpermuted")

    def save(self, done, unpermuted):
        self.minp.flush()
        if self.records is not None:
            self.records.flush()
        self.done = done
        self.unpermuted = unpermuted
        tmp = self.path + ".tmp"
        with open(tmp, "w") as fh:
            json.dump({"key": self.key, "done": done, "unpermuted": unpermuted}, fh)
        os.replace(tmp, self.path)


def _pair_digest(r1, f1, r2, f2, nf, population):
    h = hashlib.sha256()
    for a in (r1, f1, r2, f2):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(("%d,%d" % (nf, population)).encode())
    return h.hexdigest()[:24]


def run_multi_node(tasks, ranked_feature_list1, ranked_feature_list2, population_size,
                   num_threads=1, *, seed, precision="screen", group=None, engine=None,
                   compute=None, gather="minp", checkpoint=None, chunk=None, stream_id=0):
    """The permutation null sharded over torch.distributed ranks (one GPU
    each), replacing the MPI scatter/gather of src/run/multi_node.rs:47-162.

    Each rank takes a contiguous range of permutation ids (shard_range); a
    permutation is a function of (seed, stream, id), so the split does not
    change any result.  Rank 0 alone runs the unpermuted task.  The one
    exchange: rank 0 broadcasts the observed minimum p, every rank counts its
    permutations with p <= it, and the counts are summed (count_le, n_perm).
    ``gather`` adds, to rank 0: "minp" each permutation's minimum p-value
    (8 bytes a permutation; its records carry only the p-value), "records"
    every permuted task's full record, "count" nothing more.  ``seed`` must be
    the same on every rank.

    checkpoint: a directory; each rank keeps its progress there (Checkpoint)
    and a restarted job resumes each rank after its last finished chunk.
    chunk: permutations per chunk (default: the whole shard).

    ``compute(first, count, unpermuted, want_records)`` may replace the GPU
    call (tests use the CPU oracle); it returns (unpermuted record dict or
    None, minimum p-values [count], records structured array or None[, the
    run's dto_summary dict]).

    Returns, on rank 0, a RunResults list (the unpermuted result, then the
    permuted results when gathered) whose summary holds count_le, n_perm,
    empirical_pvalue and, with gather="minp", the minimum p-values in id
    order; the other ranks return an empty RunResults with their own counts.
    """
    import torch
    import torch.distributed as dist

    if gather not in ("minp", "records", "count"):
        raise ValueError("gather must be 'minp', 'records' or 'count'")
    dist_on = dist.is_available() and dist.is_initialized()
    rank = dist.get_rank(group) if dist_on else 0
    world = dist.get_world_size(group) if dist_on else 1
    n_perm = sum(1 for t in tasks if t.permute)
    first, count = shard_range(n_perm, rank, world)
    want_records = gather == "records"
    r1, f1, r2, f2, nf = dense_ids(ranked_feature_list1, ranked_feature_list2)
    if compute is None:
        eng = engine or default_engine(int(os.environ.get("LOCAL_RANK", "0")))
        dp = eng.pair(r1, f1, r2, f2, nf, population_size)
        dp.set_stream(stream_id)

        def compute(first, count, unpermuted, want_records):
            res = dp.run(count, seed=seed, precision=precision, want_records=want_records, first=first,
                         unpermuted=unpermuted)
            return res.unpermuted, res.minp, res.records, res.summary

    t0 = time.perf_counter()
    # this rank's share, chunk by chunk (resumed from the checkpoint if any)
    key = {"seed": int(seed), "stream": int(stream_id), "n_perm": n_perm, "world": world,
           "rank": rank, "first": first, "count": count, "precision": str(precision),
           "pair": _pair_digest(r1, f1, r2, f2, nf, population_size)}
    if checkpoint is not None:
        ck = Checkpoint(checkpoint, rank, key, count, want_records)
        minp, recs, done, unperm = ck.minp, ck.records, ck.done, ck.unpermuted
    else:
        from ._lib import RESULT_DTYPE
        ck = None
        minp = np.zeros(count, np.float64)
        recs = np.zeros(count, RESULT_DTYPE) if want_records else None
        done, unperm = 0, None
    step = count if not chunk else max(1, int(chunk))
    ran = 0
    bounds = {}
    while done < count or (rank == 0 and unperm is None):
        c = min(step, count - done)
        got = compute(first + done, c, rank == 0 and unperm is None, want_records)
        u, mp, rc = got[:3]
        if len(got) > 3 and got[3]:
            bounds = {"logp_err_bound_fp32": float(got[3]["logp_err_bound_screen"]),
                      "logp_err_bound_fp64": float(got[3]["logp_err_bound_fp64"])}
        if rank == 0 and unperm is None:
            unperm = {k: (v.item() if hasattr(v, "item") else v) for k, v in dict(u).items()}
        if c:
            minp[done:done + c] = mp
            if want_records:
                recs[done:done + c] = rc
        done += c
        ran += c
        if ck is not None:
            ck.save(done, unperm)
    seconds = time.perf_counter() - t0

    # the exchange: the observed p from rank 0, then the summed counts
    p_obs = torch.tensor([float(unperm["pvalue"]) if rank == 0 else 0.0], dtype=torch.float64)
    if world > 1:
        dist.broadcast(p_obs, src=dist.get_global_rank(group, 0) if group is not None else 0, group=group)
    local_le = int(np.count_nonzero(np.asarray(minp) <= float(p_obs.item())))
    tot = torch.tensor([local_le, count, ran], dtype=torch.int64)
    secs = torch.tensor([seconds], dtype=torch.float64)
    if world > 1:
        dist.all_reduce(tot, group=group)
        dist.all_reduce(secs, op=dist.ReduceOp.MAX, group=group)
    count_le, total, total_ran = (int(v) for v in tot.tolist())
    summary = {"count_le": count_le, "n_perm": total,
               "empirical_pvalue": (count_le / total) if total else 1.0,
               "perms_per_s": (total_ran / float(secs.item())) if secs.item() > 0 else None,
               "world": world, "shard": [first, count], "resumed_from": done - ran}
    summary.update(bounds)

    gathered_minp = gathered = sizes = None
    if gather != "count":
        local = np.asarray(minp, np.float64)[:, None]
        if want_records:
            fields = ("rank1", "rank2", "set1_len", "set2_len", "population_size", "intersection_size")
            local = np.zeros((count, len(fields) + 1), np.float64)
            for q, f in enumerate(fields):
                local[:, q] = np.asarray(recs)[f]
            local[:, -1] = minp
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        if world > 1:
            dist.all_gather(sizes, torch.tensor([count], dtype=torch.int64), group=group)
        else:
            sizes = [torch.tensor([count])]
        maxc = max(int(x.item()) for x in sizes)
        buf = torch.zeros((maxc, local.shape[1]), dtype=torch.float64)
        buf[:count] = torch.from_numpy(np.ascontiguousarray(local))
        if world > 1:
            gathered = [torch.zeros_like(buf) for _ in range(world)]
            dist.all_gather(gathered, buf, group=group)
        else:
            gathered = [buf]
    if rank != 0:
        return RunResults([], summary)
    out = [OptimizationResult.Best(OptimizationResultRecord.from_abi(dict(unperm, permuted=False)))]
    if gathered is not None:
        rows = [g[:int(sizes[r].item())].numpy() for r, g in enumerate(gathered)]
        allrows = np.concatenate(rows, axis=0) if rows else np.zeros((0, 1))
        if want_records:
            fields = ("rank1", "rank2", "set1_len", "set2_len", "population_size", "intersection_size")
            for row in allrows:
                d = {f: int(row[q]) for q, f in enumerate(fields)}
                d["pvalue"] = float(row[-1])
                d["permuted"] = True
                out.append(OptimizationResult.Best(OptimizationResultRecord.from_abi(d)))
        else:
            gathered_minp = allrows[:, 0].copy()
            summary["minp"] = gathered_minp
            out.extend(OptimizationResult.Best(OptimizationResultRecord.pvalue_only(p))
                       for p in gathered_minp)
    return RunResults(out, summary)
