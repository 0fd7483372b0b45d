"""A process pool over the C oracle (test infrastructure only).

The GPU parity tests at benchmark sizes check a few hundred permutations of
lists of 6,000 to 60,000 features against the oracle's optimize
(src/dto/optimize_main.rs:53-118 over process_threshold_pairs.rs:71-131); one
task takes tens of milliseconds there, so the tasks are spread over the host
cores.  The pool is started with the ``spawn`` method: a process forked after
the parent has used the GPU can hang.
"""
import multiprocessing
import os

_PAIR = None


def _init(pair):
    global _PAIR
    _PAIR = pair
    from . import oracle as O
    O.lf_table(max(int(pair[5]), 1))


def _one(job):
    from . import oracle as O
    r1, f1, r2, f2, nfeat, population = _PAIR
    idx1, idx2 = job
    best, _ = O.optimize(r1, f1, r2, f2, nfeat, population, idx1, idx2)
    return best


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def optimize_many(sorted_pair, jobs, processes=None):
    """The oracle's optimum of each job.

    sorted_pair: (ranks1, feat1, ranks2, feat2, n_features, population) with the
    lists in stable rank order; jobs: (idx1, idx2) index arrays of the permuted
    views (src/collections/permuted.rs:34), or (None, None) for the unpermuted
    task.  Returns one record dict per job, in order.
    """
    jobs = list(jobs)
    if not jobs:
        return []
    n = max(1, min(len(jobs), processes or host_cores()))
    if n == 1:
        _init(sorted_pair)
        return [_one(j) for j in jobs]
    ctx = multiprocessing.get_context("spawn")
    with ctx.Pool(n, initializer=_init, initargs=(sorted_pair,)) as pool:
        return pool.map(_one, jobs, chunksize=max(1, len(jobs) // (4 * n)))
