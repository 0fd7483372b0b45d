"""Command line, mirroring the reference binary (src/main.rs:20-166).

    python -m dual_threshold_optimization_gb300 -1 list1.csv -2 list2.csv \
        [-b background.txt] [-p 1000] [-t 1] [-m] [--seed S] [--precision screen|fp64] \
        [--perm-indices FILE]

Progress goes to stderr and the result to stdout as pretty JSON with sorted keys
(the reference prints a serde_json map, whose keys are ordered).  The
reference's nine keys (src/stat_operations/empirical_pvalue.rs:176-186) come
with three more: logp_err_bound_fp32, logp_err_bound_fp64 and perms_per_s.
Errors that make the reference panic print the same message to stderr and exit
with 101 (Rust's panic exit code).  -m runs the permutations sharded over the
ranks of a torch.distributed job (one GPU per rank); rank 0 prints the result.

--perm-indices FILE is the test mode: instead of on-device Philox permutations,
permutation t uses row t - 1 of FILE, the permuted views' index arrays of both
lists (src/collections/permuted.rs:34: positions in each list's stable rank
order, list 1's N1 entries then list 2's N2), one row per permutation, as a
.npy array of shape (P, N1 + N2) or as text with one row per line.  P is the
number of rows.
"""
import argparse
import json
import os
import sys


def build_parser():
    ap = argparse.ArgumentParser(prog="dual_threshold_optimization",
                                 description="Dual Threshold Optimization (GB300)")
    ap.add_argument("-1", "--ranked-list1", dest="ranked_list1", required=True, metavar="FILE")
    ap.add_argument("-2", "--ranked-list2", dest="ranked_list2", required=True, metavar="FILE")
    ap.add_argument("-b", "--background", default=None, metavar="FILE")
    ap.add_argument("-p", "--permutations", type=int, default=1000,
                    help="permutations (with --perm-indices: the rows of FILE)")
    ap.add_argument("-t", "--threads", type=int, default=1)
    ap.add_argument("-m", "--multi-node", dest="multi_node", action="store_true")
    ap.add_argument("--seed", type=int, default=None,
                    help="Philox seed of the permutations (random when omitted)")
    ap.add_argument("--precision", default="screen", choices=["screen", "fp64"])
    ap.add_argument("--device", type=int, default=None)
    ap.add_argument("--perm-indices", dest="perm_indices", default=None, metavar="FILE",
                    help="test mode: the permutations' index arrays, one row per permutation")
    return ap


def read_perm_indices(path):
    """The test-mode index arrays: a .npy array or text rows (comma or space
    separated) of int32, shape (P, N1 + N2)."""
    import numpy as np
    if path.endswith(".npy"):
        a = np.load(path)
    else:
        with open(path) as fh:
            text = fh.read().replace(",", " ")
        rows = [r.split() for r in text.splitlines() if r.strip()]
        a = np.array(rows, dtype=np.int64)
    a = np.asarray(a)
    if a.ndim == 1:
        a = a[None, :]
    if a.ndim != 2:
        raise ValueError("perm indices: expected one row per permutation")
    return np.ascontiguousarray(a, np.int32)


def _gave_permutations(argv):
    return any(a in ("-p", "--permutations") or a.startswith("--permutations=")
               or (a.startswith("-p") and len(a) > 2) for a in argv)


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    args = build_parser().parse_args(argv)
    from ._lib import DtoError
    from .dto import PopulationError, compute_population_size, default_engine
    from .read import ReadError, read_feature_list_from_file, read_ranked_feature_list_from_csv
    from .run import make_tasks, run_multi_node, run_single_node
    from .stat_operations import empirical_pvalue

    perm_idx = None
    if args.perm_indices:
        try:
            perm_idx = read_perm_indices(args.perm_indices)
        except (OSError, ValueError) as e:
            print("Failed to read permutation indices from %s: %s" % (args.perm_indices, e),
                  file=sys.stderr)
            return 101
        if _gave_permutations(argv) and args.permutations != perm_idx.shape[0]:
            print("--permutations %d does not match the %d rows of %s"
                  % (args.permutations, perm_idx.shape[0], args.perm_indices), file=sys.stderr)
            return 101
        args.permutations = perm_idx.shape[0]
    threads = args.threads
    if threads == 0:
        print("Warning: Number of threads cannot be 0. Setting threads to 1.", file=sys.stderr)
        threads = 1
    err = sys.stderr
    print("Ranked list 1: %s" % args.ranked_list1, file=err)
    print("Ranked list 2: %s" % args.ranked_list2, file=err)
    print("Permutations: %d" % args.permutations, file=err)
    print("Threads: %d" % threads, file=err)
    print("Multi-node mode: %s" % ("enabled" if args.multi_node else "disabled"), file=err)
    try:
        l1 = read_ranked_feature_list_from_csv(args.ranked_list1)
        l2 = read_ranked_feature_list_from_csv(args.ranked_list2)
        print("The product of the lengths of the threshold lists (this describes the asymptotic "
              "runtime of a single job): %d" % (len(l1.thresholds()) * len(l2.thresholds())), file=err)
        bg = read_feature_list_from_file(args.background) if args.background else None
        pop = compute_population_size(l1, l2, bg)
    except (ReadError, PopulationError, ValueError) as e:
        print(str(e), file=err)
        return 101
    tasks = make_tasks(args.permutations)
    eng = default_engine(args.device)
    if perm_idx is not None and perm_idx.shape[1] != len(l1) + len(l2):
        print("perm indices: rows have %d entries, the lists %d + %d"
              % (perm_idx.shape[1], len(l1), len(l2)), file=err)
        return 101
    if args.multi_node and perm_idx is not None:
        print("--perm-indices is not supported with -m", file=err)
        return 101
    if args.multi_node:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        seed = args.seed if args.seed is not None else 0
        results = run_multi_node(tasks, l1, l2, pop, threads, seed=seed, precision=args.precision)
        if results:
            print(json.dumps(empirical_pvalue(results), indent=2, sort_keys=True))
        dist.destroy_process_group()
        return 0
    try:
        results = run_single_node(tasks, l1, l2, pop, threads, seed=args.seed,
                                  precision=args.precision, engine=eng, perm_indices=perm_idx)
    except (ValueError, DtoError) as e:
        print(str(e), file=err)
        return 101
    print(json.dumps(empirical_pvalue(results), indent=2, sort_keys=True))
    return 0


if __name__ == "__main__":
    sys.exit(main())
