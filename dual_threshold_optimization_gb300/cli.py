"""Command line, mirroring the reference binary (src/main.rs:20-166).

    python -m dual_threshold_optimization_gb300 -1 list1.csv -2 list2.csv \
        [-b background.txt] [-p 1000] [-t 1] [-m] [--seed S] [--precision screen|fp64]

Progress goes to stderr and the result to stdout as pretty JSON with sorted keys
(the reference prints a serde_json map, whose keys are ordered).  Errors that
make the reference panic print the same message to stderr and exit with 101
(Rust's panic exit code).  -m runs the permutations sharded over the ranks of
a torch.distributed job (one GPU per rank); rank 0 prints the result.
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
    ap.add_argument("-p", "--permutations", type=int, default=1000)
    ap.add_argument("-t", "--threads", type=int, default=1)
    ap.add_argument("-m", "--multi-node", dest="multi_node", action="store_true")
    ap.add_argument("--seed", type=int, default=None,
                    help="Philox seed of the permutations (random when omitted)")
    ap.add_argument("--precision", default="screen", choices=["screen", "fp64"])
    ap.add_argument("--device", type=int, default=None)
    return ap


def main(argv=None):
    args = build_parser().parse_args(argv)
    from .dto import PopulationError, compute_population_size, default_engine
    from .read import ReadError, read_feature_list_from_file, read_ranked_feature_list_from_csv
    from .run import make_tasks, run_multi_node, run_single_node
    from .stat_operations import empirical_pvalue

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
    results = run_single_node(tasks, l1, l2, pop, threads, seed=args.seed, precision=args.precision,
                              engine=eng)
    print(json.dumps(empirical_pvalue(results), indent=2, sort_keys=True))
    return 0


if __name__ == "__main__":
    sys.exit(main())
