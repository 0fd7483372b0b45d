"""Benchmark: permutations per second of the DTO permutation null on one GB300.

Workload: one list pair of N = 20,000 features, list 2 from a Gaussian copula
with rho = 0.2 to list 1, no ties; 100,000 on-device Philox permutations per
step (plus the unpermuted task); the FP32-screen + FP64-refine path.  Inputs
are seeded synthetic lists (the reference's own profiling inputs are not
shipped).

Printed JSON line (one, from rank 0):
  value       perms/s over K timed steps, pair resident on the device, CUDA
              events on the library's stream around the K steps.
  e2e         the same metric through the C ABI with host buffers: every step
              creates the pair from host arrays (host-to-device copy of the
              pair tables) and returns the per-permutation minimum p-values to
              host memory.
  roofline    the grid kernel (the threshold-pair search): algorithmic work =
              8 FP32-class operations per grid cell per permutation (the
              nine-term log-pmf sum of the screen), over its CUDA-event time,
              against the measured FP32 peak (cuBLAS SGEMM on this GPU).
  cpu_baseline the reference algorithm restated in C (string hash-set
              intersection per cell, FP64 tail per cell, tasks over threads),
              timed on a row sample of one task per host thread.
  fp64_gpu    the plain FP64 GPU path (every cell's FP64 tail) on a sample.

--impl reference times the reference-algorithm CPU restatement alone, with all
host threads, on the same workload and metric.
"""
import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "perms/s on 1 GB300 at N=20k (FP32-screen vs plain FP64, same argmin); p50/p99 lat"
N_FEATURES = 20000
RHO = 0.2
PERMS_PER_STEP = 100000
# DRAM bytes per permutation of the table sweep at N = 20,000, from an ncu
# capture of one launch (dram__bytes_read.sum + dram__bytes_write.sum over its
# permutations, levels 1 and 2 of the ones that cascade included): labels read
# once (again by a cascading task), hit buffer written and re-read.
SWEEP0_DRAM_BYTES_PER_TASK = 49400.0
WORKLOAD = ("single pair, N=20000 features, list 2 Gaussian copula rho=0.2 to list 1, no ties, "
            "100000 on-device Philox permutations per step + the unpermuted task, "
            "FP32 screen + FP64 refine")


def single_config(P):
    """The config object of the headline workload, the same for both arms."""
    import math
    from dual_threshold_optimization_gb300 import synth

    def n_thresholds(max_rank):  # T = 1, T <- floor(1.01 T + 1) while T <= max rank
        n, t = 0, 1
        while t <= max_rank:
            n, t = n + 1, int(math.floor(t * 1.01 + 1.0))
        return n
    pair = synth.copula_pair(N_FEATURES, RHO, seed=2)
    grid = [n_thresholds(int(pair.ranks1.max())), n_thresholds(int(pair.ranks2.max()))]
    return {"workload": WORKLOAD, "n_features": N_FEATURES, "rho": RHO, "permutations": P,
            "grid": grid, "pair_seed": 2,
            "l2": "inputs larger than L2: each step streams %d MB of permutation labels"
                  % (P * N_FEATURES * 2 // 1000000)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi every 50 ms from start() to stop(); when the timed region is
    marked (begin() / end()), only the samples whose timestamps fall inside it
    count (all samples if none parse)."""
    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, device_index):
        self.device_index = device_index
        self.proc = None
        self.lines = []
        self.t_begin = self.t_end = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def begin(self):
        self.t_begin = datetime.datetime.now()

    def end(self):
        self.t_end = datetime.datetime.now()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    @classmethod
    def summarize(cls, lines, t_begin=None, t_end=None):
        rows = []
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm, smax = float(parts[2]), float(parts[3])
            except ValueError:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                ts = None
            rows.append((ts, sm, smax, parts[6:10]))
        window = "all samples"
        if t_begin is not None and t_end is not None:
            slack = datetime.timedelta(milliseconds=60)
            inside = [r for r in rows if r[0] is not None and t_begin - slack <= r[0] <= t_end + slack]
            if inside:
                rows, window = inside, "timed region"
        reasons = sorted({nm for r in rows for nm, v in zip(cls.NAMES, r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median([r[1] for r in rows]) if rows else None,
                "sm_max_mhz": max(r[2] for r in rows) if rows else None,
                "reasons": reasons, "samples": len(rows), "window": window}

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        return self.summarize(self.lines, self.t_begin, self.t_end)


# ---------------------------------------------------------------------------
# measured FP32 / FP64 peaks (cuBLAS GEMM without tensor-core math)
# ---------------------------------------------------------------------------
def measured_peaks(torch, device):
    out = {}
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        for name, dt, n in (("fp32_tflops", torch.float32, 8192), ("fp64_tflops", torch.float64, 4096)):
            a = torch.randn(n, n, device=device, dtype=dt)
            b = torch.randn(n, n, device=device, dtype=dt)
            torch.matmul(a, b)
            torch.cuda.synchronize()
            best = 0.0
            for _ in range(3):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                torch.matmul(a, b)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                best = max(best, 2.0 * n ** 3 / (ms * 1e-3) / 1e12)
            out[name] = best
            del a, b
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old
    return out


def load_peaks_file():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return json.load(fh)
    except Exception:
        return {}


# ---------------------------------------------------------------------------
# CPU legs (oracle = the C restatement; test infrastructure)
# ---------------------------------------------------------------------------
def cpu_reference_rate(pair, threads, target_s=12.0):
    """Reference algorithm (per-cell string hash-set intersection + FP64 tail),
    one permuted task per thread, every row_stride-th list-1 threshold.
    Returns (perms/s extrapolated to whole tasks, sample description)."""
    import numpy as np
    from oracle import oracle as O
    (r1, f1), (r2, f2) = pair.sorted_lists()
    names = pair.feature_names()
    g1 = [names[f] for f in f1]
    g2 = [names[f] for f in f2]
    n1 = len(O.thresholds(int(r1[-1])))
    n2 = len(O.thresholds(int(r2[-1])))
    rng = np.random.default_rng(123)
    idx1 = np.stack([rng.permutation(len(r1)) for _ in range(threads)]).astype(np.int32)
    idx2 = np.stack([rng.permutation(len(r2)) for _ in range(threads)]).astype(np.int32)
    # calibrate the row stride on a tiny sample
    stride = max(1, n1 // 4)
    t0 = time.perf_counter()
    _, cells = O.ref_run(g1, r1, g2, r2, pair.population, idx1[:1], idx2[:1], 1, stride, 1)
    dt = time.perf_counter() - t0
    per_cell = dt / max(cells, 1)
    want_cells = target_s / per_cell
    stride = int(max(1, min(n1, n1 * n2 / max(want_cells, 1.0))))
    t0 = time.perf_counter()
    _, cells = O.ref_run(g1, r1, g2, r2, pair.population, idx1, idx2, threads, stride, threads)
    dt = time.perf_counter() - t0
    cells_per_task = n1 * n2
    rate = cells / dt / cells_per_task
    sample = ("%d permuted tasks on %d threads, every %d-th list-1 threshold (%d of %d grid cells "
              "per task), %.1f s; perms/s extrapolated from cells/s" %
              (threads, threads, stride, cells // max(threads, 1), cells_per_task, dt))
    return rate, sample, dt


def cpu_fast_oracle_rate(pair, seconds=3.0):
    """The histogram-formulation FP64 oracle, single thread (second CPU column)."""
    import numpy as np
    from oracle import oracle as O
    (r1, f1), (r2, f2) = pair.sorted_lists()
    rng = np.random.default_rng(7)
    done = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds or done == 0:
        O.optimize(r1, f1, r2, f2, pair.n_features, pair.population,
                   rng.permutation(len(r1)).astype(np.int32), rng.permutation(len(r2)).astype(np.int32))
        done += 1
    return done / (time.perf_counter() - t0), done


# ---------------------------------------------------------------------------
def run_reference_config1(args):
    """Config 1 as stated (N = 6,000, ~10 % list-2 ties, 1,000 permutations)
    through the reference algorithm restated in C, every task in full
    (string hash-set intersection per cell, FP64 tail, tasks over all host
    threads).  Permutations: numpy's seeded generator (the reference's own
    generator is unseeded)."""
    import numpy as np
    from oracle import oracle as O
    from dual_threshold_optimization_gb300 import synth
    pair = synth.config1()
    (r1, f1), (r2, f2) = pair.sorted_lists()
    names = pair.feature_names()
    g1 = [names[f] for f in f1]
    g2 = [names[f] for f in f2]
    P = args.ref_tasks
    rng = np.random.default_rng(1)
    idx1 = np.empty((P + 1, len(r1)), np.int32)
    idx2 = np.empty((P + 1, len(r2)), np.int32)
    idx1[0], idx2[0] = np.arange(len(r1)), np.arange(len(r2))
    for t in range(1, P + 1):
        idx1[t] = rng.permutation(len(r1))
        idx2[t] = rng.permutation(len(r2))
    threads = host_threads()
    t0 = time.perf_counter()
    recs, cells = O.ref_run(g1, r1, g2, r2, pair.population, idx1, idx2, P + 1, 1, threads)
    dt = time.perf_counter() - t0
    p_obs = recs[0]["pvalue"]
    emp = O.empirical(p_obs, [r["pvalue"] for r in recs[1:]])
    line = {
        "impl": "reference", "metric": "perms/s, config 1 (N=6000, ties, 1000 permutations)",
        "value": P / dt, "unit": "perms/s", "n_gpus": 0, "steps": 1, "warmup": 0,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "dtype": "f64",
        "data": "synthetic (synth.config1: seeded Gaussian-copula lists, rho 0.3, min-method ties)",
        "config": {"workload": ("config 1: N=6000, ~10 percent of list-2 features in tie blocks of 2-5, "
                                "%d permutations + the unpermuted task, every task in full" % P),
                   "grid": [len(O.thresholds(int(r1[-1]))), len(O.thresholds(int(r2[-1])))]},
        "cpu_baseline": {"value": P / dt, "unit": "perms/s", "cores": threads, "kind": "port",
                         "sample": "all %d tasks, %d grid cells" % (P + 1, cells)},
        "result": {"rank1": recs[0]["rank1"], "rank2": recs[0]["rank2"],
                   "unpermuted_intersection_size": recs[0]["intersection_size"],
                   "unpermuted_pvalue": p_obs, "empirical_pvalue": emp,
                   "fdr": O.fdr(recs[0]["set1_len"], recs[0]["set2_len"], recs[0]["intersection_size"],
                                pair.population)},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    if args.workload == "config1":
        return run_reference_config1(args)
    from dual_threshold_optimization_gb300 import synth
    pair = synth.copula_pair(N_FEATURES, RHO, seed=2)
    threads = host_threads()
    for _ in range(args.warmup):
        cpu_reference_rate(pair, threads, target_s=2.0)
    # each step a bounded sample: --ref-seconds, and the timed steps together
    # about two minutes at most
    per_step = min(args.ref_seconds, max(2.0, 120.0 / max(args.steps, 1)))
    rates, total = [], 0.0
    sample = ""
    for _ in range(args.steps):
        r, sample, dt = cpu_reference_rate(pair, threads, target_s=per_step)
        rates.append(r)
        total += dt
    value = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "perms/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian-copula lists)",
        "config": single_config(PERMS_PER_STEP),
        "cpu_baseline": {"value": value, "unit": "perms/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "perms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference is a Rust crate and cargo is not available: this times the C "
                 "restatement of its algorithm (oracle/dto_oracle.c or_ref_run)"),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    dev = local if torch.cuda.device_count() > local else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from dual_threshold_optimization_gb300 import Engine, synth
    from dual_threshold_optimization_gb300._lib import OPTIMUM_FIELDS

    pair = synth.copula_pair(N_FEATURES, RHO, seed=2)
    eng = Engine(dev)
    dp = eng.pair(pair.ranks1, pair.feat1, pair.ranks2, pair.feat2, pair.n_features, pair.population)
    P = args.perms
    stream = torch.cuda.ExternalStream(eng.stream)
    from dual_threshold_optimization_gb300.run import shard_range

    def null_step(q, s):
        """One step: one null of world * P permutations of seed s, split over
        the ranks by contiguous id ranges (P each: weak scaling).  Rank 0 runs
        the unpermuted task; the one exchange broadcasts its p and sums the
        ranks' counts of permutations at or below it."""
        first, count = shard_range(world * P, rank, world)
        r = q.run(count, seed=s, first=first, precision="screen", unpermuted=(rank == 0))
        if world > 1:
            p_obs = torch.tensor([r.unpermuted["pvalue"] if rank == 0 else 0.0], dtype=torch.float64,
                                 device="cuda")
            torch.distributed.broadcast(p_obs, 0)
            le = torch.tensor([int(np.count_nonzero(r.minp <= float(p_obs.item())))], dtype=torch.int64,
                              device="cuda")
            torch.distributed.all_reduce(le)
            r.summary["count_le_all_ranks"] = int(le.item())
        return r
    seed = 0x5EED0000

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident throughput ----
    # the pair's level-0 quantile by timed trials (dto_pair_tune), untimed;
    # recorded for the pair's shape, so that the end-to-end pairs start with it
    tuned_q0 = dp.tune(min(P, 100_000), seed=seed + 500)
    sampler = ClockSampler(dev)
    sampler.start()  # before the warm-up, so that it samples from the timed region's start
    for w in range(args.warmup):
        null_step(dp, seed + 1000 + w)
    barrier()
    sampler.begin()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    step_ms, grid_ms, launches, summaries = [], [], 0, []
    for s in range(args.steps):
        t0 = time.perf_counter()
        r = null_step(dp, seed + s)
        step_ms.append((time.perf_counter() - t0) * 1e3)
        grid_ms.append(r.summary["grid_ms"])
        launches += r.summary["n_launches"]
        summaries.append(r.summary)
    e1.record(stream)
    barrier()
    sampler.end()
    clocks = sampler.stop()
    total_ms = e0.elapsed_time(e1)
    t_max = total_ms
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t.item())
    value = world * P * args.steps / (t_max * 1e-3)

    # ---- end to end through the C ABI with host buffers ----
    barrier()
    e2e_ms, h2d, d2h = [], 0, 0
    for s in range(args.e2e_steps):
        t0 = time.perf_counter()
        dq = eng.pair(pair.ranks1, pair.feat1, pair.ranks2, pair.feat2, pair.n_features, pair.population)
        rr = null_step(dq, seed + 500 + s)
        h2d = dq.upload_bytes + rr.summary["h2d_bytes"]
        d2h = rr.summary["d2h_bytes"]
        dq.close()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    barrier()
    e2e_value = world * P / (statistics.mean(e2e_ms) * 1e-3) if e2e_ms else None

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    # ---- roofline of the dominant kernel: the level-0 table sweep ----
    cells = dp.n1 * dp.n2
    peaks = measured_peaks(torch, "cuda")
    fp32_peak = peaks.get("fp32_tflops")
    s0_ms = sum(s_["sweep0_ms"] for s_ in summaries)
    s0_tasks = sum(s_["sweep0_tasks"] for s_ in summaries)
    s0_launches = sum(s_["sweep0_launches"] for s_ in summaries)
    achieved = 8.0 * cells * s0_tasks / (s0_ms * 1e-3) / 1e12 if s0_ms > 0 else None
    grid_s = sum(grid_ms) * 1e-3
    whole = 8.0 * cells * args.steps * (P + 1) / grid_s / 1e12
    traffic = args.traffic
    if traffic is None and s0_launches and P == PERMS_PER_STEP:
        traffic = SWEEP0_DRAM_BYTES_PER_TASK * s0_tasks / s0_launches
    roofline = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": (achieved / fp32_peak) if (fp32_peak and achieved) else None,
                "traffic": traffic,
                "kernel": "table_hw_kernel<40>: the table sweep, level 0 with levels 1 and 2 cascaded in the "
                          "same launch (main stream)",
                "work_per_task": "8 FP32-class ops x %d cells (the nine-term log-pmf sum per cell)" % cells,
                "launch_ms": s0_ms / s0_launches if s0_launches else None,
                "tasks_per_launch": s0_tasks / s0_launches if s0_launches else None,
                "peak_source": "measured: cuBLAS SGEMM 8192^3 without TF32 on this GPU (FP32 pipe)",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one level-0 "
                                  "launch at N=20000, per task, scaled to this launch's tasks",
                "whole_search": {"achieved": whole, "frac": whole / fp32_peak if fp32_peak else None,
                                 "note": "all search kernels of a step (table levels, exhaustive "
                                         "fallback, first batch), CUDA-event times summed over streams"},
                "grid_ms_per_step": statistics.mean(grid_ms),
                "perm_ms_per_step": statistics.mean(s_["perm_ms"] for s_ in summaries)}

    # ---- plain FP64 GPU path on a sample ----
    fp64 = None
    if args.fp64_perms > 0:
        r64 = dp.run(args.fp64_perms, seed=seed + 777, precision="fp64")
        r32 = dp.run(args.fp64_perms, seed=seed + 777, precision="screen")
        fp64 = {"value": args.fp64_perms / (r64.summary["device_ms"] * 1e-3), "unit": "perms/s",
                "perms": args.fp64_perms,
                # the optimum fields (the route code differs by design)
                "same_argmin_as_screen": bool(np.array_equal(r64.minp, r32.minp) and all(
                    r64.unpermuted[k] == r32.unpermuted[k] for k in OPTIMUM_FIELDS)),
                "same_minp": bool(np.array_equal(r64.minp, r32.minp))}

    extras = None
    if world == 1 and not args.no_extras:
        extras = extra_configs(eng, args, torch)

    # ---- CPU baseline (reference algorithm restated) ----
    cpu = None
    if not args.no_cpu:
        threads = host_threads()
        rate, sample, _ = cpu_reference_rate(pair, threads, target_s=args.ref_seconds)
        fast, ndone = cpu_fast_oracle_rate(pair)
        cpu = {"value": rate, "unit": "perms/s", "cores": threads, "kind": "port", "sample": sample,
               "fast_oracle_1thread": {"value": fast, "unit": "perms/s", "tasks": ndone,
                                       "note": "histogram-formulation FP64 oracle"}}
        if extras is not None:
            from dual_threshold_optimization_gb300 import synth
            for key, make in (("config1", synth.config1), ("config4", synth.config4)):
                f, n = cpu_fast_oracle_rate(make())
                extras[key]["fast_oracle_1thread"] = {"value": f, "unit": "perms/s", "tasks": n}

    s0 = summaries[-1]
    line = {
        "metric": METRIC, "value": value, "unit": "perms/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f32 screen, f64 refine",
        "data": "synthetic (seeded Gaussian-copula lists)",
        "config": single_config(P),
        "ladder": "value: the pair keeps the table ladder its warm-up runs measured; e2e: a new "
                  "pair each step, which starts from the ladder of the earlier pairs of its shape",
        "level0_quantile": {"value": tuned_q0, "source": "dto_pair_tune: timed trial runs of 0.80, 0.85 "
                                                         "and 0.90 before the warm-up"},
        "timeline_ms_per_step": {
            "permutations": statistics.mean(s_["perm_ms"] for s_ in summaries),
            "level0_sweeps": statistics.mean(s_["sweep0_ms"] for s_ in summaries),
            "after_last_level0": statistics.mean(s_["tail_ms"] for s_ in summaries),
            "note": "device times of the library's CUDA events; the permutations and the table sweeps "
                    "(level 0, with levels 1 and 2 cascaded in the same launch) run one after another on "
                    "the main stream; after_last_level0 is what follows the last sweep (fallbacks, result "
                    "copy)"},
        "routes_per_step": {k: v / args.steps for k, v in
                            ((k, sum(s_["n_route"][k] for s_ in summaries)) for k in summaries[0]["n_route"])},
        "latency_ms": {"p50": statistics.median(step_ms),
                       "p99": sorted(step_ms)[min(len(step_ms) - 1, int(0.99 * len(step_ms)))]},
        "e2e": {"value": e2e_value, "unit": "perms/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "fp64_gpu": fp64,
        "clocks": clocks,
        "gpu_launches": launches,
        "other_configs": extras,
        "screen": {"fp64_refines_per_task": s0["n_refined"] / (P + 1),
                   "stage2_per_task": s0["n_stage2"] / (P + 1),
                   "logp_err_bound_screen": s0["logp_err_bound_screen"],
                   "logp_err_bound_fp64": s0["logp_err_bound_fp64"],
                   "empirical_pvalue": s0["empirical_pvalue"], "fdr": s0["fdr"]},
        "peaks": {"fp32_tflops": fp32_peak, "fp64_tflops": peaks.get("fp64_tflops"),
                  "hbm_gbs": load_peaks_file().get("hbm_gbs")},
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# the other benchmark configurations, as short extra keys of the N=1 line
# ---------------------------------------------------------------------------
def _timed_runs(dp, P, seeds, torch):
    """Device-resident perms/s of dp.run(P) over the given seeds (one run each,
    CUDA events on the library's stream)."""
    ms = []
    res = None
    for sd in seeds:
        torch.cuda.synchronize()
        res = dp.run(P, seed=sd, precision="screen")
        ms.append(res.summary["device_ms"])
    return P / (statistics.mean(ms) * 1e-3), statistics.mean(ms), res


def fp64_rate(dp, perms, seed):
    """The plain FP64 GPU path on `perms` permutations (device time), and
    whether its optima equal the screen path's."""
    import numpy as np
    from dual_threshold_optimization_gb300._lib import OPTIMUM_FIELDS
    r64 = dp.run(perms, seed=seed, precision="fp64")
    r32 = dp.run(perms, seed=seed, precision="screen")
    same = bool(np.array_equal(r64.minp, r32.minp)
                and all(r64.unpermuted[k] == r32.unpermuted[k] for k in OPTIMUM_FIELDS))
    return {"value": perms / (r64.summary["device_ms"] * 1e-3), "unit": "perms/s", "perms": perms,
            "same_optima_as_screen": same}


def extra_configs(eng, args, torch):
    """Configs 1, 3, 4 and 5 of the benchmark set, each short: perms/s with the
    pair resident (warm ladder after one untimed run), its statistics, and
    the batch and serving numbers."""
    from dual_threshold_optimization_gb300 import synth
    out = {}
    # config 1: N = 6,000, ~10 % ties; 1,000 permutations as stated, and 100,000
    p1 = synth.config1()
    d1 = eng.pair(p1.ranks1, p1.feat1, p1.ranks2, p1.feat2, p1.n_features, p1.population)
    d1.run(1000, seed=1)
    v1000, ms1000, r1k = _timed_runs(d1, 1000, [11, 12, 13], torch)
    d1.run(100000, seed=2)
    q1 = d1.tune(100000, seed=3)
    v1e5, ms1e5, _ = _timed_runs(d1, 100000, [21, 22, 23], torch)
    out["config1"] = {"workload": "N=6000, rho 0.3, ~10% of list-2 features in tie blocks of 2-5",
                      "perms_1000": {"value": v1000, "unit": "perms/s", "ms_per_run": ms1000},
                      "perms_100000": {"value": v1e5, "unit": "perms/s", "ms_per_run": ms1e5,
                                       "level0_quantile": q1},
                      "unpermuted_pvalue": r1k.unpermuted["pvalue"],
                      "empirical_pvalue": r1k.summary["empirical_pvalue"], "fdr": r1k.summary["fdr"],
                      "fp64_gpu": fp64_rate(d1, 512, 31)}
    d1.close()
    # config 4: 25,000-feature rankings on an 18,000-feature background,
    # geometric ties, 10^6 permutations
    p4 = synth.config4()
    d4 = eng.pair(p4.ranks1, p4.feat1, p4.ranks2, p4.feat2, p4.n_features, p4.population)
    d4.run(1_000_000, seed=41)
    q4 = d4.tune(200_000, seed=45)
    v4, ms4, r4 = _timed_runs(d4, 1_000_000, [42], torch)
    out["config4"] = {"workload": "25000-feature rankings restricted to an 18000-feature background, "
                                  "geometric tie blocks (mean 5), rho 0.1, 1000000 permutations",
                      "value": v4, "unit": "perms/s", "ms_per_run": ms4,
                      "unpermuted_pvalue": r4.unpermuted["pvalue"],
                      "empirical_pvalue": r4.summary["empirical_pvalue"],
                      "count_le": r4.summary["count_le"], "fdr": r4.summary["fdr"],
                      "routes": r4.summary["n_route"], "level0_quantile": q4,
                      "fp64_gpu": fp64_rate(d4, 256, 43)}
    d4.close()
    # config 3: 512 uneven pairs x 10,000 permutations (seeds differ per run)
    pairs = synth.batch_pairs(512, 2000, 30000, 0.0, 0.4, seed=3)
    dps = [eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population) for p in pairs]
    eng.batch_run(dps, 10000, [0xBA7C0000 + q for q in range(512)], lanes=args.lanes)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.batch_run(dps, 10000, [0xBA7D0000 + q for q in range(512)], lanes=args.lanes)
    dtb = time.perf_counter() - t0
    f64 = [fp64_rate(dps[q], 256, 44) for q in range(0, 512, 128)]
    out["config3_batch"] = {"workload": "512 pairs, N ~ U[2000, 30000], rho ~ U[0, 0.4], 10000 "
                                        "permutations each: waves of pairs per multi-pair sweep (pairs "
                                        "without a ladder on %d lanes)" % args.lanes,
                            "value": 512 * 10000 / dtb, "unit": "perms/s", "ms_per_batch": dtb * 1e3,
                            "fp64_gpu": {"value": 4 * 256 / sum(256 / f["value"] for f in f64),
                                         "unit": "perms/s", "sample": "256 permutations of pairs 0, 128, "
                                                                     "256, 384",
                                         "same_optima_as_screen": all(f["same_optima_as_screen"] for f in f64)}}
    for d in dps:
        d.close()
    # config 5: a short serving run (60 requests)
    sv = serve_measure(eng, 60, args.lanes, [0.5])
    sv.pop("lists"), sv.pop("Ps")
    out["config5_serve"] = sv
    return out


# ---------------------------------------------------------------------------
# many pairs: the batch of uneven pairs and the serving loop
# ---------------------------------------------------------------------------
BATCH_METRIC = "perms/s over a batch of 512 uneven pairs (N 2k-30k, 10k permutations each) on 1 GB300"
SERVE_METRIC = ("serving: perms/s and p50/p99 request latency under Poisson arrivals "
                "(N 1k-60k log-uniform, 1k-100k permutations log-uniform) on 1 GB300")


def run_batch(args):
    import numpy as np
    import torch
    from dual_threshold_optimization_gb300 import Engine, synth
    rank, world, local = dist_env()
    dev = local if torch.cuda.device_count() > local else 0
    torch.cuda.set_device(dev)
    npairs, P = args.batch_pairs, args.batch_perms
    pairs = synth.batch_pairs(npairs, 2000, 30000, 0.0, 0.4, seed=3)
    eng = Engine(dev)
    dps = [eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population) for p in pairs]
    cells = sum(dp.n1 * dp.n2 for dp in dps)
    # every run takes seeds of its own: a pair's stored ladder never comes from
    # the very permutations it then screens
    def step_seeds(k):
        return [0xBA7C0000 + 0x10000 * k + q for q in range(npairs)]
    for w in range(args.warmup):
        eng.batch_run(dps, P, step_seeds(1000 + w), lanes=args.lanes)
    torch.cuda.synchronize()
    sampler = ClockSampler(dev)
    sampler.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        res = eng.batch_run(dps, P, step_seeds(k), lanes=args.lanes)
    dt = (time.perf_counter() - t0) / max(args.steps, 1)
    clocks = sampler.stop()
    value = npairs * P / dt
    # end to end: pairs created from host arrays inside the timed region
    e2e_t, h2d = [], 0
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        dq = [eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population) for p in pairs]
        rr = eng.batch_run(dq, P, step_seeds(2000), lanes=args.lanes)
        e2e_t.append(time.perf_counter() - t0)
        h2d = sum(d.upload_bytes for d in dq)
        for d in dq:
            d.close()
    d2h = sum(8 * P + 80 for _ in pairs)
    launches = sum(r.summary["n_launches"] for r in res)
    line = {
        "metric": BATCH_METRIC, "value": value, "unit": "perms/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32+f32 screen, f64 refine",
        "data": "synthetic (seeded Gaussian-copula lists, N ~ U[2000, 30000], rho ~ U[0, 0.4])",
        "config": {"workload": "batch: %d pairs x %d permutations, waves of pairs per multi-pair sweep "
                               "(pairs without a ladder on %d lanes)" % (npairs, P, args.lanes),
                   "pairs": npairs, "permutations_per_pair": P, "lanes": args.lanes,
                   "grid_cells_total": cells,
                   "l2": "inputs larger than L2: each step streams %d MB of permutation labels"
                         % (sum(p.ranks1.shape[0] for p in pairs) * P * 2 // 1000000)},
        "e2e": {"value": npairs * P / statistics.mean(e2e_t) if e2e_t else None, "unit": "perms/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "cells_per_s": cells * P / dt,
        "clocks": clocks, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    return 0


def serve_measure(eng, M, lanes, loads, rng_seed=5):
    """Config 5: M requests (N log-uniform in [1,000, 60,000], permutations
    log-uniform in [1,000, 100,000], rho uniform in [0, 0.4]), each creating its
    pair from host arrays at arrival and submitted to a server of `lanes`
    lanes: all at once (saturated), then Poisson arrivals at each fraction of
    the saturated rate.  Latency = arrival to completion (host clock)."""
    import numpy as np
    from dual_threshold_optimization_gb300 import synth
    def requests(seed, pair_seed0):
        rng = np.random.default_rng(seed)
        Ns = np.exp(rng.uniform(np.log(1000), np.log(60000), M)).astype(int)
        Ps = np.exp(rng.uniform(np.log(1000), np.log(100000), M)).astype(int)
        rhos = rng.uniform(0.0, 0.4, M)
        lists = [synth.copula_pair(int(n), float(r), seed=pair_seed0 + q) for q, (n, r) in enumerate(zip(Ns, rhos))]
        return Ns, Ps, lists

    # the warm-up plays requests of its own (other sizes, other lists): the
    # timed requests find only what earlier timed requests left
    _, Ps_w, lists_w = requests(rng_seed + 1000, 50_000)
    Ns, Ps, lists = requests(rng_seed, 500)
    rng = np.random.default_rng(rng_seed + 1)
    total_perms = int(Ps.sum())

    def play(srv, arrivals, seed0, lists=lists, Ps=Ps):
        jobs = []
        t0 = time.perf_counter()
        for q in range(M):
            now = time.perf_counter() - t0
            if arrivals[q] > now:
                time.sleep(arrivals[q] - now)
            ta = time.perf_counter()
            p = lists[q]
            dp = eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
            ts = time.perf_counter()
            jobs.append((srv.submit(dp, int(Ps[q]), seed=seed0 + q), dp, ta, ts))
        lat, t_end = [], 0.0
        for job, dp, ta, ts in jobs:
            job.wait()
            done = ts + (job.queue_ms + job.run_ms) * 1e-3
            lat.append(done - ta)
            t_end = max(t_end, done)
            dp.close()
        return np.array(lat), t_end - t0

    with eng.server(lanes=lanes) as srv:
        play(srv, np.zeros(M), 900, lists_w, Ps_w)  # warm-up: every request at once
        lat0, span = play(srv, np.zeros(M), 1900)
        cap_rps = M / span
        rates = []
        for k, frac in enumerate(loads):
            lam = frac * cap_rps
            arr = np.cumsum(rng.exponential(1.0 / lam, M))
            lat, span_r = play(srv, arr, 2900 + 1000 * k)
            rates.append({"load": frac, "rate_rps": lam, "p50_ms": float(np.median(lat) * 1e3),
                          "p99_ms": float(np.quantile(lat, 0.99) * 1e3),
                          "perms_per_s": total_perms / span_r})
    return {"requests": M, "lanes": lanes, "permutations_total": total_perms,
            "n_range": [int(Ns.min()), int(Ns.max())], "perm_range": [int(Ps.min()), int(Ps.max())],
            "saturated": {"perms_per_s": total_perms / span, "requests_per_s": cap_rps,
                          "p50_ms": float(np.median(lat0) * 1e3), "p99_ms": float(np.quantile(lat0, 0.99) * 1e3)},
            "poisson": rates, "lists": lists, "Ps": Ps}


def run_serve(args):
    import torch
    from dual_threshold_optimization_gb300 import Engine
    rank, world, local = dist_env()
    dev = local if torch.cuda.device_count() > local else 0
    torch.cuda.set_device(dev)
    eng = Engine(dev)
    sampler = ClockSampler(dev)
    sampler.start()
    sv = serve_measure(eng, args.serve_requests, args.lanes, args.serve_loads)
    clocks = sampler.stop()
    lists, Ps = sv.pop("lists"), sv.pop("Ps")
    M = sv["requests"]
    # the plain FP64 GPU path on a sample of the same requests (256 permutations each)
    fp64_perms, fp64_s, nreq = 0, 0.0, 0
    for q in range(0, M, max(1, M // 4)):
        p = lists[q]
        dp = eng.pair(p.ranks1, p.feat1, p.ranks2, p.feat2, p.n_features, p.population)
        r = dp.run(256, seed=1, precision="fp64")
        fp64_perms += 256
        fp64_s += r.summary["device_ms"] * 1e-3
        nreq += 1
        dp.close()
    sat = sv["saturated"]
    line = {
        "metric": SERVE_METRIC, "value": sat["perms_per_s"], "unit": "perms/s", "n_gpus": 1,
        "steps": 1, "warmup": 1, "ms_per_step": sv["permutations_total"] / sat["perms_per_s"] * 1e3,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32+f32 screen, f64 refine",
        "data": "synthetic (seeded Gaussian-copula lists)",
        "config": {"workload": "serve: %d requests, %d lanes" % (M, args.lanes), "requests": M,
                   "lanes": args.lanes, "permutations_total": sv["permutations_total"],
                   "n_range": sv["n_range"], "perm_range": sv["perm_range"]},
        "saturated": sat, "poisson": sv["poisson"],
        "fp64_gpu": {"value": fp64_perms / fp64_s, "unit": "perms/s",
                     "sample": "%d permutations over %d of the requests" % (fp64_perms, nreq)},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--perms", type=int, default=PERMS_PER_STEP)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--fp64-perms", type=int, default=2432)
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per grid-kernel launch from an ncu capture")
    ap.add_argument("--no-extras", action="store_true",
                    help="leave out the short runs of configs 1, 3 and 4 from the N=1 line")
    ap.add_argument("--ref-tasks", type=int, default=1000,
                    help="--impl reference --workload config1: permutations run in full")
    ap.add_argument("--workload", default="single", choices=["single", "batch", "serve", "config1"],
                    help="single: the headline pair; batch: 512 uneven pairs; serve: Poisson request loop")
    ap.add_argument("--lanes", type=int, default=4)
    ap.add_argument("--batch-pairs", type=int, default=512)
    ap.add_argument("--batch-perms", type=int, default=10000)
    ap.add_argument("--serve-requests", type=int, default=120)
    ap.add_argument("--serve-loads", type=float, nargs="*", default=[0.5, 0.8])
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
