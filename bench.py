"""Benchmark of the GB300 SCAMP engine.

Default workload (the configuration the headline target is quoted on): a
self-join of a seeded random walk plus 0.5 N(0,1) noise, n = 2^24 points,
window m = 1024, 1NN_INDEX, mixed precision.  A step is one complete join
through the C ABI's scamp_gb300_join with pinned host buffers: ``value`` is
comparisons/s over the join's device time (the CUDA events the join records
on its stream around its device work, statistics to final profile, after
the input copy), ``e2e`` the same comparisons over the wall clock of the
whole call (host->device copy of the series and the best-so-far profile,
the join, device->host copy of the profile).  The series (128 MiB) and its
statistics (1.2 GiB) exceed the 129 MB L2, so nothing is flushed between
steps.  The FP64 form and the mixed-vs-FP64 error check run on the first
2^22 samples (the whole FP64 join takes about 17 minutes); the CPU baseline
on the first 2^17 samples.

``--workload ab``: the AB-join of 2^20 x 2^19 random walks with planted
motifs and NaNs, m = 256, 1NN_INDEX both directions; ``value`` with the
series resident in HBM (scamp_gb300_join_dev), ``e2e`` through
scamp_gb300_join.  ``--workload batch`` / ``gaps``: the batched and the
gapped large self-join workloads.

``--impl reference`` times the CPU path instead: the reference's own CPU
join compiled from its sources where that was possible, else the oracle's C
restatement of it (the reference tree does not exist on the GPU host), with
every host thread, on a bounded sample of the workload per step.

Multi-GPU (torchrun): every rank runs an independent replica of the join
(the engine is single-GPU); the timed region is barrier-bracketed and the
max over ranks is reported.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "gpu-scrimp-large_gb300"))

METRIC = "pairwise comparisons/s (1 GB300), mixed-precision vs FP64 at max|r err|≤1e-5"
WORKLOAD = ("AB-join: A = random walk 2^20, B = random walk 2^19, 64 planted sin motifs "
            "(len 256), 0.1% NaN samples, m=256, 1NN_INDEX both directions (keep_rows)")
NA, NB, M = 1 << 20, 1 << 19, 256
# CPU sample: the same distributions, A[:2^17] x B[:2^16], both directions.
CPU_NA, CPU_NB = 1 << 17, 1 << 16
# Algorithmic work per comparison: 2 FMA (covariance update) + 2 MUL
# (r = cov * inv_c * inv_r), counted on the FMA pipe.
OPS_PER_CELL = 4
# DRAM bytes of one launch of the mixed join kernel on this workload: not
# captured for the current kernel (captures beyond the launch times run on
# small cases: profiles/join_mixed_1nn_coarse_selfjoin_2e20_m1024.txt for the
# default workload), so the line reports none.
DRAM_BYTES_PER_LAUNCH = None


def max_over_ranks(x, dist, device):
    """The largest per-rank value (seconds or ms of a step): replicas are
    timed by their slowest rank.  `dist` is torch.distributed or None."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def replica_value(cells_per_rank, world, step_seconds):
    """Whole-job comparisons/s of N replicas: all ranks' cells over the
    slowest rank's step time (weak scaling)."""
    return cells_per_rank * world / step_seconds


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


# Second workload (--workload self): the precision study's large self-join,
# random walk + 0.5 N(0,1) noise, n = 2^24, m = 1024.  Its FP64 leg and the
# error check run on the first 2^22 samples (FP64 on the whole join takes
# ~20 minutes); comparisons/s are per-cell rates, so they carry over.
SELF_WORKLOAD = "self-join: random walk + 0.5 N(0,1) noise, n=2^24, m=1024, 1NN_INDEX"
SELF_M = 1024
SELF_FP64_PREFIX = 1 << 22
WORKLOAD_KIND = "self"


def make_workload(na=None, nb=None):
    from scamp_gb300 import workloads

    if WORKLOAD_KIND == "self":
        a, m = workloads.noisy_walk_selfjoin(n=na or NA, m=SELF_M)
        return a, None, m
    return workloads.motif_abjoin(na=na or NA, nb=nb or NB, m=M)


def _cpu_join():
    """The CPU join the reference arm and the baseline leg time: the
    reference's own CPU path compiled from its sources (oracle/_ref) where it
    was built on this machine, else the oracle's restatement of it.
    Returns (join(a, b, m, threads), kind)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle

    oracle.load()
    if oracle.ref_available():
        return (lambda a, b, m, threads: oracle.ref_join(a, b, m, keep_rows=b is not None,
                                                         threads=threads)), "reference"
    return (lambda a, b, m, threads: oracle.join(a, b, m, keep_rows=b is not None,
                                                 threads=threads)), "port"


def run_reference(args, world, rank):
    """CPU path of the reference (its compiled sources where built here, else
    the oracle restatement), bounded sample."""
    if rank != 0:
        return
    cpu_join, kind = _cpu_join()
    import oracle  # on sys.path once _cpu_join has run

    a, b, cells, sample = cpu_sample()
    m = M if WORKLOAD_KIND == "ab" else SELF_M
    threads = oracle.max_threads()
    for _ in range(args.warmup):
        cpu_join(a, b, m, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_join(a, b, m, threads)
    dt = (time.perf_counter() - t0) / args.steps
    value = cells / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "comparisons/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD if WORKLOAD_KIND == "ab" else SELF_WORKLOAD,
                   "sample": sample},
        "cpu_baseline": {"value": value, "unit": "comparisons/s", "cores": threads,
                         "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": "comparisons/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_sample():
    """Bounded CPU sample of the workload: (a, b, cells, description)."""
    if WORKLOAD_KIND == "self":
        a, _, m = make_workload(1 << 24)
        a = a[:CPU_NA]
        ns = len(a) - m + 1
        e = m // 4
        cells = (ns - e) * (ns - e + 1) // 2
        return a, None, cells, "first 2^17 samples of the workload, self-join, DOUBLE"
    a, b, m = make_workload(1 << 20, 1 << 19)
    a, b = a[:CPU_NA], b[:CPU_NB]
    cells = (len(a) - m + 1) * (len(b) - m + 1)
    return a, b, cells, "A[:2^17] x B[:2^16] of the workload, both directions, DOUBLE"


def cpu_baseline_leg():
    cpu_join, kind = _cpu_join()
    import oracle  # on sys.path once _cpu_join has run

    a, b, cells, sample = cpu_sample()
    m = M if WORKLOAD_KIND == "ab" else SELF_M
    threads = oracle.max_threads()
    t0 = time.perf_counter()
    cpu_join(a, b, m, threads)
    dt = time.perf_counter() - t0
    return {"value": cells / dt, "unit": "comparisons/s", "cores": threads, "kind": kind,
            "sample": sample + ", %.1f s" % dt}


BATCH_WORKLOAD = ("4096 independent self-joins: lengths round(2^U[10,16]), random walks scaled by "
                  "LogU(1e-3,1e3) and offset by U(-1e4,1e4), windows from {32,64,128}, 1NN_INDEX")


GAPS_WORKLOAD = ("self-join: random walk n=2^23 with 1% of samples in NaN gaps of length "
                 "U[1,500], m=4096, 1NN_INDEX and SUM_THRESH (r > 0.9)")
GAPS_FP64_PREFIX = 1 << 21


def run_gaps_workload(args, world, rank, local):
    """--workload gaps: the very large self-join's distribution, 2^23 samples
    by default (--na-log2 27 runs its stated size, about 35 minutes per
    form); mixed 1NN and SUM_THRESH (--gaps-profiles) on the whole series,
    each after --warmup joins; FP64 and the mixed-vs-FP64 errors on the
    first 2^21 samples."""
    import scamp_gb300
    from scamp_gb300 import workloads

    n = 1 << (args.na_log2 or 23)
    x, m = workloads.gapped_walk_selfjoin(n=n, m=4096)
    res = {}
    for prof in args.gaps_profiles.split(","):
        r = None
        for _ in range(args.warmup + 1):
            r = scamp_gb300.join(x, None, m, prof, "mixed", threshold=0.9, device=local)
        res[prof] = {"value": r["comparisons"] / (r["elapsed_ms"] * 1e-3), "ms": r["elapsed_ms"],
                     "comparisons": r["comparisons"], "join_kernel_ms": r["join_kernel_ms"],
                     "work_counters": r["counters"], "gpu_launches": r["gpu_launches"],
                     "reported_max_abs_r_err": r["max_abs_r_err"],
                     "max_tie_margin": r["max_tie_margin"]}
        try:
            import torch

            free, total = torch.cuda.mem_get_info(local)
            res[prof]["device_memory_in_use_gib"] = (total - free) / 2 ** 30
        except Exception:  # the figure is informational
            pass
        xp = x[:GAPS_FP64_PREFIX]
        mp = scamp_gb300.join(xp, None, m, prof, "mixed", threshold=0.9, return_corr=True,
                              device=local)
        fp = scamp_gb300.join(xp, None, m, prof, "double", threshold=0.9, return_corr=True,
                              device=local)
        res[prof]["fp64_value"] = fp["comparisons"] / (fp["elapsed_ms"] * 1e-3)
        if prof == "1NN_INDEX":
            ok = fp["corr_a"] >= -1
            _, i1 = scamp_gb300.unpack_profile(mp["profile_a"])
            _, i2 = scamp_gb300.unpack_profile(fp["profile_a"])
            res[prof]["max_abs_r_err"] = float(np.max(np.abs(mp["corr_a"][ok] - fp["corr_a"][ok])))
            res[prof]["index_agreement"] = float(np.mean(i1[ok] == i2[ok]))
        else:
            d = np.abs(mp["sum_a"] - fp["sum_a"])
            res[prof]["max_abs_sum_diff"] = float(d.max())
            res[prof]["mean_sum"] = float(np.mean(fp["sum_a"]))
    if rank != 0:
        return
    first = res[args.gaps_profiles.split(",")[0]]
    line = {"metric": METRIC, "value": first["value"], "unit": "comparisons/s",
            "n_gpus": 1, "steps": 1, "warmup": args.warmup,
            "ms_per_step": first["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": GAPS_WORKLOAD.replace("n=2^23", "n=2^%d" % (n.bit_length() - 1)),
                       "fp64": "first 2^21 samples (FP64 and the error checks)"},
            "forms": res}
    print(json.dumps(line), flush=True)


def run_batch_workload(args, world, rank, local):
    """--workload batch: every series of the batch in one scamp_gb300_join_batch
    call (host buffers in and out, so value and e2e are both whole calls);
    beside it the same series joined one call at a time, a sample checked
    against FP64 single joins, and the CPU port on a sample of series."""
    import torch

    import scamp_gb300
    from scamp_gb300 import workloads

    torch.cuda.set_device(local)
    batch = workloads.walk_batch()
    if args.batch_series:
        batch = batch[: args.batch_series]  # a smaller batch, for profiling captures
    series = [x for x, _ in batch]
    windows = [m for _, m in batch]
    if args.profile_only:
        # the batched calls alone, at the tile-height rule (ncu captures)
        for _ in range(args.warmup + args.steps):
            scamp_gb300.join_batch(series, windows, "mixed", device=local)
        torch.cuda.synchronize(local)
        return
    # tile height per window, tuned once (kept for every later call)
    t0 = time.perf_counter()
    seg = scamp_gb300.tune_batch(series, windows, "mixed", device=local)
    tune_s = time.perf_counter() - t0
    tuned = {int(m): int(max(k for k, w in zip(seg, windows) if w == m)) for m in sorted(set(windows))}
    for _ in range(max(args.warmup, 3)):
        out = scamp_gb300.join_batch(series, windows, "mixed", return_corr=True, device=local)
    cells = sum(r["comparisons"] for r in out)
    dev_ms, wall = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            out = scamp_gb300.join_batch(series, windows, "mixed", return_corr=True, device=local)
            wall.append(time.perf_counter() - t0)
            dev_ms.append(out[0]["elapsed_ms"])
    clocks = clk.summary()
    ms_step = sum(dev_ms) / len(dev_ms)
    wall_s = sum(wall) / len(wall)
    # the same series one join per call
    t0 = time.perf_counter()
    for x, m in batch:
        scamp_gb300.join(x, None, m, "1NN_INDEX", "mixed", device=local)
    loop_s = time.perf_counter() - t0
    # accuracy: FP64 single joins of a sample of the series
    max_err, agree, nv = 0.0, 0, 0
    for k in range(0, len(batch), 128):
        x, m = batch[k]
        f = scamp_gb300.join(x, None, m, "1NN_INDEX", "double", return_corr=True, device=local)
        ok = f["corr_a"] >= -1
        if ok.any():
            max_err = max(max_err, float(np.max(np.abs(out[k]["corr_a"][ok] - f["corr_a"][ok]))))
            _, i1 = scamp_gb300.unpack_profile(out[k]["profile_a"])
            _, i2 = scamp_gb300.unpack_profile(f["profile_a"])
            agree += int(np.sum(i1[ok] == i2[ok]))
            nv += int(ok.sum())
    peak32 = scamp_gb300.pipe_peak("fp32", local)
    k_ms = out[0]["join_kernel_ms"] - out[0]["counters"]["verify_kernel_ms"]
    achieved = cells * OPS_PER_CELL / (k_ms * 1e-3)
    if rank != 0:
        return
    h2d = sum(len(x) * 8 + (len(x) - m + 1) * 8 for x, m in batch)
    d2h = sum((len(x) - m + 1) * 16 for x, m in batch)
    line = {
        "metric": METRIC, "value": cells / (ms_step * 1e-3), "unit": "comparisons/s",
        "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": BATCH_WORKLOAD, "form": "mixed, one scamp_gb300_join_batch call",
                   "comparisons_per_step": cells, "series": len(batch),
                   "segment_rows_by_window": tuned, "autotune_s": tune_s,
                   "timing": "device events from the first H2D copy to the last D2H copy; "
                             "device part one CUDA graph, replayed"},
        "max_abs_r_err_vs_fp64_sample": max_err,
        "index_agreement_vs_fp64_sample": agree / max(nv, 1),
        "one_call_per_series_s": loop_s,
        "batched_speedup_vs_one_call_per_series": loop_s / wall_s,
        "roofline": {"bound": "fp32_fma_pipe", "achieved": achieved / 1e12, "peak": peak32 / 1e12,
                     "unit": "Tops/s", "frac": achieved / peak32, "traffic": None,
                     "kernel": "join_mixed_1nn_kernel", "kernel_ms": k_ms,
                     "ops_per_comparison": OPS_PER_CELL},
        "e2e": {"value": cells / wall_s, "unit": "comparisons/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": out[0]["gpu_launches"] * args.steps,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle

        oracle.load()
        threads = oracle.max_threads()
        sample = batch[:256]
        c_cells = 0
        t0 = time.perf_counter()
        for x, m in sample:
            oracle.join(x, None, m, threads=threads)
            ns = len(x) - m + 1
            e = m // 4
            c_cells += max(ns - e, 0) * max(ns - e + 1, 0) // 2
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": c_cells / dt, "unit": "comparisons/s", "cores": threads,
                                "kind": "port", "sample": "first 256 series of the batch, DOUBLE, "
                                                          "%.1f s" % dt}
    print(json.dumps(line), flush=True)


# DRAM bytes (read + write) of one band-kernel launch on the 2^24-point
# self-join: a one-launch ncu capture of the first 2^20 samples (196.0 MB
# read + 648.2 MB written, profiles/join_mixed_1nn_coarse_selfjoin_2e20_m1024
# .txt), scaled by the window count (x16), since the bytes are mostly the
# 16-byte verification requests, whose number grows with the windows.
SELF_DRAM_BYTES_PER_LAUNCH = (196.0e6 + 648.2e6) * 16


def run_self_headline(args, world, rank, local):
    """The default workload: the 2^24-point m = 1024 self-join, one join per
    step through scamp_gb300_join (host buffers)."""
    import torch

    import scamp_gb300

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    a_np, _, m = make_workload()
    n = len(a_np)
    ns = n - m + 1
    a_pin = torch.from_numpy(a_np).pin_memory().numpy()
    p_pin = torch.empty(ns, dtype=torch.int64).pin_memory().numpy().view(np.uint64)

    def step():
        p_pin[:] = scamp_gb300.NO_MATCH  # an empty best-so-far profile
        t0 = time.perf_counter()
        r = scamp_gb300.join(a_pin, None, m, "1NN_INDEX", "mixed", profile_a=p_pin,
                             inplace=True, device=local)
        return time.perf_counter() - t0, r

    for _ in range(args.warmup):
        step()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    dev_ms, wall, kernel_ms, verify_ms, launches = [], [], [], [], 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            dt, r = step()
            wall.append(dt)
            dev_ms.append(r["elapsed_ms"])
            kernel_ms.append(r["join_kernel_ms"] - r["counters"]["verify_kernel_ms"])
            verify_ms.append(r["counters"]["verify_kernel_ms"])
            launches += r["gpu_launches"]
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = clk.summary()
    cells = r["comparisons"]
    ms_step = max_over_ranks(sum(dev_ms) / len(dev_ms), dist, dev)
    e2e_s = max_over_ranks(sum(wall) / len(wall), dist, dev)
    value = replica_value(cells, world, ms_step * 1e-3)

    # FP64 form and the error check on the first 2^22 samples
    xp = a_np[:SELF_FP64_PREFIX] if n > SELF_FP64_PREFIX else a_np
    r64 = scamp_gb300.join(xp, None, m, "1NN_INDEX", "double", return_corr=True, device=local)
    rmx = scamp_gb300.join(xp, None, m, "1NN_INDEX", "mixed", return_corr=True, device=local)
    ok = r64["corr_a"] >= -1
    max_err = float(np.max(np.abs(rmx["corr_a"][ok] - r64["corr_a"][ok]), initial=0.0))
    _, i64 = scamp_gb300.unpack_profile(r64["profile_a"])
    _, imx = scamp_gb300.unpack_profile(rmx["profile_a"])
    agree = float(np.mean(i64[ok] == imx[ok])) if ok.any() else 1.0
    fp64_value = r64["comparisons"] / (r64["elapsed_ms"] * 1e-3)

    peak32 = scamp_gb300.pipe_peak("fp32", local)
    peak64 = scamp_gb300.pipe_peak("fp64", local)
    k_ms = sum(kernel_ms) / len(kernel_ms)
    achieved = cells * OPS_PER_CELL / (k_ms * 1e-3)
    achieved64 = r64["comparisons"] * OPS_PER_CELL / (r64["join_kernel_ms"] * 1e-3)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    traffic = None
    if SELF_DRAM_BYTES_PER_LAUNCH is not None and n == 1 << 24:
        traffic = SELF_DRAM_BYTES_PER_LAUNCH
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "comparisons/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded random walk plus noise)",
        "config": {"workload": SELF_WORKLOAD if n == 1 << 24 else
                   SELF_WORKLOAD.replace("n=2^24", "n=%d" % n),
                   "form": "mixed (FP32 recurrence behind an FP32 filter, FP64-centred "
                           "anchors, FP64 re-evaluation of every reported cell)",
                   "comparisons_per_step": cells,
                   "l2": "not flushed: inputs larger than L2 (series 128 MiB, statistics and "
                         "profile 1.2 GiB per join)",
                   "timing": "value: the join's own device events (statistics to final "
                             "profile); e2e: wall clock of scamp_gb300_join with pinned host "
                             "buffers",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "max_abs_r_err": rmx["max_abs_r_err"],
        "max_tie_margin": rmx["max_tie_margin"],
        "max_abs_r_err_vs_fp64": max_err,
        "index_agreement_vs_fp64": agree,
        "fp64_error_check": "first 2^22 samples: mixed vs FP64 form, both engine joins",
        "fp64": {"value": fp64_value, "unit": "comparisons/s",
                 "comparisons_per_step": r64["comparisons"], "ms_per_step": r64["elapsed_ms"],
                 "sample": "first 2^22 samples of the workload",
                 "roofline": {"bound": "fp64_fma_pipe", "achieved": achieved64 / 1e12,
                              "peak": peak64 / 1e12, "unit": "Tops/s",
                              "frac": achieved64 / peak64, "peak_source": "measured DFMA probe"}},
        "speedup_mixed_vs_fp64": value / world / fp64_value,
        "roofline": {"bound": "fp32_fma_pipe", "achieved": achieved / 1e12, "peak": peak32 / 1e12,
                     "unit": "Tops/s", "frac": achieved / peak32, "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + write.sum)",
                     "kernel": "join_mixed_1nn_kernel", "kernel_ms": k_ms,
                     "ops_per_comparison": OPS_PER_CELL,
                     "verify_kernel_ms": sum(verify_ms) / len(verify_ms),
                     "work_counters": r["counters"],
                     "peak_source": "measured packed-FP32 FMA probe (scamp_gb300_pipe_peak)"},
        "e2e": {"value": replica_value(cells, world, e2e_s), "unit": "comparisons/s",
                "h2d_bytes_per_step": n * 8 + ns * 8, "d2h_bytes_per_step": ns * 8},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_leg()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    # three ~21 s joins of the default workload: about a minute timed
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--fp64-steps", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", default="self", choices=["self", "ab", "batch", "gaps"],
                   help="self: the 2^24-point m=1024 self-join (default); ab: the AB-join "
                        "of 2^20 x 2^19 random walks with motifs and NaNs, m=256")
    p.add_argument("--gaps-profiles", default="1NN_INDEX,SUM_THRESH",
                   help="--workload gaps: profile types to run, comma-separated")
    p.add_argument("--na-log2", type=int, default=None,
                   help="log2 length of A (B is half); smaller only for profiling captures")
    p.add_argument("--batch-series", type=int, default=0,
                   help="--workload batch: only the first N series (profiling captures)")
    p.add_argument("--profile-form", default="mixed", choices=["mixed", "double"],
                   help="form run by --profile-only")
    p.add_argument("--anchor-study", action="store_true",
                   help="--workload self: also time the mixed form at anchor intervals "
                        "K = 128, 256, 1024, 4096 rows on the FP64 leg's samples, each with "
                        "its max |r| error and index agreement against the FP64 form")
    p.add_argument("--profile-only", action="store_true",
                   help="run only the timed mixed joins (for ncu captures); prints no JSON")
    args = p.parse_args()
    global NA, NB, WORKLOAD_KIND
    WORKLOAD_KIND = args.workload
    if args.workload == "self":
        NA = 1 << (args.na_log2 or 24)
        NB = NA
    else:
        na_log2 = args.na_log2 or 20
        NA, NB = 1 << na_log2, 1 << (na_log2 - 1)
    self_join = args.workload == "self"
    world, rank, local = dist_env()

    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.workload == "self" and not (args.anchor_study or args.profile_only):
        run_self_headline(args, world, rank, local)
        return
    if args.workload == "batch":
        run_batch_workload(args, world, rank, local)
        return
    if args.workload == "gaps":
        import torch

        torch.cuda.set_device(local)
        run_gaps_workload(args, world, rank, local)
        return

    import torch

    import scamp_gb300

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    a_np, b_np, m = make_workload()
    nsa = NA - m + 1
    nsb = nsa if self_join else NB - m + 1
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    a_d = torch.from_numpy(a_np).to(dev)
    b_d = a_d if self_join else torch.from_numpy(b_np).to(dev)
    no_match = int(scamp_gb300.NO_MATCH)
    prof_a = torch.empty(nsa, dtype=torch.int64, device=dev)
    prof_b = torch.empty(1 if self_join else nsb, dtype=torch.int64, device=dev)
    corr_a = torch.empty(nsa, dtype=torch.float64, device=dev)
    corr_b = torch.empty(1 if self_join else nsb, dtype=torch.float64, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    nm = no_match - (1 << 64) if no_match >= (1 << 63) else no_match

    def one(precision, n_a=None, anchor=0):
        """One join (the whole workload, or the self-join's first n_a samples;
        anchor: the mixed form's anchor interval, 0 = its default rule)."""
        with torch.cuda.stream(stream):
            prof_a.fill_(nm)
            prof_b.fill_(nm)
            flush.fill_(1)  # L2 flush before the timed join
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        r = scamp_gb300.join_device(
            a_d.data_ptr(), n_a or NA, m, None if self_join else b_d.data_ptr(),
            0 if self_join else NB, "1NN_INDEX", precision,
            computing_rows=True, keep_rows=not self_join, profile_a_ptr=prof_a.data_ptr(),
            profile_b_ptr=None if self_join else prof_b.data_ptr(), corr_a_ptr=corr_a.data_ptr(),
            corr_b_ptr=None if self_join else corr_b.data_ptr(), stream=stream.cuda_stream,
            anchor_interval=anchor, device=local)
        ev1.record(stream)
        ev1.synchronize()
        # the join's own CUDA events on this stream bracket its device work
        # (statistics to final profile); the events above also hold the host's
        # return from the call, so they serve as a check only
        outer = ev0.elapsed_time(ev1)
        inner = r["elapsed_ms"]
        return (inner if 0 < inner <= outer else outer), r

    if args.profile_only and args.profile_form == "double":
        for _ in range(args.warmup + args.steps):
            one("double")
        return

    # ---- mixed form (headline) ----
    for _ in range(max(args.warmup, 1 if self_join else 3)):
        one("mixed")
    barrier()
    torch.cuda.synchronize()
    times, kernel_ms, verify_ms, launches = [], [], [], 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ms, r = one("mixed")
            times.append(ms)
            kernel_ms.append(r["join_kernel_ms"] - r["counters"]["verify_kernel_ms"])
            verify_ms.append(r["counters"]["verify_kernel_ms"])
            launches += r["gpu_launches"]
    torch.cuda.synchronize()
    barrier()
    clocks = clk.summary()
    if args.profile_only:
        return
    cells = r["comparisons"]
    ms_step = max_over_ranks(sum(times) / len(times), dist, dev)
    value = replica_value(cells, world, ms_step * 1e-3)
    mixed_corr = (corr_a.cpu().numpy().copy(), corr_b.cpu().numpy().copy())
    mixed_idx = (prof_a.cpu().numpy().view(np.uint64) >> np.uint64(32),
                 prof_b.cpu().numpy().view(np.uint64) >> np.uint64(32))

    # ---- FP64 form: throughput and the accuracy reference ----
    n_fp64 = None
    if self_join and NA > SELF_FP64_PREFIX:
        # the study's FP64 leg and error check: the first 2^22 samples
        n_fp64 = SELF_FP64_PREFIX
        one("mixed", n_fp64)
        one("mixed", n_fp64)
        mixed_corr = (corr_a.cpu().numpy()[: n_fp64 - m + 1].copy(), mixed_corr[1])
        mixed_idx = ((prof_a.cpu().numpy().view(np.uint64) >> np.uint64(32))[: n_fp64 - m + 1],
                     mixed_idx[1])
    one("double", n_fp64)
    fp64_ms, fp64_kernel = [], []
    for _ in range(max(1, args.fp64_steps)):
        ms, r64 = one("double", n_fp64)
        fp64_ms.append(ms)
        fp64_kernel.append(r64["join_kernel_ms"])
    cells64 = r64["comparisons"]
    n_f = (n_fp64 or NA) - m + 1
    f_corr = (corr_a.cpu().numpy()[:n_f], corr_b.cpu().numpy())
    f_idx = ((prof_a.cpu().numpy().view(np.uint64) >> np.uint64(32))[:n_f],
             prof_b.cpu().numpy().view(np.uint64) >> np.uint64(32))
    max_err, idx_agree, n_valid = 0.0, 0, 0
    for k in range(1 if self_join else 2):
        ok = f_corr[k] >= -1
        if ok.any():
            max_err = max(max_err, float(np.max(np.abs(mixed_corr[k][ok] - f_corr[k][ok]))))
        idx_agree += int(np.sum(mixed_idx[k][ok] == f_idx[k][ok]))
        n_valid += int(ok.sum())
    study = []
    if args.anchor_study and self_join:
        # the precision study's anchor intervals (one slab, 128 rows, is the
        # shortest segment the band kernel runs)
        ok = f_corr[0] >= -1
        for K in (128, 256, 1024, 4096):
            ms, rk = one("mixed", n_fp64, anchor=K)
            c = corr_a.cpu().numpy()[:n_f]
            ix = (prof_a.cpu().numpy().view(np.uint64) >> np.uint64(32))[:n_f]
            study.append({"anchor_interval": K, "ms": ms, "comparisons": rk["comparisons"],
                          "comparisons_per_s": rk["comparisons"] / (ms * 1e-3),
                          "max_abs_r_err_vs_fp64": float(np.max(np.abs(c[ok] - f_corr[0][ok]),
                                                                initial=0.0)),
                          "index_agreement_vs_fp64": float(np.mean(ix[ok] == f_idx[0][ok])),
                          "work_counters": rk["counters"]})

    # ---- e2e through the host-buffer C ABI ----
    a_pin = torch.from_numpy(a_np).pin_memory().numpy()
    b_pin = None if self_join else torch.from_numpy(b_np).pin_memory().numpy()
    pa_pin = torch.empty(nsa, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
    pb_pin = torch.empty(nsb, dtype=torch.int64).pin_memory().numpy().view(np.uint64)
    pa_pin[:] = scamp_gb300.NO_MATCH
    pb_pin[:] = scamp_gb300.NO_MATCH
    e2e_t = []
    for it in range(args.warmup + args.steps):
        # every step starts from an empty profile, like the device-resident leg
        pa_pin[:] = scamp_gb300.NO_MATCH
        pb_pin[:] = scamp_gb300.NO_MATCH
        with torch.cuda.stream(stream):
            flush.fill_(2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = scamp_gb300.join(a_pin, b_pin, m, "1NN_INDEX", "mixed", keep_rows=not self_join,
                             profile_a=pa_pin, profile_b=None if self_join else pb_pin,
                             device=local, inplace=True)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            e2e_t.append(dt)
            launches_e2e = r["gpu_launches"]
    e2e_s = max_over_ranks(sum(e2e_t) / len(e2e_t), dist, dev)
    if self_join:
        h2d, d2h = NA * 8 + nsa * 8, nsa * 8
    else:
        h2d = (NA + NB) * 8 + (nsa + nsb) * 8
        d2h = (nsa + nsb) * 8

    # ---- roofline: the join kernel against the measured FMA-pipe peaks ----
    peak32 = scamp_gb300.pipe_peak("fp32", local)
    peak64 = scamp_gb300.pipe_peak("fp64", local)
    k_ms = sum(kernel_ms) / len(kernel_ms)
    achieved = cells * OPS_PER_CELL / (k_ms * 1e-3)
    k64 = sum(fp64_kernel) / len(fp64_kernel)
    achieved64 = cells64 * OPS_PER_CELL / (k64 * 1e-3)

    if rank != 0:
        return
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "comparisons/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded random walks with planted motifs and NaNs)",
        "config": {"workload": SELF_WORKLOAD if self_join else WORKLOAD,
                   "form": "mixed (FP32 recurrence, FP64-centred anchors)",
                   "comparisons_per_step": cells, "l2": "flushed (512 MB write) before each step",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "max_abs_r_err_vs_fp64": max_err,
        "index_agreement_vs_fp64": idx_agree / max(n_valid, 1),
        "fp64": {"value": cells64 / (sum(fp64_ms) / len(fp64_ms) * 1e-3), "unit": "comparisons/s",
                 "comparisons_per_step": cells64,
                 "ms_per_step": sum(fp64_ms) / len(fp64_ms),
                 "roofline": {"bound": "fp64_fma_pipe", "achieved": achieved64 / 1e12,
                              "peak": peak64 / 1e12, "unit": "Tops/s",
                              "frac": achieved64 / peak64, "peak_source": "measured DFMA probe"}},
        "speedup_mixed_vs_fp64": value / world / (cells64 / (sum(fp64_ms) / len(fp64_ms) * 1e-3)),
        "roofline": {"bound": "fp32_fma_pipe", "achieved": achieved / 1e12, "peak": peak32 / 1e12,
                     "unit": "Tops/s", "frac": achieved / peak32,
                     "traffic": DRAM_BYTES_PER_LAUNCH if (NA == 1 << 20 and not self_join) else None,
                     "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + write.sum)",
                     "kernel": "join_mixed_1nn_kernel", "kernel_ms": k_ms,
                     "ops_per_comparison": OPS_PER_CELL,
                     "verify_kernel_ms": sum(verify_ms) / len(verify_ms),
                     "work_counters": r["counters"],
                     "peak_source": "measured packed-FP32 FMA probe (scamp_gb300_pipe_peak)"},
        "e2e": {"value": replica_value(cells, world, e2e_s), "unit": "comparisons/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if study:
        line["anchor_study"] = study
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_leg()
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
