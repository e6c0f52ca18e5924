#!/usr/bin/env python
"""Benchmark of the V:N:M reordering hot path on GB300.

Workload (one step): the plain NM reorder of the R-MAT 16384 x 16384 matrix
(a, b, c, d = .57, .19, .19, .05; 131072 edges drawn, symmetrised; N(0, 1)
values; 2:4) as the `spmm` command runs it first -- find_best_2toX, all four
schedules -- through the library's C ABI.

  value  whole-job reorders per second (all ranks), inputs resident in HBM
  e2e    the same through the public API with host (pinned) buffers: the
         COO goes host->device and the result back every step
  roofline  the persistent reorder kernel (k_nm_rounds) against HBM
  cpu_baseline  the CPU port of the reference path (oracle/) on the host cores

--impl reference runs the CPU port of the reference algorithm (the
reference's own NM path is CUDA code; its CPU-side restatement stands in) on
the same workload and prints the same JSON line with "impl": "reference".

Multi-GPU: replicas only -- each rank reorders its own seeded matrix (the
path has no exchange step); value = all ranks' reorders / max elapsed time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "vnm-graph-reordering_gb300")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

N_NM, M_NM, V = 2, 4, 64
WORKLOAD = "C2: R-MAT 16384x16384 (a=.57,b=.19,c=.19), 131072 edges symmetrised, N(0,1), 2:4, find_best_2toX"
METRIC = "plain NM reorder throughput (find_best_2toX over schedules 0-3, R-MAT 16384, 2:4)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload(rank):
    from vnm_gb300 import synth
    return synth.rmat_c2(seed=rank)


def cpu_port_find_best(nr, r, c, v, threads):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    best, _ = oracle.find_best(nr, r, c, v, N_NM, M_NM)
    return time.perf_counter() - t0, best


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args, rank, world):
    """CPU port of the reference path, on the host cores, rank 0 only."""
    if rank != 0:
        return
    nr, r, c, v = workload(0)
    threads = host_threads()
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_port_find_best(nr, r, c, v, threads)
    times = []
    for _ in range(args.steps):
        dt, best = cpu_port_find_best(nr, r, c, v, threads)
        times.append(dt)
    tot = sum(times)
    value = args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "reorders/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT)",
        "config": {"workload": WORKLOAD, "nrows": nr, "nnz": int(len(r)), "N": N_NM, "M": M_NM,
                   "schedules": 4, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "reorders/s", "cores": threads, "kind": "port",
                         "sample": "full find_best_2toX of the workload matrix per step (C++ restatement "
                                   "of reorder/reorder.h + main.cu, OpenMP)"},
        "e2e": {"value": value, "unit": "reorders/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import torch
    import vnm_gb300
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    nr, r, c, v = workload(rank)
    ctx = vnm_gb300.Context(local)
    dev = torch.device("cuda", local)
    tr = torch.from_numpy(r).to(dev)
    tc = torch.from_numpy(c).to(dev)
    tv = torch.from_numpy(v).to(dev)
    # pinned host copies for the end-to-end measurement
    hr = torch.from_numpy(r).pin_memory()
    hc = torch.from_numpy(c).pin_memory()
    hv = torch.from_numpy(v).pin_memory()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def step(device_inputs):
        flush.zero_()
        torch.cuda.synchronize()
        if device_inputs:
            return ctx.nm_search(nr, tr, tc, tv, N_NM, M_NM, want_newpos=True)
        return ctx.nm_search(nr, hr.numpy(), hc.numpy(), hv.numpy(), N_NM, M_NM, want_newpos=True)

    for _ in range(args.warmup):
        best, res, newpos = step(True)
    # timed region: inputs resident in HBM
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    dev_ms, main_ms, launches, wall = 0.0, 0.0, 0, 0.0
    stats_sum = None
    phase_sum = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        best, res, newpos = step(True)
        wall += time.perf_counter() - t0
        dev_ms += ctx.last_kernel_ms
        main_ms += ctx.last_main_kernel_ms
        launches += ctx.last_launch_count
        st = ctx.last_stats()
        ph = st.pop("phase_kcycles")
        stats_sum = st if stats_sum is None else {k: stats_sum[k] + st[k] for k in st}
        phase_sum = ph if stats_sum is st else {k: phase_sum[k] + ph[k] for k in ph}
    barrier()
    clk = clocks.stop()
    # the search launches the four jobs and then a second single job for the
    # winner's permutation; the kernel-time sum covers both
    elapsed = dev_ms / 1000.0
    if world > 1:
        t = torch.tensor([elapsed], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * args.steps / elapsed
    # end to end: pinned host buffers through the public API
    for _ in range(1):
        step(False)
    barrier()
    e2e_t = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step(False)
        e2e_t += time.perf_counter() - t0
    barrier()
    if world > 1:
        t = torch.tensor([e2e_t], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e_value = world * args.steps / e2e_t
    h2d = 12 * len(r)
    d2h = 4 * 20 + 4 + 4 * nr
    # roofline of the persistent reorder kernel: bytes its algorithm must move
    # per launch = per round the segment-count scan (4 B x nseg) + per
    # gathered column entry 4 B (row id) + 16 B record update, + per touched
    # row the 16 B record read and clear
    st = stats_sum
    alg_bytes = 4.0 * st["rounds"] * st["nseg"] + 20.0 * st["gathered"] + 32.0 * st["touched"]
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (main_ms / 1000.0) / 1e9 if main_ms > 0 else 0.0
    out = {
        "metric": METRIC, "value": value, "unit": "reorders/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded R-MAT, seed = rank)",
        "config": {"workload": WORKLOAD, "nrows": nr, "nnz": int(len(r)), "N": N_NM, "M": M_NM, "schedules": 4,
                   "parallelism": "replicas" if world > 1 else "single", "l2": "flushed (256 MB write) before "
                   "every step", "best_sched": int(best), "rounds_per_search": int(st["rounds"] // args.steps)},
        "e2e": {"value": e2e_value, "unit": "reorders/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1000.0 * e2e_t / args.steps},
        "roofline": {"kernel": "k_nm_rounds<4>", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                     "alg_bytes_per_step": alg_bytes / args.steps,
                     "kernel_ms_per_step": main_ms / args.steps,
                     "note": "latency-bound sequential greedy; see profiles/",
                     "round_phase_share": {k: round(v / max(1, sum(phase_sum.values())), 4)
                                           for k, v in phase_sum.items()},
                     "us_per_round": 1000.0 * main_ms / max(1, st["rounds"] / max(1, st["jobs"]))},
        "gpu_launches": launches,
        "clocks": clk,
        "wall_ms_per_step": 1000.0 * wall / args.steps,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = host_threads()
        dt, cbest = cpu_port_find_best(nr, r, c, v, threads)
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "reorders/s", "cores": threads, "kind": "port",
                               "sample": "one full find_best_2toX of the same matrix (C++ restatement of the "
                                         "reference NM path, OpenMP)", "best_sched": int(cbest)}
        out["cpu_baseline_agrees"] = bool(cbest == best)
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
