#!/usr/bin/env python
"""Benchmark of the V:N:M reordering hot path on GB300.

Headline workload (one step): the R-MAT 16384 x 16384 matrix (a, b, c, d =
.57, .19, .19, .05; 131072 edges drawn, symmetrised; N(0, 1) values; 2:4) as
the `spmm` command handles it -- find_best_2toX over the four schedules
(bit-exact with the reference), the winner's relabelling, V:N:M compression
(V=64) and the SpMM with a 16384x128 BF16 operand -- through the library's
C ABI.

  value  whole-job steps per second (all ranks), inputs resident in HBM, L2
         flushed before every step
  e2e    the same through the public API with host (pinned) buffers: the
         COO and B go host->device and the permutation and C come back
  roofline  the persistent reorder kernel (k_nm_rounds, 96 % of the step)
         against HBM; the SpMM's issued and useful tensor rates beside it
  cpu_baseline  the CPU port of the reference path (oracle/) on the host cores

After the headline (one GPU, rank 0, not part of its timing) the other
configurations are measured and reported in the same JSON line:
  c3_batch    256 matrices in one persistent launch vs one call each
  c4_learned  learned-proposal reorder vs the plain exact reorder on R-MAT
              65536: wall time to the plain reorder's retained-nnz
  c5_gcn      Chung-Lu 262144 graph: learned reorder, compression and 100
              SpMMs with a 262144x256 BF16 / FP16 operand, error vs FP64
  s1_structured_spmm  a matrix in full V:2:8 form (the operand V:N:M is
              made for) through the tensor-core SpMM, beside cuBLAS/cuSPARSE
(--no-extended skips them.)

--impl reference runs the CPU port of the reference algorithm (the
reference's own NM path is CUDA code; its CPU-side restatement stands in) on
the same workload and prints the same JSON line with "impl": "reference".

Multi-GPU: replicas only -- each rank reorders its own seeded matrix (the
path has no exchange step); value = all ranks' steps / max elapsed time.
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

N_NM, M_NM, V, N_B = 2, 4, 64, 128
# target segments each proposing segment samples per learned round (swept on
# GB300 at R-MAT 65536 2:8: 2 / 4 / 8 / 16 / 32 -> 2.9 / 3.0 / 3.2 / 3.6 /
# 5.7 ms to the plain reorder's retained-nnz with the network, all in 3
# rounds); 4 keeps the candidate pool wide at little cost
TARGETS = 4
WORKLOAD = ("C2: R-MAT 16384x16384 (a=.57,b=.19,c=.19), 131072 edges symmetrised, N(0,1), 2:4, V=64; "
            "find_best_2toX + V:N:M SpMM with B 16384x128 bf16")
# the headline metric of the workload table; `value` is its plain-reorder +
# SpMM step on the R-MAT 16384 workload, the learned-vs-plain half is under
# c4_learned and the SpMM TFLOP/s under spmm / c5_gcn
METRIC = "reorder wall-time to equal retained-nnz (learned vs plain); V:N:M SpMM TFLOP/s"
VALUE_IS = ("hot-path steps/s of the R-MAT 16384 2:4 step (find_best_2toX + relabel + V:N:M compress + SpMM); "
            "learned vs plain in c4_learned, SpMM TFLOP/s in spmm and c5_gcn")
GOLD = os.path.join(REPO, "tests", "golden")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extended", action="store_true", help="skip the batched, learned and GCN configurations")
    ap.add_argument("--c5-spmm-only", action="store_true",
                    help="only the GCN workload's BF16 SpMM, --steps runs, with the reorder's state released first "
                         "(a few GB on the device: the command profiles of that kernel use)")
    ap.add_argument("--s1-spmm-only", action="store_true",
                    help="only the structured V:2:8 SpMM workload on the tensor cores, --steps runs (the command "
                         "profiles of the tensor-core kernel use)")
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


def load_tensor_peak(sustained=False):
    """The measured bf16 tensor peak: the burst figure for a kernel timed
    alone, the sustained one for a kernel timed inside a long loop."""
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if sustained and "bf16_tflops_sustained" in d:
            return float(d["bf16_tflops_sustained"]), "measured (sustained)"
        return float(d["bf16_tflops"]), "measured (burst)"
    return (1700.0, "fallback (sustained)") if sustained else (1900.0, "fallback")


def whole_job_rate(elapsed_s, steps, world, device=None):
    """Replicas: every rank ran `steps` steps on its own matrix; the job's
    rate is all ranks' steps over the slowest rank's time (MAX over ranks,
    on whatever process group is initialised: NCCL in the bench, gloo in
    the CPU tests).  Returns (steps per second, slowest elapsed)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([elapsed_s], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        elapsed_s = float(x.item())
    return world * steps / elapsed_s, elapsed_s


def workload(rank):
    from vnm_gb300 import synth
    return synth.rmat_c2(seed=rank)


def cpu_port_find_best(nr, r, c, v, threads):
    """The oracle's find_best_2toX on `threads` host threads: (seconds, the
    schedule it picks, the four result vectors)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    best, out = oracle.find_best(nr, r, c, v, N_NM, M_NM)
    dt = time.perf_counter() - t0
    # find_best's rows: nrows, nnz, density, init_size, final_size, init_cnt,
    # final_cnt, improve, rounds, ... (main.cu:59-69)
    res4 = np.rint(out[:, [3, 4, 5, 6, 8]]).astype(np.int32)
    return dt, best, res4


def cpu_port_one_schedule(nr, r, c, v, sched, threads):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    oracle.nm_run(nr, r, c, v, N_NM, M_NM, sched)
    return time.perf_counter() - t0


def oracle_nm_run(nr, r, c, v, sched, N=N_NM, M=M_NM):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(host_threads())
    return oracle.nm_run(nr, r, c, v, N, M, sched)


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_port_step(nr, r, c, v, B64, threads):
    """The CPU port of one hot-path step: find_best_2toX (C++ restatement of
    the reference NM path, OpenMP) and the SpMM of the reordered matrix
    (scalar FP64 loop; the reference ships no CPU SpMM)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(threads)
    t0 = time.perf_counter()
    best, _ = oracle.find_best(nr, r, c, v, N_NM, M_NM)
    _, rr, cc, _ = oracle.nm_run(nr, r, c, v, N_NM, M_NM, best)
    oracle.spmm_f64(nr, rr, cc, v.astype(np.float64), B64)
    return time.perf_counter() - t0, best


def scale_golden(name):
    """The oracle's committed results at a benchmarked size (made by
    tests/golden/make_scale_goldens.py), or None when absent."""
    p = os.path.join(GOLD, "scale_oracle_goldens.npz")
    if not os.path.exists(p):
        return None
    g = np.load(p)
    if name + "__res5x4" not in g:
        return None
    return {"res5x4": g[name + "__res5x4"], "newpos4": g[name + "__newpos4"], "best": int(g[name + "__best"]),
            "sha256": str(g[name + "__sha256"])}


def coo_digest(nrows, row, col, val):
    import hashlib
    h = hashlib.sha256()
    h.update(np.int64(nrows).tobytes())
    for a, t in ((row, np.int32), (col, np.int32), (val, np.float32)):
        h.update(np.ascontiguousarray(a, t).tobytes())
    return h.hexdigest()


def nonzero_groups(nrows, row, col, val, M):
    """Nonzero (row, M-column segment) groups of the pattern (val != 0)."""
    m = val != 0
    return int(len(np.unique(row[m].astype(np.int64) * (nrows // M) + col[m] // M)))


def spmm_hbm_bytes(nrows, nnz, n, elem=2):
    """Algorithmic bytes of C = A B: A as CSR (a 16-bit value and a 32-bit
    column per nonzero, 32-bit row pointers), B read once, C (FP32) written
    once."""
    return nnz * (elem + 4) + 4 * (nrows + 1) + nrows * n * elem + nrows * n * 4


def time_cuda(fn, reps, stream=None):
    """Median milliseconds of fn() over reps runs, CUDA events on the
    current stream, one warm-up run."""
    import torch
    fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.median(ms))


def library_spmm_baselines(nr, r, c, v, n, dtype, dense=True, reps=10):
    """Context baselines for the V:N:M SpMM (not the product): cuSPARSE CSR
    SpMM through torch.sparse (FP32, and the 16-bit type where the build
    supports it) and, where the densified matrix fits, a cuBLAS GEMM of the
    densified matrix (16-bit operands, FP32 accumulation)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {}
    g = torch.Generator().manual_seed(99)
    Bf = torch.randn((nr, n), generator=g).to(dev)
    idx = torch.from_numpy(np.stack([r, c]).astype(np.int64)).to(dev)
    A32 = torch.sparse_coo_tensor(idx, torch.from_numpy(v).to(dev), (nr, nr)).coalesce().to_sparse_csr()
    flops = 2.0 * len(r) * n
    try:
        ms = time_cuda(lambda: torch.sparse.mm(A32, Bf), reps)
        out["cusparse_csr_fp32"] = {"ms": ms, "useful_tflops": flops / ms / 1e9}
    except Exception as e:  # report, keep the rest
        out["cusparse_csr_fp32"] = {"error": "%s: %s" % (type(e).__name__, e)}
    try:
        A16 = A32.to(dtype)
        B16 = Bf.to(dtype)
        ms = time_cuda(lambda: torch.sparse.mm(A16, B16), reps)
        out["cusparse_csr_16bit"] = {"ms": ms, "useful_tflops": flops / ms / 1e9, "dtype": str(dtype)}
    except Exception as e:
        out["cusparse_csr_16bit"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if dense and nr * nr * 2 <= (2 << 30):
        Ad = A32.to_dense().to(dtype)
        B16 = Bf.to(dtype)
        ms = time_cuda(lambda: torch.matmul(Ad, B16), reps)
        out["cublas_dense_16bit"] = {"ms": ms, "dense_tflops": 2.0 * nr * nr * n / ms / 1e9,
                                     "useful_tflops": flops / ms / 1e9, "dtype": str(dtype),
                                     "note": "the densified matrix times B; output in the 16-bit type"}
        del Ad
    del A32, Bf
    torch.cuda.empty_cache()
    return out


def reference_gpu(nr, r, c, v, N=N_NM, M=M_NM, timeout=300.0):
    """The reference's own GPU reorder (reorder/reorder.h built from its
    sources with N and M fixed into oracle/_ref/ref_nm_n<N>_m<M> by
    oracle/ref_build.py) on the same matrix, schedule by schedule, as
    find_best_2toX (main.cu:72-114) runs them: wall seconds per schedule
    and the result integers."""
    import tempfile
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ref_build
    from vnm_gb300 import synth
    try:
        exe = ref_build.ensure("ref_nm_n%d_m%d" % (N, M))
    except Exception as e:
        return {"unavailable": "%s: %s" % (type(e).__name__, e)}
    out = {"what": "the reference's own GPU find_best_2toX schedules (reorder/reorder.h, main.cu:72-114), built "
                   "from its sources for sm_103a; includes each run's file read and CUDA set-up, as the "
                   "reference's command does", "seconds": {}, "res5": {}}
    with tempfile.TemporaryDirectory() as td:
        mtx = os.path.join(td, "in.mtx")
        synth.write_mtx(mtx, nr, r, c, v)
        for sch in range(4):
            o = os.path.join(td, "res%d.txt" % sch)
            t0 = time.perf_counter()
            try:
                p = subprocess.run([exe, mtx, str(sch), o], capture_output=True, text=True, timeout=timeout)
                out["seconds"][sch] = time.perf_counter() - t0
                if p.returncode == 0:
                    with open(o) as f:
                        out["res5"][sch] = [int(x) for x in f.readline().split()[2:7]]
                else:
                    out["res5"][sch] = "rc %d" % p.returncode
            except subprocess.TimeoutExpired:
                out["seconds"][sch] = None
                out["res5"][sch] = "timeout after %.0f s" % timeout
    secs = [x for x in out["seconds"].values() if x is not None]
    out["total_seconds"] = sum(secs) if len(secs) == 4 else None
    return out


def vnm_stage_port(nr, r, c, v):
    """The CPU port of reordering.py (the oracle's restatement) on the same
    matrix at M=8, V=64, one thread: seconds per VNM round.  (At the step's
    2:4 a segment has 4 columns, so no V-block can be invalid and the stage
    does no round.)"""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(1)
    t0 = time.perf_counter()
    out5, _, _, _ = oracle.vnm_run(nr, nr, r, c, 8, V, 10)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "rounds": int(out5[4]), "seconds_per_round": dt / max(1, int(out5[4])),
            "out5": out5.tolist(), "cores": 1, "kind": "port",
            "what": "C++ restatement of reordering.py (M=8, V=64) on the R-MAT 16384 matrix"}


def run_reference(args, rank, world):
    """CPU port of the reference path, on the host cores, rank 0 only.  The
    line also carries the reference's own GPU reorder on the same matrix
    (reference_gpu), the port on one thread, and the VNM-stage port."""
    if rank != 0:
        return
    nr, r, c, v = workload(0)
    B64 = np.random.default_rng(1234).standard_normal((nr, N_B))
    threads = host_threads()
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_port_step(nr, r, c, v, B64, threads)
    times = []
    for _ in range(args.steps):
        dt, best = cpu_port_step(nr, r, c, v, B64, threads)
        times.append(dt)
    tot = sum(times)
    value = args.steps / tot
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "hot-path steps/s", "value_is": VALUE_IS,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32 (reorder), fp64 (SpMM)",
        "data": "synthetic (seeded R-MAT)",
        "config": {"workload": WORKLOAD, "nrows": nr, "nnz": int(len(r)), "N": N_NM, "M": M_NM, "V": V,
                   "n_B": N_B, "schedules": 4, "l2": "n/a (CPU)", "best_sched": int(best)},
        "cpu_baseline": {"value": value, "unit": "hot-path steps/s", "cores": threads, "kind": "port",
                         "sample": "full step per measurement: find_best_2toX + the winner's run (C++ "
                                   "restatement of reorder/reorder.h + main.cu, OpenMP) + FP64 SpMM"},
        "e2e": {"value": value, "unit": "hot-path steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_extended:
        line["cpu_baseline"]["one_thread"] = {
            "seconds_one_schedule": cpu_port_one_schedule(nr, r, c, v, int(best), 1), "cores": 1,
            "sample": "schedule %d of find_best_2toX on one thread" % int(best)}
        line["vnm_stage_port"] = vnm_stage_port(nr, r, c, v)
        line["reference_gpu"] = reference_gpu(nr, r, c, v)
        from vnm_gb300 import synth
        n1, r1, c1, v1 = synth.uniform_c1(0)
        line["reference_gpu_c1"] = dict(reference_gpu(n1, r1, c1, v1, 2, 8), workload=C1_WORKLOAD)
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
    g = torch.Generator().manual_seed(1234 + rank)
    Bh = torch.randn((nr, N_B), generator=g).to(torch.bfloat16)
    tr = torch.from_numpy(r).to(dev)
    tc = torch.from_numpy(c).to(dev)
    tv = torch.from_numpy(v).to(dev)
    tB = Bh.to(dev)
    tC = torch.empty((nr, N_B), dtype=torch.float32, device=dev)
    # pinned host copies for the end-to-end measurement
    hr = torch.from_numpy(r).pin_memory()
    hc = torch.from_numpy(c).pin_memory()
    hv = torch.from_numpy(v).pin_memory()
    hB = Bh.view(torch.int16).pin_memory()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def step_device():
        """One pass of the hot path, inputs in HBM: schedule search, the
        winner's relabelling, V:N:M compression, SpMM.  Returns timings."""
        flush.zero_()
        torch.cuda.synchronize()
        t = {}
        best, res, newpos = ctx.nm_search(nr, tr, tc, tv, N_NM, M_NM, want_newpos=True)
        t["reorder_ms"] = ctx.last_kernel_ms
        t["rounds_kernel_ms"] = ctx.last_main_kernel_ms
        t["launches"] = ctx.last_launch_count
        t["stats"] = ctx.last_stats()
        pr, pc = tr.clone(), tc.clone()
        ctx.permute_coo(nr, pr, pc, torch.from_numpy(newpos).to(dev))
        t["permute_ms"] = ctx.last_kernel_ms
        t["launches"] += ctx.last_launch_count
        A = vnm_gb300.SpmmMatrix(ctx, nr, pr, pc, tv, M_NM, V, "bf16")
        t["compress_ms"] = ctx.last_kernel_ms
        t["launches"] += ctx.last_launch_count
        A.run(tB, tC)
        t["spmm_call_ms"] = ctx.last_kernel_ms
        t["spmm_kernel_ms"] = ctx.last_main_kernel_ms
        t["launches"] += ctx.last_launch_count
        t["info"] = A.info()
        t["best"] = best
        t["res4"] = res
        t["newpos"] = newpos
        A.close()
        return t

    # pinned host buffers of the pass through the public API, made once as a
    # caller running many steps would: the relabelled COO and the result
    hpr = torch.empty(len(r), dtype=torch.int32).pin_memory()
    hpc = torch.empty(len(c), dtype=torch.int32).pin_memory()
    hC = torch.empty((nr, N_B), dtype=torch.float32).pin_memory()

    def step_host():
        """The same pass through the public API with host buffers."""
        best, res, newpos = ctx.nm_search(nr, hr.numpy(), hc.numpy(), hv.numpy(), N_NM, M_NM, want_newpos=True)
        pr, pc = ctx.permute_coo(nr, hr.numpy(), hc.numpy(), newpos, out=(hpr.numpy(), hpc.numpy()))
        A = vnm_gb300.SpmmMatrix(ctx, nr, pr, pc, hv.numpy(), M_NM, V, "bf16")
        C = A.run(hB.numpy(), C=hC.numpy())
        A.close()
        return C

    for _ in range(args.warmup):
        t = step_device()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    tot = {"reorder_ms": 0.0, "rounds_kernel_ms": 0.0, "permute_ms": 0.0, "compress_ms": 0.0,
           "spmm_call_ms": 0.0, "spmm_kernel_ms": 0.0}
    launches, wall = 0, 0.0
    stats_sum = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        t = step_device()
        wall += time.perf_counter() - t0
        for k in tot:
            tot[k] += t[k]
        launches += t["launches"]
        st = {k: x for k, x in t["stats"].items() if not isinstance(x, dict)}
        stats_sum = st if stats_sum is None else {k: stats_sum[k] + st[k] for k in st}
    barrier()
    clk = clocks.stop()
    # where a round's time goes: one more step with the round kernel's phase
    # timers on (outside the timed region; the timers cost ~2.5 % of the kernel)
    ctx.set_phase_timing(True)
    tph = step_device()
    ctx.set_phase_timing(False)
    phase_sum, phase_kus = tph["stats"]["phase_us"], tph["stats"].get("kernel_us", 0)
    info, best = t["info"], t["best"]
    step_ms = (tot["reorder_ms"] + tot["permute_ms"] + tot["compress_ms"] + tot["spmm_call_ms"]) / args.steps
    elapsed = step_ms * args.steps / 1000.0
    value, elapsed = whole_job_rate(elapsed, args.steps, world, dev)
    # end to end through the public API with pinned host buffers
    step_host()
    barrier()
    e2e_t = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        C = step_host()
        e2e_t += time.perf_counter() - t0
    barrier()
    e2e_value, e2e_t = whole_job_rate(e2e_t, args.steps, world, dev)
    nnz = len(r)
    h2d = 12 * nnz + 8 * nnz + 4 * nr + 12 * nnz + 2 * nr * N_B
    d2h = 4 * 20 + 4 + 4 * nr + 8 * nnz + 4 * nr * N_B
    newpos = t["newpos"]
    # SpMM accuracy against the FP64 oracle (outside the timed region)
    spmm_err = spmm_err_norm = None
    if rank == 0:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        rr, cc = newpos[r], newpos[c]
        ref = oracle.spmm_f64(nr, rr, cc, v.astype(np.float64), Bh.float().numpy().astype(np.float64))
        spmm_err = oracle.rowwise_rel_err(C, ref)
        spmm_err_norm = float(np.abs(C.astype(np.float64) - ref).max() / np.abs(ref).max())
        del ref
    # roofline of the persistent reorder kernel.  Algorithmic bytes per round
    # of the scorer (the byte model of the workload table): the CSR pattern
    # read once, 4 (R + 1) + 4 nnz, plus the (row, segment) group bitmap
    # written and read, 2 B per nonzero group; the scored-pair term (8 M^2 B
    # per pair) is left out, so this is a lower bound on the bytes.  The
    # kernel's own work counters (entries gathered, rows touched) give the
    # second, incremental figure.
    stt = stats_sum
    groups = nonzero_groups(nr, r, c, v, M_NM)
    bytes_per_round = 4.0 * (nr + 1) + 4.0 * stt["pattern_nnz"] / max(1, args.steps) + 2.0 * groups
    alg_bytes = stt["rounds"] * bytes_per_round
    inc_bytes = (4.0 * stt["rounds"] * stt["nseg"] / max(1, args.steps) + 20.0 * stt["gathered"] +
                 32.0 * stt["touched"])
    peak, peak_kind = load_peaks()
    kt = tot["rounds_kernel_ms"] / 1000.0
    achieved = alg_bytes / kt / 1e9 if kt > 0 else 0.0
    tflops_peak, tkind = load_tensor_peak()
    issued = 2.0 * 128 * 16 * N_B * info["ksteps"]
    useful = 2.0 * nnz * N_B
    sk = tot["spmm_kernel_ms"] / args.steps / 1000.0
    spmm_bytes = spmm_hbm_bytes(nr, nnz, N_B)
    # parity at this size: the GPU search against the oracle's committed
    # results (all four schedules' result integers, the winner and its
    # permutation), the input checked by its SHA-256 first
    parity = {}
    gold = scale_golden("c2")
    if gold is not None and rank == 0:
        same_input = coo_digest(nr, r, c, v) == gold["sha256"]
        parity["c2_vs_oracle_goldens"] = bool(same_input and np.array_equal(t["res4"], gold["res5x4"]) and
                                              best == gold["best"] and
                                              np.array_equal(newpos, gold["newpos4"][gold["best"]]))
    out = {
        "metric": METRIC, "value": value, "unit": "hot-path steps/s", "value_is": VALUE_IS, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32 (reorder), bf16 x bf16 -> fp32 (SpMM)",
        "data": "synthetic (seeded R-MAT, seed = rank; B ~ N(0,1))",
        "config": {"workload": WORKLOAD, "nrows": nr, "nnz": nnz, "N": N_NM, "M": M_NM, "V": V, "n_B": N_B,
                   "schedules": 4, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed (256 MB write) before every step", "best_sched": int(best),
                   "rounds_per_search": int(stt["rounds"] // args.steps),
                   "blocks_per_job": int(t["stats"]["blocks_per_job"])},
        "breakdown_ms": {"reorder_search": tot["reorder_ms"] / args.steps, "permute": tot["permute_ms"] / args.steps,
                         "compress": tot["compress_ms"] / args.steps, "spmm_call": tot["spmm_call_ms"] / args.steps,
                         "spmm_kernel": tot["spmm_kernel_ms"] / args.steps},
        "e2e": {"value": e2e_value, "unit": "hot-path steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1000.0 * e2e_t / args.steps},
        "roofline": {"kernel": "k_nm_rounds<4>", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "bytes_model": "per round 4(R+1) + 4 nnz (CSR pattern) + 2 B per nonzero (row, segment) "
                                    "group; %d groups" % groups,
                     # dram__bytes_read.sum + dram__bytes_write.sum of one launch, from the ncu
                     # capture summarised in profiles/k_nm_rounds_c2_rmat16384_m4.md
                     "traffic": 1.079e6, "traffic_unit": "bytes per launch",
                     "traffic_source": "profiles/k_nm_rounds_c2_rmat16384_m4.md",
                     "alg_bytes_per_launch": alg_bytes / args.steps,
                     "kernel_ms_per_launch": tot["rounds_kernel_ms"] / args.steps,
                     # the launch's time over the mean rounds of its (concurrent) jobs
                     "us_per_round": 1000.0 * tot["rounds_kernel_ms"] / max(1.0, stt["rounds"] / max(1, stt["jobs"])) /
                     max(1, args.steps),
                     "incremental_bytes_per_launch": inc_bytes / args.steps,
                     "incremental_frac": inc_bytes / kt / 1e9 / peak if kt > 0 else 0.0,
                     "note": "latency-bound sequential greedy (4 jobs x cluster of %d blocks); see profiles/"
                             % int(t["stats"]["blocks_per_job"]),
                     # shares of the leaders' time from the kernel's start to its end, from
                     # one extra step with the phase timers on (its kernel time beside)
                     "round_phase_share": dict({k: round(vv / max(1, phase_kus, sum(phase_sum.values())), 4)
                                                for k, vv in phase_sum.items()},
                                               outside_rounds=round(max(0, phase_kus - sum(phase_sum.values())) /
                                                                    max(1, phase_kus), 4)),
                     "phase_timed_kernel_ms": tph["rounds_kernel_ms"]},
        "spmm": {"kernel": ("k_spmm_vnm<64|128|256> (column-block width picked by timing on the first call) + "
                            "k_spmm_res" if info["tensor_tiles"] > 0 else "k_spmm_res + k_spmm_fin (CUDA cores)"),
                 "routing": "%d tensor-core tiles; %d residual nonzeros on the CUDA cores (V-blocks with fewer "
                            "than dense_min = %d nonzeros)" % (info["tensor_tiles"], info["residual_nnz"],
                                                               info["dense_min"]),
                 "useful_tflops": useful / sk / 1e12,
                 "issued_tflops": issued / sk / 1e12,
                 "bound": "tensor" if info["tensor_tiles"] > 0 else "hbm (gathered B rows)",
                 "peak_tflops": tflops_peak,
                 "peak_kind": tkind, "issued_frac": issued / sk / 1e12 / tflops_peak,
                 "hbm": {"alg_bytes": spmm_bytes, "achieved_gbs": spmm_bytes / sk / 1e9, "peak": peak,
                         "frac": spmm_bytes / sk / 1e9 / peak, "peak_kind": peak_kind,
                         "bytes_model": "A as CSR (2 B value + 4 B column per nonzero, row pointers), B read "
                                        "once, C (fp32) written once"},
                 "max_rel_err_vs_fp64_per_row": spmm_err, "max_rel_err_vs_fp64_normwise": spmm_err_norm,
                 "slices": info["slices"], "ksteps": info["ksteps"],
                 "blocks": info["blocks"], "valid_blocks": info["valid_blocks"]},
        "parity": parity,
        "gpu_launches": launches,
        "clocks": clk,
        "wall_ms_per_step": 1000.0 * wall / args.steps,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = host_threads()
        dt, cbest, ores = cpu_port_find_best(nr, r, c, v, threads)
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "hot-path steps/s", "cores": threads, "kind": "port",
                               "sample": "one full find_best_2toX of the same matrix (C++ restatement of the "
                                         "reference NM path, OpenMP); the SpMM part is not included",
                               "best_sched": int(cbest)}
        # the same port on one thread, on a bounded sample: the winning
        # schedule alone (a quarter of find_best_2toX)
        dt1 = cpu_port_one_schedule(nr, r, c, v, int(cbest), 1)
        out["cpu_baseline"]["one_thread"] = {"seconds_one_schedule": dt1, "cores": 1,
                                             "sample": "schedule %d of find_best_2toX on one thread" % int(cbest)}
        # live parity against the oracle run here: all four schedules' result
        # integers, the winner, and the winner's permutation
        _, _, _, opos = oracle_nm_run(nr, r, c, v, int(cbest))
        parity["c2_vs_oracle_live"] = bool(cbest == best and np.array_equal(ores, t["res4"]) and
                                           np.array_equal(opos, newpos))
        out["cpu_baseline_agrees"] = parity["c2_vs_oracle_live"]
    if rank == 0 and world == 1 and not args.no_extended:
        try:
            out["baselines_c2_spmm"] = library_spmm_baselines(nr, newpos[r], newpos[c], v, N_B, torch.bfloat16)
            ours = tot["spmm_kernel_ms"] / args.steps
            for k, d in out["baselines_c2_spmm"].items():
                if "ms" in d:
                    d["vnm_kernel_speedup"] = d["ms"] / ours
        except Exception as e:
            out["baselines_c2_spmm"] = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0 and world == 1 and not args.no_extended:
        # the other configurations, untimed by the headline (one GPU, after it)
        for key, fn in (("c1_plain_small", bench_plain_c1), ("vnm_stage_c2", bench_vnm_stage), ("c3_batch", bench_batch_c3),
                        ("c4_learned", bench_learned_c4), ("c5_gcn", bench_gcn_c5),
                        ("s1_structured_spmm", bench_structured_spmm)):
            try:
                out[key] = fn(ctx)
            except Exception as e:  # report, keep the headline line
                out[key] = {"error": "%s: %s" % (type(e).__name__, e)}
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def _median(xs):
    return float(np.median(np.asarray(xs, np.float64)))


def bench_batch_c3(ctx, reps=3):
    """256 R-MAT matrices (rows log-uniform in [256, 8192], degree U[4, 32]),
    2:8, schedule 0: one persistent launch against one call per matrix."""
    import vnm_gb300
    from vnm_gb300 import synth
    M = 8
    mats = []
    for n, r, c, v in synth.rmat_batch(256):
        mats.append(((n + M - 1) // M * M, r, c, v))
    nnz = sum(len(m[1]) for m in mats)
    # the matrices as the C call takes them (packed once, as a caller that
    # reorders the same batch layout repeatedly holds them)
    import torch
    nr_, off_, r_, c_, v_ = ctx.pack_batch(mats)
    packed = (nr_, off_) + tuple(torch.from_numpy(x).pin_memory().numpy() for x in (r_, c_, v_))  # pinned
    ctx.nm_reorder_batch(packed, 2, M, 0)  # warm-up
    bt, bw = [], []
    for _ in range(reps):
        t0 = time.perf_counter()
        res_b, pos_b = ctx.nm_reorder_batch(packed, 2, M, 0)
        bw.append(1000.0 * (time.perf_counter() - t0))
        bt.append(ctx.last_kernel_ms)
    loop_ms, loop_wall, same = 0.0, 0.0, True
    for b, (n, r, c, v) in enumerate(mats):
        t0 = time.perf_counter()
        res, pos = ctx.nm_reorder(n, r, c, v, 2, M, 0)
        loop_wall += 1000.0 * (time.perf_counter() - t0)
        loop_ms += ctx.last_kernel_ms
        same = same and np.array_equal(res, res_b[b]) and np.array_equal(pos, pos_b[b])
    # three members (the smallest, a middle one, the largest) against the
    # oracle run here, outside the timed runs
    sizes = np.array([m[0] for m in mats])
    order = np.argsort(sizes, kind="stable")
    checked = {}
    for b in (int(order[0]), int(order[len(order) // 2]), int(order[-1])):
        n, r, c, v = mats[b]
        ores, _, _, opos = oracle_nm_run(n, r, c, v, 0, N=2, M=M)
        checked[str(b)] = {"nrows": int(n), "same_as_oracle": bool(np.array_equal(res_b[b], ores) and
                                                                   np.array_equal(pos_b[b], opos))}
    return {"workload": "C3: 256 R-MAT matrices, rows log-uniform [256, 8192], degree U[4,32], U[-1,1], 2:8, "
                        "schedule 0, nm_maxiter 10",
            "members_vs_oracle": checked,
            "parity_members_vs_oracle": all(x["same_as_oracle"] for x in checked.values()),
            "matrices": len(mats), "nnz_total": int(nnz), "rows_total": int(sum(m[0] for m in mats)),
            "batched_device_ms": _median(bt), "batched_wall_ms": _median(bw),
            "per_matrix_device_ms_sum": loop_ms, "per_matrix_wall_ms_sum": loop_wall,
            "speedup_wall": loop_wall / _median(bw), "bit_exact_vs_per_matrix": bool(same),
            "launches": "one persistent launch (a two-block cluster per matrix)",
            "host_inputs": "packed once into pinned arrays (8.6 M entries); the per-matrix calls take each "
                           "matrix's own arrays"}


def bench_learned_c4(ctx, reps=3):
    """Learned-proposal reorder against the plain exact reorder on R-MAT
    65536 (degree 32), 2:8: wall time to the plain reorder's retained-nnz."""
    import vnm_gb300
    from vnm_gb300 import learned, synth
    N, M = 2, 8
    n, r, c, v = synth.rmat_c4(0)
    net = learned.load(ctx, N, M)
    t0 = time.perf_counter()
    best, res4, newpos = ctx.nm_search(n, r, c, v, N, M)
    plain_wall = 1000.0 * (time.perf_counter() - t0)
    plain_dev = ctx.last_kernel_ms
    base, _, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=vnm_gb300.LEARNED_RANDOM, max_rounds=0)
    ret0 = base["init_retained"]
    # retained nonzeros of the plain result, counted by the library itself:
    # zero learned rounds on the permuted matrix report its totals
    pr, pc = ctx.permute_coo(n, r, c, newpos)
    o = np.lexsort((pc, pr))
    pl, _, _ = vnm_gb300.nm_learned(ctx, n, pr[o], pc[o], v[o], N, M, mode=vnm_gb300.LEARNED_RANDOM, max_rounds=0)
    target = pl["init_retained"] - ret0
    gold = scale_golden("c4")
    parity = None
    if gold is not None:
        parity = bool(coo_digest(n, r, c, v) == gold["sha256"] and np.array_equal(res4, gold["res5x4"]) and
                      best == gold["best"] and np.array_equal(newpos, gold["newpos4"][gold["best"]]))
    out = {"workload": "C4: R-MAT 65536x65536, 1048576 edges symmetrised (%d entries), N(0,1), 2:8" % len(r),
           "plain": {"what": "find_best_2toX, 4 schedules, bit-exact with the reference", "wall_ms": plain_wall,
                     "device_ms": plain_dev, "best_sched": int(best), "retained": int(pl["init_retained"]),
                     "invalid_groups": int(pl["init_invalid"]), "retained_gain": int(target)},
           "parity_plain_vs_oracle_goldens": parity,
           "init_retained": int(ret0)}
    modes = (("network_top8", vnm_gb300.LEARNED_MLP, 8), ("network_top1", vnm_gb300.LEARNED_MLP, 1),
             ("random_top8", vnm_gb300.LEARNED_RANDOM, 8), ("exhaustive", vnm_gb300.LEARNED_EXHAUSTIVE, 8))
    for name, mode, topk in modes:
        row = {}
        for label, stop in (("to_plain", target), ("converged", 0)):
            walls, devs = [], []
            for _ in range(reps):
                t0 = time.perf_counter()
                res, pos, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=mode,
                                                   net=net if mode == vnm_gb300.LEARNED_MLP else None, topk=topk,
                                                   targets=TARGETS, max_rounds=64, patience=3, seed=1, stop_gain=stop)
                walls.append(1000.0 * (time.perf_counter() - t0))
                devs.append(ctx.last_kernel_ms)
            row[label] = {"wall_ms": _median(walls), "device_ms": _median(devs), "rounds": res["rounds"],
                          "retained": int(res["final_retained"]), "retained_gain": int(res["gain"]),
                          "reached_plain": bool(res["gain"] >= target), "exact_scored": int(res["exact_scored"])}
        out[name] = row
    lw = out["network_top8"]["to_plain"]["wall_ms"]
    out["speedup_to_equal_retained_wall"] = plain_wall / lw
    # the same two calls with the COO already in HBM (device arrays): the
    # reorders alone, without the host-to-device copy of the matrix
    import torch
    dr, dc, dv = (torch.from_numpy(x).cuda() for x in (r, c, v))
    torch.cuda.synchronize()
    dev_plain, dev_net = [], []
    for _ in range(reps):
        ctx.nm_search(n, dr, dc, dv, N, M, want_newpos=False)
        dev_plain.append(ctx.last_kernel_ms)
        vnm_gb300.nm_learned(ctx, n, dr, dc, dv, N, M, mode=vnm_gb300.LEARNED_MLP, net=net, topk=8, targets=TARGETS,
                             max_rounds=64, patience=3, seed=1, stop_gain=target, want_newpos=False)
        dev_net.append(ctx.last_kernel_ms)
    out["inputs_in_hbm"] = {"plain_device_ms": _median(dev_plain), "network_top8_to_plain_device_ms": _median(dev_net),
                            "speedup": _median(dev_plain) / _median(dev_net)}
    out["retained_converged_vs_plain"] = out["network_top8"]["converged"]["retained"] / max(1, pl["init_retained"])
    # the V:N:M retained-nnz at V=128 (per V-block and segment the 4 columns
    # with the most nonzeros kept, then per row at most N of them), counted
    # by the oracle on the input, the plain result and the learned result
    res, pos, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=vnm_gb300.LEARNED_MLP, net=net, topk=8,
                                       targets=TARGETS, max_rounds=64, patience=3, seed=1)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    Vc = 128
    out["vnm_retained_v128"] = {"input": int(oracle.retained_vnm(n, r, c, v, N, M, Vc)),
                                "plain": int(oracle.retained_vnm(n, newpos[r], newpos[c], v, N, M, Vc)),
                                "network_top8_converged": int(oracle.retained_vnm(n, pos[r], pos[c], v, N, M, Vc)),
                                "nnz": int(len(r))}
    out["hybrid_maxiter30"] = hybrid_cli(n, r, c, v, N, M, Vc, 30)
    X = np.random.default_rng(0).normal(0, 1, (1 << 20, 32)).astype(np.float32)
    ms = []
    for _ in range(4):
        net.forward(X)
        ms.append(ctx.last_main_kernel_ms)
    fl = (1 << 20) * 2.0 * (32 * 128 + 128 * 128)
    tpk, tkind = load_tensor_peak()
    out["mlp_inference"] = {"kernel": "k_l_mlp (tcgen05, plain rows)", "rows": 1 << 20,
                            "ms": _median(ms[1:]), "tflops": fl / _median(ms[1:]) / 1e9,
                            "frac_of_bf16_peak": fl / _median(ms[1:]) / 1e9 / tpk, "peak_kind": tkind}
    net.close()
    return out


def bench_vnm_stage(ctx, reps=5):
    """The VNM stage (reordering.py --m 8 --v 64) on the R-MAT 16384 matrix
    on the GPU, against the reference script's own run of it (a committed
    fixture made where the script runs: its result and its seconds on that
    machine's one core) and the oracle's port on one host core."""
    from vnm_gb300 import synth
    nr, r, c, v = synth.rmat_c2(0)
    ms, out5 = [], None
    for _ in range(reps):
        t0 = time.perf_counter()
        out5, _, _, _ = ctx.vnm_reorder(nr, nr, r, c, 8, 64, maxiter=10)
        ms.append(1000.0 * (time.perf_counter() - t0))
    out = {"workload": "R-MAT 16384 (C2 matrix), VNM stage at M=8, V=64, maxiter 10", "wall_ms": _median(ms),
           "device_ms": ctx.last_kernel_ms, "out5": out5.tolist()}
    p = os.path.join(GOLD, "scale_vnm_c2.npz")
    if os.path.exists(p):
        g = np.load(p)
        out["same_as_reordering_py"] = out5.tolist() == g["out5"].tolist()
        out["reordering_py_seconds_1core"] = float(g["seconds"])
        out["reordering_py_note"] = "measured where the reference checkout is (x86 host), not on this machine"
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.set_threads(1)
    t0 = time.perf_counter()
    o5, _, _, _ = oracle.vnm_run(nr, nr, r, c, 8, 64, 10)
    out["port_1core_ms"] = 1000.0 * (time.perf_counter() - t0)
    out["same_as_port"] = o5.tolist() == out5.tolist()
    return out


C1_WORKLOAD = "C1: uniform 512x512, ~2 % density (seed 0), U[-1,1]; 2:8, V=64, maxiter 10, schedule 0"


def bench_plain_c1(ctx, reps=3):
    """C1 through the drop-in `spmm` command (find_best_2toX, then 10 rounds
    of the VNM stage and the NM reorder): process wall time, the CSV line's
    counts, the retained-nnz of the written matrix, and the same command
    composed by the oracle on one host thread, whose 15 CSV fields and
    output text must match."""
    import tempfile
    from vnm_gb300 import synth
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    N, M, Vc, maxiter = 2, 8, 64, 10
    n, r, c, v = synth.uniform_c1(0)
    exe = os.path.join(PKG, "spmm")
    with tempfile.TemporaryDirectory() as td:
        mtx, out = os.path.join(td, "c1.mtx"), os.path.join(td, "out.mtx")
        synth.write_mtx(mtx, n, r, c, v)
        walls = []
        for _ in range(reps):
            t0 = time.perf_counter()
            p = subprocess.run([exe, "--mtxfile", mtx, "--outmtxfile", out, "--maxiter", str(maxiter), "--n", "64",
                                "--sched", "0", "--v", str(Vc), "--N", str(N), "--M", str(M)],
                               cwd=td, capture_output=True, text=True, timeout=600)
            walls.append(time.perf_counter() - t0)
            if p.returncode != 0:
                return {"error": p.stderr[-500:]}
        f = [float(x) for x in p.stdout.strip().split(",")]
        with open(out) as fh:
            text = fh.read()
        oracle.set_threads(1)
        t0 = time.perf_counter()
        csv, best, onr, orr, occ, ovv = oracle.spmm_cli(mtx, N, M, Vc, maxiter)
        ot = time.perf_counter() - t0
        oracle.set_threads(oracle.max_threads())
        op = os.path.join(td, "oracle_out.mtx")
        oracle.write_mtx(op, onr, onr, orr, occ, ovv)
        with open(op) as fh:
            otext = fh.read()
    same = bool(np.allclose(f[:15], csv[:15], rtol=1e-5, atol=1e-6)) and text == otext
    return {"workload": C1_WORKLOAD, "nnz": int(len(r)), "process_wall_ms": 1000.0 * _median(walls),
            "hybrid_ms": f[15], "best_sched": int(best), "init_cnt": f[5], "final_cnt": f[6],
            "init_vblocks": f[8], "final_vblocks": f[9], "nm_rounds": f[12], "vnm_rounds": f[13],
            "retained_nm": int(oracle.retained_nm(onr, orr, occ, ovv, N, M)),
            "retained_vnm": int(oracle.retained_vnm(onr, orr, occ, ovv, N, M, Vc)),
            "csv_and_output_match_oracle": same,
            "oracle_one_thread": {"seconds": ot, "cores": 1, "kind": "port",
                                  "what": "the oracle's composition of the spmm command (orc_spmm_cli)"}}


def hybrid_cli(n, r, c, v, N, M, Vc, maxiter):
    """The drop-in `spmm` command (find_best_2toX, then maxiter rounds of the
    VNM stage and the NM reorder, main.cu:195-337) on a matrix written as a
    Matrix Market file: its own CSV line (field 16 is the hybrid loop's
    milliseconds, timed as the reference times it) and the process's wall
    time including the file read and write."""
    import tempfile
    from vnm_gb300 import synth
    exe = os.path.join(PKG, "spmm")
    with tempfile.TemporaryDirectory() as td:
        mtx = os.path.join(td, "in.mtx")
        synth.write_mtx(mtx, n, r, c, v)
        t0 = time.perf_counter()
        p = subprocess.run([exe, "--mtxfile", mtx, "--outmtxfile", os.path.join(td, "out.mtx"), "--maxiter",
                            str(maxiter), "--n", "64", "--sched", "0", "--v", str(Vc), "--N", str(N), "--M", str(M)],
                           cwd=td, capture_output=True, text=True, timeout=1200)
        wall = time.perf_counter() - t0
    if p.returncode != 0:
        return {"error": p.stderr[-500:]}
    f = [float(x) for x in p.stdout.strip().split(",")]
    return {"what": "spmm command, --maxiter %d --v %d, %d:%d" % (maxiter, Vc, N, M), "hybrid_ms": f[15],
            "process_wall_s": wall, "init_cnt": f[5], "final_cnt": f[6], "init_vblocks": f[8], "final_vblocks": f[9],
            "nm_rounds": f[12], "vnm_rounds": f[13]}


def bench_gcn_c5(ctx, reps=100):
    """Chung-Lu 262144 nodes (exponent 2.1, mean degree 20), symmetric-
    normalised weights: learned reorder at 2:8, V:N:M compress (V=128), and
    100 SpMMs with X 262144x256 in BF16 and in FP16."""
    import torch
    import vnm_gb300
    from vnm_gb300 import learned, synth
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    N, M, Vc, nB = 2, 8, 128, 256
    n, r, c, v = synth.chung_lu_c5(0)
    net = learned.load(ctx, N, M)
    t0 = time.perf_counter()
    res, newpos, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=vnm_gb300.LEARNED_MLP, net=net, topk=8,
                                          targets=TARGETS, max_rounds=64, patience=3, seed=1)
    reorder_wall = 1000.0 * (time.perf_counter() - t0)
    reorder_dev = ctx.last_kernel_ms
    # the same search with random proposals and with every candidate scored
    # exactly, to convergence: what the network buys on this graph
    modes = {"network_top8": {"wall_ms": reorder_wall, "device_ms": reorder_dev, "rounds": res["rounds"],
                              "final_invalid": int(res["final_invalid"]),
                              "final_retained": int(res["final_retained"]),
                              "exact_scored": int(res["exact_scored"])}}
    for name, mode in (("random_top8", vnm_gb300.LEARNED_RANDOM), ("exhaustive", vnm_gb300.LEARNED_EXHAUSTIVE)):
        t1 = time.perf_counter()
        rm, _, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=mode, topk=8, targets=TARGETS, max_rounds=64,
                                        patience=3, seed=1, want_newpos=False)
        modes[name] = {"wall_ms": 1000.0 * (time.perf_counter() - t1), "device_ms": ctx.last_kernel_ms,
                       "rounds": rm["rounds"], "final_invalid": int(rm["final_invalid"]),
                       "final_retained": int(rm["final_retained"]), "exact_scored": int(rm["exact_scored"])}
    net.close()
    pr, pc = ctx.permute_coo(n, r, c, newpos)
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator().manual_seed(7)
    X32 = torch.randn((n, nB), generator=g)
    tr, tc, tv = (torch.from_numpy(x).to(dev) for x in (pr, pc, v))
    out = {"workload": "C5: Chung-Lu 262144 nodes, exponent 2.1, mean degree 20 (%d entries), D^-1/2 A D^-1/2, "
                       "2:8, V=128, X 262144x256 N(0,1)" % len(r),
           "reorder": {"mode": "network top8", "wall_ms": reorder_wall, "device_ms": reorder_dev,
                       "rounds": res["rounds"], "init_retained": int(res["init_retained"]),
                       "final_retained": int(res["final_retained"]), "init_invalid": int(res["init_invalid"]),
                       "final_invalid": int(res["final_invalid"])},
           "reorder_modes_converged": modes}
    for dt, tdt in (("bf16", torch.bfloat16), ("fp16", torch.float16)):
        A = vnm_gb300.SpmmMatrix(ctx, n, tr, tc, tv, M, Vc, dt)
        comp_ms = ctx.last_kernel_ms
        info = A.info()
        Xd = X32.to(tdt).to(dev)
        C = torch.empty((n, nB), dtype=torch.float32, device=dev)
        A.run(Xd, C)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kms = 0.0
        e0.record()
        for _ in range(reps):
            A.run(Xd, C)
            kms += ctx.last_main_kernel_ms
        e1.record()
        torch.cuda.synchronize()
        total_ms = e0.elapsed_time(e1)
        # error against the FP64 oracle on the same (rounded) X
        ref = oracle.spmm_f64(n, pr, pc, v.astype(np.float64), X32.to(tdt).float().numpy().astype(np.float64))
        Ch = C.cpu().numpy().astype(np.float64)
        err = oracle.rowwise_rel_err(Ch, ref)
        err_norm = float(np.abs(Ch - ref).max() / np.abs(ref).max())
        del ref
        useful = 2.0 * len(r) * nB
        issued = 2.0 * 128 * 16 * nB * info["ksteps"]
        sk = kms / reps / 1000.0
        tpk, tkind = load_tensor_peak(sustained=True)  # 100 calls back to back: about half a second
        hpk, hkind = load_peaks()
        hb = spmm_hbm_bytes(n, len(r), nB)
        out["spmm_" + dt] = {"runs": reps, "total_ms": total_ms, "kernel_ms_per_run": kms / reps,
                             "compress_ms": comp_ms, "useful_tflops": useful / sk / 1e12,
                             "issued_tflops": issued / sk / 1e12, "issued_frac": issued / sk / 1e12 / tpk,
                             "peak_kind": tkind,
                             "hbm": {"alg_bytes": hb, "achieved_gbs": hb / sk / 1e9, "frac": hb / sk / 1e9 / hpk,
                                     "peak": hpk, "peak_kind": hkind},
                             "max_rel_err_vs_fp64_per_row": err,
                             "max_rel_err_vs_fp64_normwise": err_norm, "ksteps": info["ksteps"],
                             "slices": info["slices"], "valid_blocks": info["valid_blocks"]}
        A.close()
    try:
        out["baselines_spmm"] = library_spmm_baselines(n, pr, pc, v, nB, torch.bfloat16, dense=False)
        ours = out["spmm_bf16"]["kernel_ms_per_run"]
        for k, d in out["baselines_spmm"].items():
            if "ms" in d:
                d["vnm_kernel_speedup"] = d["ms"] / ours
    except Exception as e:
        out["baselines_spmm"] = {"error": "%s: %s" % (type(e).__name__, e)}
    return out


def bench_structured_spmm(ctx, reps=20):
    """The operand V:N:M is made for: a 19456 x 19456 matrix (152 row tiles
    of 128, one per SM) already in full V:2:8 form with V=128 (density 1/4,
    94.6 M nonzeros), times B 19456 x 256 BF16 -- all on the tensor cores.
    Beside it: the same product on the CUDA-core residual path, cuSPARSE CSR
    and a dense cuBLAS GEMM of the densified matrix.  Error per row against
    float64 on 1024 sampled rows."""
    import torch
    import vnm_gb300
    from vnm_gb300 import synth
    R, M, Vs, nB = 19456, 8, 128, 256
    n, r, c, v = synth.vnm_structured(R, M, Vs, seed=3)
    dev = torch.device("cuda", torch.cuda.current_device())
    tr, tc, tv = (torch.from_numpy(x).to(dev) for x in (r, c, v))
    g = torch.Generator().manual_seed(11)
    X = torch.randn((n, nB), generator=g).to(torch.bfloat16)
    Xd = X.to(dev)
    C = torch.empty((n, nB), dtype=torch.float32, device=dev)
    tpk, tkind = load_tensor_peak()
    hpk, hkind = load_peaks()
    out = {"workload": "S1: 19456x19456 in full V:2:8 form (V=128, every block 4 columns x 2 nonzeros a row; "
                       "%d nonzeros), B 19456x256 bf16 N(0,1)" % len(r)}
    rows = np.sort(np.random.default_rng(5).choice(n, 1024, replace=False))
    ptr = np.searchsorted(r, np.arange(n + 1))
    Xf = X.float().numpy().astype(np.float64)
    ref = np.stack([(v[ptr[i]:ptr[i + 1]].astype(np.float64)[:, None] * Xf[c[ptr[i]:ptr[i + 1]]]).sum(0) for i in rows])
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    for label, dm in (("tensor_cores", None), ("cuda_core_residual", 1 << 30)):
        old = os.environ.get("VNM_SPMM_DENSE_MIN")
        if dm is None:
            os.environ.pop("VNM_SPMM_DENSE_MIN", None)
        else:
            os.environ["VNM_SPMM_DENSE_MIN"] = str(dm)
        try:
            A = vnm_gb300.SpmmMatrix(ctx, n, tr, tc, tv, M, Vs, "bf16")
        finally:
            if old is None:
                os.environ.pop("VNM_SPMM_DENSE_MIN", None)
            else:
                os.environ["VNM_SPMM_DENSE_MIN"] = old
        info = A.info()
        A.run(Xd, C)
        A.run(Xd, C)
        ms = []
        for _ in range(reps):
            A.run(Xd, C)
            ms.append(ctx.last_main_kernel_ms)
        k = _median(ms)
        useful = 2.0 * len(r) * nB
        issued = 2.0 * 128 * 16 * nB * info["ksteps"]
        hb = info["a_bytes"] + info["residual_nnz"] * 8 + n * nB * 2 + n * nB * 4
        err = oracle.rowwise_rel_err(C[torch.from_numpy(rows).to(dev)].cpu().numpy(), ref)
        out[label] = {"kernel_ms": k, "useful_tflops": useful / k / 1e9, "issued_tflops": issued / k / 1e9,
                      "issued_frac": issued / k / 1e9 / tpk, "peak_kind": tkind,
                      "hbm": {"bytes": hb, "achieved_gbs": hb / k / 1e6, "frac": hb / k / 1e6 / hpk,
                              "what": "A as stored (tiles, or 8 B per residual nonzero) + B + C once"},
                      "max_rel_err_vs_fp64_per_row_sampled": err, "ksteps": info["ksteps"],
                      "residual_nnz": info["residual_nnz"], "tensor_tiles": info["tensor_tiles"]}
        A.close()
    try:
        out["baselines"] = library_spmm_baselines(n, r, c, v, nB, torch.bfloat16, dense=True, reps=10)
        for kk, d in out["baselines"].items():
            if "ms" in d:
                d["vnm_tensor_speedup"] = d["ms"] / out["tensor_cores"]["kernel_ms"]
    except Exception as e:
        out["baselines"] = {"error": "%s: %s" % (type(e).__name__, e)}
    del tr, tc, tv, Xd, C
    torch.cuda.empty_cache()
    return out


def run_s1_spmm_only(steps):
    """The structured V:2:8 operand of bench_structured_spmm through the
    tensor-core SpMM alone, `steps` calls."""
    import torch
    import vnm_gb300
    from vnm_gb300 import synth
    R, M, Vs, nB = 19456, 8, 128, 256
    n, r, c, v = synth.vnm_structured(R, M, Vs, seed=3)
    dev = torch.device("cuda", 0)
    with vnm_gb300.Context(0) as ctx:
        tr, tc, tv = (torch.from_numpy(x).to(dev) for x in (r, c, v))
        A = vnm_gb300.SpmmMatrix(ctx, n, tr, tc, tv, M, Vs, "bf16")
        X = torch.randn((n, nB), generator=torch.Generator().manual_seed(11)).to(torch.bfloat16).to(dev)
        C = torch.empty((n, nB), dtype=torch.float32, device=dev)
        ms = []
        for _ in range(max(steps, 1)):
            A.run(X, C)
            ms.append(ctx.last_main_kernel_ms)
        info = A.info()
        A.close()
    best = min(ms)
    return {"workload": "S1 SpMM only: 19456x19456 full V:2:8 (V=128), B 19456x256 bf16", "runs": len(ms),
            "kernel_ms_min": best, "issued_tflops": 2.0 * 128 * 16 * nB * info["ksteps"] / (best * 1e-3) / 1e12,
            "useful_tflops": 2.0 * len(r) * nB / (best * 1e-3) / 1e12, "info": info}


def run_c5_spmm_only(steps):
    """The GCN workload's operand built as bench_gcn_c5 builds it, then only
    its BF16 SpMM: the learned reorder runs in a context that is closed
    before the operand is compressed in a fresh one, so its 8.6 GB group
    table is gone while the SpMM runs."""
    import torch
    import vnm_gb300
    from vnm_gb300 import learned, synth
    N, M, Vc, nB = 2, 8, 128, 256
    n, r, c, v = synth.chung_lu_c5(0)
    with vnm_gb300.Context(0) as ctx:
        net = learned.load(ctx, N, M)
        res, newpos, _ = vnm_gb300.nm_learned(ctx, n, r, c, v, N, M, mode=vnm_gb300.LEARNED_MLP, net=net, topk=8,
                                              targets=TARGETS, max_rounds=64, patience=3, seed=1)
        net.close()
        pr, pc = ctx.permute_coo(n, r, c, newpos)
    dev = torch.device("cuda", 0)
    ctx = vnm_gb300.Context(0)
    tr, tc, tv = (torch.from_numpy(x).to(dev) for x in (pr, pc, v))
    A = vnm_gb300.SpmmMatrix(ctx, n, tr, tc, tv, M, Vc, "bf16")
    X = torch.randn((n, nB), generator=torch.Generator().manual_seed(7)).to(torch.bfloat16).to(dev)
    C = torch.empty((n, nB), dtype=torch.float32, device=dev)
    ms = []
    for _ in range(max(steps, 1)):
        A.run(X, C)
        ms.append(ctx.last_main_kernel_ms)
    info = A.info()
    A.close()
    ctx.close()
    best = min(ms)
    return {"workload": "C5 SpMM only: Chung-Lu 262144, learned reorder 2:8, V=128, X 262144x256 bf16",
            "runs": len(ms), "kernel_ms_min": best, "kernel_ms_median": sorted(ms)[len(ms) // 2],
            "issued_tflops": 2.0 * 128 * 16 * nB * info["ksteps"] / (best * 1e-3) / 1e12, "info": info}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.c5_spmm_only:
        print(json.dumps(run_c5_spmm_only(args.steps)))
        return
    if args.s1_spmm_only:
        print(json.dumps(run_s1_spmm_only(args.steps)))
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
