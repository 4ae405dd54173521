#!/usr/bin/env python3
"""Benchmark of the sketch-and-precondition least-squares hot path.

Workload (the configuration the headline metric is quoted on): overdetermined
least squares with A of 100000 x 500, A = U diag(sigma) V^T, sigma log-spaced
from 1 to 1e-8 (kappa = 1e8), b = A x* + 1e-6 N(0,1), Gaussian sketch
d = 4n = 2000, preconditioned LSQR to relative tolerance 1e-12.  Inputs are
seeded synthetic data generated on the GPU (torch CUDA generator); A (400 MB)
is larger than L2, so no flush is needed between steps.

One step = one blendenpik solve (sketch S [A b], QR of the sketch, R^-1,
preconditioned LSQR, x = R^-1 z) through the library's device-pointer entry
point.  `value` is solves/s with inputs resident in HBM; `e2e` is the same
metric through the host-pointer entry point with pinned host buffers (A and b
copied in, x copied out inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload batched [--problems P]   # secondary line

`--workload batched` times many independent problems of mixed shape
(m in [1000, 50000], n in [16, 256], m >= 8 n, kappa 1e6) through one
rnla_solve_batched call per step, beside a loop of plain FP64 solves.
Under torchrun each rank takes its own P problems of the sequence (no
collective): value = all ranks' problems / the slowest rank's time.

With N > 1 (torchrun) every rank solves its own replica (the path has no
exchange step); value = all ranks' solves / max-over-ranks time.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "rand_svd & sketch-LS solves/sec on 1 GB300: BF16-sketch vs plain FP64 at stated error"
UNIT = "solves/s"
CFG = dict(m=100000, n=500, kappa=1e8, noise=1e-6, sampling_factor=4.0, tol=1e-12)
LSQR_DRAM_BYTES_PER_ROW_PASS = (5.819774e9 + 0.0375055e9) / (36 * 40000)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--m", type=int, default=CFG["m"])
    p.add_argument("--n", type=int, default=CFG["n"])
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison path")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--workload", choices=["blendenpik", "batched"], default="blendenpik",
                   help="batched: many small problems through rnla_solve_batched (secondary line)")
    p.add_argument("--problems", type=int, default=512, help="problems in the batched workload")
    return p.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas)
# ---------------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, local, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def wait_first(self, timeout=3.0):
        """Block until the sampler has produced a row (its start-up, which
        talks to the driver, then stays out of the timed region)."""
        t0 = time.time()
        while self.proc is not None and not self.rows and time.time() - t0 < timeout:
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) >= 9:
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# problem generation (seeded, on the GPU)
# ---------------------------------------------------------------------------
def make_problem(m, n, kappa, noise, dev):
    """A = U diag(sigma) V^T with U, V the orthonormal factors (this library's
    Householder Orth) of seeded Gaussian matrices; b = A x* + noise."""
    import numpy as np
    import torch
    import randnla_gb300 as R
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    U = R.Orth(torch.randn(n, m, generator=g, device=dev, dtype=torch.float64).t().cpu().numpy())
    g.manual_seed(2)
    V = R.Orth(torch.randn(n, n, generator=g, device=dev, dtype=torch.float64).t().cpu().numpy())
    sig = np.logspace(0, -math.log10(kappa), n)
    Ut = torch.from_numpy(np.asfortranarray(U)).to(dev)
    Vt = torch.from_numpy(np.ascontiguousarray(V.T * sig[:, None])).to(dev)   # diag(sigma) V^T
    A = (Ut @ Vt).t().contiguous().t()            # column-major, ld = m
    del Ut
    g.manual_seed(3)
    xs = torch.randn(n, generator=g, device=dev, dtype=torch.float64)
    g.manual_seed(4)
    b = A @ xs + noise * torch.randn(m, generator=g, device=dev, dtype=torch.float64)
    return A, b


def workload_name(m, n):
    """The bench workload's name, shared by both arms' JSON lines."""
    return "blendenpik_overdetermined %dx%d kappa=1e8 d=%d lsqr tol=1e-12" % (
        m, n, int(CFG["sampling_factor"] * n))


def rel_residual(A, x, b):
    return float((A @ x - b).norm() / b.norm())


def lapack_rel_residual(A, b):
    """Relative residual of numpy/LAPACK least squares (host, FP64)."""
    import numpy as np
    Ah = A.cpu().numpy()
    bh = b.cpu().numpy()
    xl = np.linalg.lstsq(Ah, bh, rcond=None)[0]
    return float(np.linalg.norm(Ah @ xl - bh) / np.linalg.norm(bh))


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, local, ws):
    import torch
    import numpy as np
    import randnla_gb300 as R

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = R.lib()
    m, n = args.m, args.n
    A, b = make_problem(m, n, CFG["kappa"], CFG["noise"], dev)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    tol = CFG["tol"]
    sf = CFG["sampling_factor"]
    l = 10 * n

    tc = True
    o_fast = R.options(precision=R.Precision.BF16X, inner_solver=R.InnerSolver.LSQR, atol=tol, btol=tol,
                       seed=42)
    try:
        R.blendenpik_dev(A, b, x, tol, l, sf, o_fast)
    except R.Unsupported:
        tc = False
    o_fp64 = R.options(precision=R.Precision.FP64, inner_solver=R.InnerSolver.LSQR, atol=tol, btol=tol,
                       seed=42)
    o = o_fast if tc else o_fp64

    # accuracy of the timed path against the plain FP64 path and LAPACK (cuSOLVER QR)
    st = R.blendenpik_dev(A, b, x, tol, l, sf, o)
    torch.cuda.synchronize()
    rr = rel_residual(A, x, b)
    x64 = torch.zeros_like(x)
    st64 = R.blendenpik_dev(A, b, x64, tol, l, sf, o_fp64)
    torch.cuda.synchronize()
    rr64 = rel_residual(A, x64, b)
    rrl = lapack_rel_residual(A, b)

    # the clock sampler runs from before the warm-up to after the timed steps
    clocks = ClockSampler(local)
    clocks.start()
    clocks.wait_first()
    for _ in range(args.warmup):
        R.blendenpik_dev(A, b, x, tol, l, sf, o)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    launches0 = lib.rnla_kernel_launches()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    solve_ms = []
    e0.record(stream)
    for _ in range(args.steps):
        s_ = R.blendenpik_dev(A, b, x, tol, l, sf, o)
        solve_ms.append((s_["ms_solve"], s_["iterations"], s_["ms_sketch"], s_["ms_factor"], s_["ms_kernel"]))
    e1.record(stream)
    torch.cuda.synchronize()
    launches = lib.rnla_kernel_launches() - launches0
    clk = clocks.stop()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(ms, ws)
    value = ws * args.steps / (ms_max / 1e3)

    # plain FP64 GPU path throughput (same problem, same solver settings)
    fp64 = None
    if not args.no_fp64 and tc:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        R.blendenpik_dev(A, b, x64, tol, l, sf, o_fp64)
        reps = 2
        t0.record(stream)
        for _ in range(reps):
            R.blendenpik_dev(A, b, x64, tol, l, sf, o_fp64)
        t1.record(stream)
        torch.cuda.synchronize()
        fp64 = {"value": reps / (t0.elapsed_time(t1) / 1e3), "unit": UNIT,
                "rel_residual": rr64, "iterations": st64["iterations"]}

    # end to end through the host-pointer entry point with pinned buffers
    Ah = torch.empty((n, m), dtype=torch.float64, pin_memory=True).t()   # column-major host
    Ah.copy_(A.cpu())
    bh = torch.empty(m, dtype=torch.float64, pin_memory=True)
    bh.copy_(b.cpu())
    xh = torch.empty(n, dtype=torch.float64, pin_memory=True)
    st_e = R.Stats()
    o_c = o

    def e2e_call():
        rc = lib.rnla_blendenpik_overdetermined_ex(
            ctypes.c_void_p(Ah.data_ptr()), m, n, m, ctypes.c_void_p(bh.data_ptr()), tol, l, sf,
            ctypes.byref(o_c), ctypes.c_void_p(xh.data_ptr()), ctypes.byref(st_e))
        if rc != 0:
            raise RuntimeError(lib.rnla_last_error_message().decode())

    for _ in range(2):
        e2e_call()
    barrier(ws)
    t_start = time.perf_counter()
    ke = max(2, args.steps // 2)
    for _ in range(ke):
        e2e_call()
    t_e2e = time.perf_counter() - t_start
    t_e2e = max_over_ranks(t_e2e, ws)
    e2e_val = ws * ke / t_e2e

    # roofline of the dominant kernel
    ms_solve = sum(s[0] for s in solve_ms) / len(solve_ms)
    ms_sketch = sum(s[2] for s in solve_ms) / len(solve_ms)
    ms_factor = sum(s[3] for s in solve_ms) / len(solve_ms)
    iters = solve_ms[-1][1]
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            peaks = json.load(f)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    ms_kernel = sum(s[4] for s in solve_ms) / len(solve_ms)
    elem = m * n * 8
    # one launch = iters + 1 streamed passes; each reads the float-float copy
    # of A (8 bytes per element) and reads + writes u (2 x 8 bytes per row)
    passes = iters + 1
    lsqr_bytes = passes * (elem + 2 * 8 * m)
    lsqr_gbs = lsqr_bytes / (ms_kernel / 1e3) / 1e9 if ms_kernel > 0 else None
    # DRAM bytes (read + write) per row and pass of lsqr_ff_kernel from one ncu
    # capture (40000 x 500, 36 passes: 5.8198 GB read + 0.0375 GB written),
    # scaled by rows and passes
    lsqr_traffic = LSQR_DRAM_BYTES_PER_ROW_PASS * m * passes if n == 500 else None
    sketch_flops = 2.0 * int(CFG["sampling_factor"] * n) * m * (n + 1)   # S [A b]
    sketch_tflops = sketch_flops / (ms_sketch / 1e3) / 1e12
    stages = {"sketch_ms": ms_sketch, "qr_rinv_ms": ms_factor, "lsqr_ms": ms_solve,
              "lsqr_iterations": iters}
    if (ms_solve >= ms_sketch or not tc) and lsqr_gbs is not None:
        roof = {"bound": "hbm",
                "kernel": "lsqr_ff_kernel (one streamed A y / A^T u pass over the float-float copy of A "
                          "per LSQR iteration)",
                "achieved": lsqr_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": lsqr_gbs / hbm_peak,
                "traffic": lsqr_traffic, "peak_source": peak_src, "kernel_ms_per_launch": ms_kernel,
                "algorithmic_bytes_per_launch": lsqr_bytes}
    else:
        roof = {"bound": "tensor", "kernel": "sketch_tc (digit-sliced bf16 S [A b])",
                "achieved": sketch_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": sketch_tflops / bf16_peak, "traffic": None, "peak_source": peak_src,
                "algorithmic_flops_per_launch": sketch_flops}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 digit-sliced sketch + float-float (fp32 pairs) QR/LSQR" if tc else "f64",
        "data": "synthetic (seeded torch CUDA generator)",
        "config": {"workload": workload_name(m, n),
                   "m": m, "n": n, "d": int(CFG["sampling_factor"] * n), "kappa": CFG["kappa"],
                   "precision": "BF16X" if tc else "FP64", "inner_solver": "LSQR",
                   "l2": "inputs larger than L2 (A is %d MB)" % (elem >> 20),
                   "parallelism": "replicas" if ws > 1 else "single"},
        "accuracy": {"rel_residual": rr, "rel_residual_fp64_path": rr64, "rel_residual_lapack": rrl,
                     "abs_diff_vs_fp64": abs(rr - rr64), "abs_diff_vs_lapack": abs(rr - rrl)},
        "stages": stages,
        "fp64_path": fp64,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": elem + m * 8,
                "d2h_bytes_per_step": n * 8},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk,
    }
    return line


# ---------------------------------------------------------------------------
# batched workload: many independent problems of mixed shape
# ---------------------------------------------------------------------------
def batched_shapes(count, seed=12, rank=0, world=1):
    """Problem p of the seeded sequence: m ~ U[1000, 50000], n ~ U[16, 256],
    redrawn until m >= 8 n.  Rank r of `world` takes problems
    [r count, (r + 1) count) -- independent units, no exchange between
    ranks, the same work per rank at every world size.  Returns
    (global index, (m, n)) pairs."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count * (rank + 1):
        m, n = int(rng.integers(1000, 50001)), int(rng.integers(16, 257))
        if m >= 8 * n:
            out.append((m, n))
    return list(enumerate(out))[count * rank:]


def make_batched(shapes, dev, kappa=1e6, noise=1e-6, seed=12):
    """A_p = U_p diag(sigma) V_p^T (orthonormal factors of seeded Gaussian
    matrices, sigma log-spaced to kappa), b_p = A_p x* + noise, on the GPU;
    problem p's data depends only on its global index."""
    import torch
    g = torch.Generator(device=dev)
    probs = []
    for p, (m, n) in shapes:
        g.manual_seed(seed * 1000003 + p)
        U = torch.linalg.qr(torch.randn(m, n, generator=g, device=dev, dtype=torch.float64))[0]
        V = torch.linalg.qr(torch.randn(n, n, generator=g, device=dev, dtype=torch.float64))[0]
        sig = torch.logspace(0, -math.log10(kappa), n, device=dev, dtype=torch.float64)
        A = ((U * sig) @ V.t()).t().contiguous().t()
        del U, V
        b = A @ torch.randn(n, generator=g, device=dev, dtype=torch.float64)
        b += noise * torch.randn(m, generator=g, device=dev, dtype=torch.float64)
        probs.append((A, b, torch.zeros(n, dtype=torch.float64, device=dev)))
    return probs


def run_batched(args, rank, local, ws):
    import torch
    import numpy as np
    import randnla_gb300 as R

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = R.lib()
    indexed = batched_shapes(args.problems, rank=rank, world=ws)
    probs = make_batched(indexed, dev)
    shapes = [mn for _, mn in indexed]
    tol, sf = 1e-12, CFG["sampling_factor"]
    o = R.options(precision=R.Precision.BF16X, inner_solver=R.InnerSolver.LSQR, atol=tol, btol=tol)
    o64 = R.options(precision=R.Precision.FP64, inner_solver=R.InnerSolver.LSQR, atol=tol, btol=tol)
    l = 2000
    status, stats = R.solve_batched_dev(probs, tol, l, sf, o)
    torch.cuda.synchronize()
    if any(status):
        raise RuntimeError("batched solve failed: %s" % sorted(set(status)))
    # accuracy on the first problems against LAPACK
    worst = 0.0
    for a, b, x in probs[:4]:
        Ah, bh, xh = a.cpu().numpy(), b.cpu().numpy(), x.cpu().numpy()
        xl = np.linalg.lstsq(Ah, bh, rcond=None)[0]
        rr = np.linalg.norm(Ah @ xh - bh) / np.linalg.norm(bh)
        rl = np.linalg.norm(Ah @ xl - bh) / np.linalg.norm(bh)
        worst = max(worst, abs(rr - rl))

    clocks = ClockSampler(local)
    clocks.start()
    clocks.wait_first()
    for _ in range(args.warmup):
        R.solve_batched_dev(probs, tol, l, sf, o)
    torch.cuda.synchronize()
    barrier(ws)
    launches0 = lib.rnla_kernel_launches()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        status, stats = R.solve_batched_dev(probs, tol, l, sf, o)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = lib.rnla_kernel_launches() - launches0
    clk = clocks.stop()
    barrier(ws)
    ms = max_over_ranks(e0.elapsed_time(e1), ws)
    value = ws * args.steps * len(probs) / (ms / 1e3)

    # the plain FP64 path as a loop of single-problem solves, on the first 32
    sub = probs[:32]
    for a, b, x in sub[:2]:
        R.blendenpik_dev(a, b, x, tol, l, sf, o64)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for a, b, x in sub:
        R.blendenpik_dev(a, b, x, tol, l, sf, o64)
    t1.record(stream)
    torch.cuda.synchronize()
    fp64_value = len(sub) / (t0.elapsed_time(t1) / 1e3)

    # A is read once by the sketch and once per LSQR pass (float-float copy)
    its = [s_["iterations"] for s_ in stats]
    byts = sum(8.0 * m * n * (2 + it) for (m, n), it in zip(shapes, its))
    gbs = byts * args.steps / (ms / 1e3) / 1e9
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            peaks = json.load(f)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    return {
        "metric": "batched least-squares problems/s on 1 GB300 (BF16X sketch, float-float LSQR)",
        "value": value, "unit": "problems/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 digit-sliced sketch + float-float (fp32 pairs) QR/LSQR",
        "data": "synthetic (seeded torch CUDA generator)",
        "config": {"workload": "%d blendenpik problems per rank, m in [1000, 50000], n in [16, 256], m >= 8n, "
                               "kappa 1e6, d = 4n, lsqr tol 1e-12, one rnla_solve_batched call per step"
                               % len(probs),
                   "problems": len(probs), "total_A_GB": sum(8.0 * m * n for m, n in shapes) / 1e9,
                   "l2": "inputs larger than L2",
                   "parallelism": "problems sharded over %d ranks, no collective" % ws if ws > 1 else "single"},
        "accuracy": {"max_abs_diff_rel_residual_vs_lapack_first4": worst},
        "mean_iterations": float(np.mean(its)),
        "stages_mean_ms": {k: float(np.mean([s_[k] for s_ in stats]))
                           for k in ("ms_sketch", "ms_factor", "ms_solve", "ms_total")},
        "fp64_path": {"value": fp64_value, "unit": "problems/s",
                      "sample": "loop of single-problem FP64 solves over the first %d problems" % len(sub)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "whole batch (sketch read + one read of A per LSQR pass)",
                     "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                     "traffic": None, "algorithmic_bytes_per_step": byts},
        "clocks": clk,
    }


# ---------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference algorithm
# ---------------------------------------------------------------------------
def cpu_sample(m_full, n, iters, sample_rows):
    """Reference blendenpik (sketch_and_precondition.rs:26-59: dense Gaussian
    S, S a, QR, R^-1, explicit a R^-1, CGLS) on a row-subsampled problem with
    the same n, kappa and d; CGLS runs `iters` iterations.  Returns
    (seconds for the sample, full-size solves/s by linear scaling in m)."""
    import numpy as np
    from oracle import oracle as O
    ms = sample_rows
    d = int(CFG["sampling_factor"] * n)
    rng = np.random.default_rng(0)
    U = np.linalg.qr(rng.standard_normal((ms, n)))[0]
    V = np.linalg.qr(rng.standard_normal((n, n)))[0]
    A = (U * np.logspace(0, -8, n)) @ V.T
    b = A @ rng.standard_normal(n) + 1e-6 * rng.standard_normal(ms)
    S = O.sketch(O.DIST_GAUSSIAN, d, ms)
    t0 = time.perf_counter()
    O.blendenpik_overdetermined(A, b, 1e-300, iters, CFG["sampling_factor"], S=S)
    t = time.perf_counter() - t0
    # the sketch generation is part of the reference call (sketch.rs:102-130); time it too
    t1 = time.perf_counter()
    O.sketch(O.DIST_GAUSSIAN, d, min(ms, 20000))
    tg = (time.perf_counter() - t1) * ms / min(ms, 20000)
    total = t + tg
    return total, 1.0 / (total * m_full / ms)


def lapack_sample(m_full, n, sample_rows):
    """numpy/LAPACK FP64 least squares (gelsd through numpy.linalg.lstsq, all
    host threads) on the same kind of row sample as cpu_sample.  Returns
    (seconds for the sample, full-size solves/s by linear scaling in m: the
    cost is O(m n^2))."""
    import numpy as np
    rng = np.random.default_rng(1)
    U = np.linalg.qr(rng.standard_normal((sample_rows, n)))[0]
    V = np.linalg.qr(rng.standard_normal((n, n)))[0]
    A = np.asfortranarray((U * np.logspace(0, -8, n)) @ V.T)
    b = A @ rng.standard_normal(n) + 1e-6 * rng.standard_normal(sample_rows)
    np.linalg.lstsq(A[:1000], b[:1000], rcond=None)          # load LAPACK once
    t0 = time.perf_counter()
    np.linalg.lstsq(A, b, rcond=None)
    t = time.perf_counter() - t0
    return t, 1.0 / (t * m_full / sample_rows)


def run_reference(args, rank, ws):
    """The reference arm: the oracle's CPU restatement of the reference's
    path on the host cores, rank 0 only."""
    if rank != 0:
        return None
    import numpy as np
    iters = 40
    rows = max(2 * int(CFG["sampling_factor"] * args.n), 10000)
    samples = []
    for _ in range(args.warmup):
        cpu_sample(args.m, args.n, iters, rows)
    for _ in range(args.steps):
        samples.append(cpu_sample(args.m, args.n, iters, rows)[1])
    v = float(np.median(samples))
    cores = os.cpu_count()
    return {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy generator)",
        "impl": "reference",
        "config": {"workload": workload_name(args.m, args.n), "m": args.m, "n": args.n,
                   "d": int(CFG["sampling_factor"] * args.n), "kappa": CFG["kappa"],
                   "algorithm": "the reference's data flow: dense Gaussian S, S a, Householder QR, "
                                "explicit a R^-1, CGLS (%d iterations, the count LSQR needs at "
                                "tol 1e-12 on this problem, within a few)" % iters},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "oracle restatement of sketch_and_precondition.rs:26-59 "
                                   "(numpy/LAPACK on all host threads, C sketch generator) on "
                                   "%d x %d rows with %d CGLS iterations, scaled linearly in m "
                                   "to %d rows" % (rows, args.n, iters, args.m)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, local, ws = dist_init()
    if args.impl == "reference":
        line = run_reference(args, rank, ws)
        if line is not None:
            print(json.dumps(line))
        return
    if args.workload == "batched":
        line = run_batched(args, rank, local, ws)
        if rank == 0:
            print(json.dumps(line))
        return
    line = run_ours(args, rank, local, ws)
    if rank == 0 and not args.no_cpu:
        iters = line["stages"]["lsqr_iterations"]
        rows = max(2 * int(CFG["sampling_factor"] * args.n), 10000)
        t, v = cpu_sample(args.m, args.n, max(iters, 1), rows)
        line["cpu_baseline"] = {
            "value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "sample": "oracle restatement of sketch_and_precondition.rs:26-59 (numpy/LAPACK on all "
                      "host threads, C sketch generator) on %d x %d rows, %d CGLS iterations "
                      "(the GPU's iteration count), %.2f s, scaled linearly in m to %d rows"
                      % (rows, args.n, iters, t, args.m)}
        tl, vl = lapack_sample(args.m, args.n, rows)
        line["cpu_baseline"]["lapack_lstsq"] = {
            "value": vl, "unit": UNIT, "cores": os.cpu_count(),
            "sample": "numpy.linalg.lstsq (LAPACK gelsd, FP64, all host threads) on %d x %d rows, "
                      "%.2f s, scaled linearly in m to %d rows" % (rows, args.n, tl, args.m)}
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
