#!/usr/bin/env python3
"""Benchmark of the sketch-and-precondition least-squares hot path.

Workloads (`--workload`, seeded synthetic inputs of the stated shapes; no
dataset is involved):

  precision_ls (default)  overdetermined least squares, A of 1048576 x 1024
                          stored in FP32, A = U diag(sigma) V^T with U, V the
                          orthonormal factors of seeded Gaussian matrices and
                          sigma log-spaced 1 -> 1e-6 (kappa 1e6); b = A x* +
                          1e-8 N(0,1) in FP64; Gaussian sketch d = 4096;
                          preconditioned LSQR to tolerance 1e-10.
  plain_ls                A of 100000 x 500 in FP64, sigma 1 -> 1e-8
                          (kappa 1e8), b = A x* + 1e-6 N(0,1), d = 2000,
                          LSQR to tolerance 1e-12.
  precision_svd           rand_svd (RandNLA mode, tensor cores) of A of
                          65536 x 16384 stored in FP32, sigma_i = exp(-i/64)
                          on rank 1536 plus a 1e-6 noise floor; k = 256,
                          p = 32, q = 2.
  plain_svd               rand_svd of A of 2000 x 1000 (FP64, sigma_i =
                          10^(-i/100)); k = 50, p = 10, q = 2.
  batched                 2048 independent least-squares problems of mixed
                          shape (m in [1000, 50000], n in [16, 256],
                          m >= 8 n, kappa 1e6) through one rnla_solve_batched
                          call per step.

One least-squares step = one blendenpik solve (sketch S [A b], factorization
of the sketch, R^-1, preconditioned LSQR, x = R^-1 z) through the library's
device-pointer entry point; one rand_svd step = one rand_svd through
rnla_rand_svd_dev.  `value` is solves/s with inputs resident in HBM; `e2e` is the same
metric through the host-pointer entry point with pinned host buffers (A and b
copied in, x copied out inside the timed region), over max(5, K) calls after
max(3, W) untimed ones, with the per-call median / min / max and the plain
pinned-copy bandwidth of A beside it (the host link of a shared machine
slows single copies by 2-3x at times, and the total includes those calls).
A is larger than L2 in every workload, so no flush is needed between steps.

The CPU legs (`cpu_baseline` and `--impl reference`) run the oracle's
restatement of the reference path at the FULL size of the workload: no row
sampling, no extrapolation; each CPU solve runs in a subprocess with a
10-minute cap and is reported as "not finished (cap)" if it exceeds it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload precision_ls|plain_ls|precision_svd|plain_svd|batched]

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
CPU_CAP_S = 600.0
WORKLOADS = {
    "precision_ls": dict(m=1048576, n=1024, kappa=1e6, noise=1e-8, sampling_factor=4.0, tol=1e-10,
                         f32=True, seeds=(8, 9, 10, 11)),
    "plain_ls": dict(m=100000, n=500, kappa=1e8, noise=1e-6, sampling_factor=4.0, tol=1e-12,
                     f32=False, seeds=(1, 2, 3, 4)),
}
# rand_svd workloads: A = U diag(sigma) V^T (+ noise floor), Gaussian range
# finder with k + p columns and q power iterations (RandNLA mode, Philox key 42)
SVD_WORKLOADS = {
    "precision_svd": dict(m=65536, n=16384, rank=1536, decay="exp(-i/64)", noise=1e-6, k=256, p=32, q=2,
                          f32=True, seeds=(5, 6, 7)),
    "plain_svd": dict(m=2000, n=1000, rank=1000, decay="10^(-i/100)", noise=0.0, k=50, p=10, q=2,
                      f32=False, seeds=(1, 2, 0)),
}
# DRAM bytes (read + write) per row and pass of lsqr_ff_kernel from one ncu
# capture (40000 x 500, float-float copy, 36 passes: 5.8198 GB read + 0.0375
# GB written); per row and pass the kernel moves 8 ldf + 16 bytes.
LSQR_DRAM_BYTES_PER_ROW_PASS = (5.819774e9 + 0.0375055e9) / (36 * 40000)
LSQR_NCU_ALGO_BYTES_PER_ROW_PASS = 8 * 500 + 16
# the same ratio for FP32 rows: one ncu capture at 131072 x 1024 (31 passes: 16.9706 GB
# read + 0.0752 GB written)
LSQR_F32_DRAM_RATIO = (16.970577e9 + 0.075243e9) / (31 * (4 * 1024 + 16) * 131072)


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["precision_ls", "plain_ls", "precision_svd", "plain_svd", "batched"],
                   default="precision_ls")
    p.add_argument("--m", type=int, default=None, help="rows (default: the workload's)")
    p.add_argument("--n", type=int, default=None, help="columns (default: the workload's)")
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison path")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffers) leg")
    p.add_argument("--problems", type=int, default=2048, help="problems in the batched workload")
    p.add_argument("--cpu-leg", choices=["port", "lapack"], default=None, help=argparse.SUPPRESS)
    return p.parse_args(argv)


def workload(args):
    """The workload's parameters with the command line's --m / --n applied."""
    if args.workload in SVD_WORKLOADS:
        wl = dict(SVD_WORKLOADS[args.workload])
        if args.m:
            wl["m"] = args.m
        if args.n:
            wl["n"] = args.n
        wl["rank"] = min(wl["rank"], wl["m"], wl["n"])
        return wl
    wl = dict(WORKLOADS[args.workload])
    if args.m:
        wl["m"] = args.m
    if args.n:
        wl["n"] = args.n
    wl["d"] = int(wl["sampling_factor"] * wl["n"])
    return wl


def workload_config(args, wl, ws):
    """The `config` object both arms print (identical, so the lines compare)."""
    if args.workload in SVD_WORKLOADS:
        return {"workload": "rand_svd %dx%d %s sigma_i=%s (rank %d) noise=%g k=%d p=%d q=%d"
                            % (wl["m"], wl["n"], "fp32" if wl["f32"] else "fp64", wl["decay"], wl["rank"],
                               wl["noise"], wl["k"], wl["p"], wl["q"]),
                "name": args.workload, "m": wl["m"], "n": wl["n"], "k": wl["k"], "p": wl["p"], "q": wl["q"],
                "a_storage": "fp32" if wl["f32"] else "fp64",
                "l2": "A is %d MB%s" % ((wl["m"] * wl["n"] * (4 if wl["f32"] else 8)) >> 20,
                                        " (larger than L2)" if wl["m"] * wl["n"] * 4 > 129e6 else
                                        " (fits in L2: no flush between steps)"),
                "parallelism": "replicas" if ws > 1 else "single"}
    return {"workload": "blendenpik_overdetermined %dx%d %s kappa=%g d=%d lsqr tol=%g"
                        % (wl["m"], wl["n"], "fp32" if wl["f32"] else "fp64", wl["kappa"], wl["d"], wl["tol"]),
            "name": args.workload, "m": wl["m"], "n": wl["n"], "d": wl["d"], "kappa": wl["kappa"],
            "a_storage": "fp32" if wl["f32"] else "fp64", "tol": wl["tol"],
            "l2": "inputs larger than L2 (A is %d MB)" % ((wl["m"] * wl["n"] * (4 if wl["f32"] else 8)) >> 20),
            "parallelism": "replicas" if ws > 1 else "single"}


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


def time_host_calls(call, steps, warmup, ws):
    """End-to-end leg: `warmup` (at least 3) untimed calls, then `steps`
    calls timed one by one on the host clock (each call returns only once
    its results are in host memory).  Returns the max-over-ranks total
    seconds and the per-call milliseconds: the total gives `e2e.value`,
    the spread shows calls slowed by the host link."""
    for _ in range(max(3, warmup)):
        call()
    barrier(ws)
    per = []
    t_start = time.perf_counter()
    for _ in range(steps):
        t = time.perf_counter()
        call()
        per.append((time.perf_counter() - t) * 1e3)
    total = max_over_ranks(time.perf_counter() - t_start, ws)
    per.sort()
    return total, {"median": per[len(per) // 2], "min": per[0], "max": per[-1]}


def pinned_h2d_gbs(host, dev, reps=5):
    """Bandwidth of plain copies of a pinned host tensor to the device (the
    same bytes the end-to-end call uploads): median and slowest of `reps`
    copies, for reading the end-to-end figure against the host link."""
    import torch
    d = torch.empty_like(host, device=dev)      # same strides: one contiguous copy
    rates = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        d.copy_(host, non_blocking=True)
        torch.cuda.synchronize()
        rates.append(host.numel() * host.element_size() / (time.perf_counter() - t) / 1e9)
    del d
    rates.sort()
    return {"median": rates[len(rates) // 2], "min": rates[0]}


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
def make_problem(wl, dev):
    """A = U diag(sigma) V^T with U, V the orthonormal factors of seeded
    Gaussian matrices (m x n and n x n), sigma log-spaced 1 -> 1/kappa;
    b = A x* + noise N(0, 1) (FP64).  The FP32 workload rounds A to FP32 and
    forms b from the rounded A.  Returns column-major A (ld = m) and b."""
    import numpy as np
    import torch
    import randnla_gb300 as R
    m, n = wl["m"], wl["n"]
    su, sv, sx, sb = wl["seeds"]
    g = torch.Generator(device=dev)
    if wl["f32"]:
        sig = torch.logspace(0, -math.log10(wl["kappa"]), n, device=dev, dtype=torch.float64)
        g.manual_seed(su)
        U = torch.linalg.qr(torch.randn(m, n, generator=g, device=dev, dtype=torch.float64))[0]
        g.manual_seed(sv)
        V = torch.linalg.qr(torch.randn(n, n, generator=g, device=dev, dtype=torch.float64))[0]
        At = (V * sig) @ U.t()                   # A^T, row-major n x m = A column-major
        del U
        A = At.float().t()
        del At
        Ad = A.double()
    else:
        g.manual_seed(su)
        U = R.Orth(torch.randn(n, m, generator=g, device=dev, dtype=torch.float64).t().cpu().numpy())
        g.manual_seed(sv)
        V = R.Orth(torch.randn(n, n, generator=g, device=dev, dtype=torch.float64).t().cpu().numpy())
        sig = np.logspace(0, -math.log10(wl["kappa"]), n)
        Ut = torch.from_numpy(np.asfortranarray(U)).to(dev)
        Vt = torch.from_numpy(np.ascontiguousarray(V.T * sig[:, None])).to(dev)   # diag(sigma) V^T
        A = (Ut @ Vt).t().contiguous().t()            # column-major, ld = m
        del Ut
        Ad = A
    g.manual_seed(sx)
    xs = torch.randn(n, generator=g, device=dev, dtype=torch.float64)
    g.manual_seed(sb)
    b = Ad @ xs + wl["noise"] * torch.randn(m, generator=g, device=dev, dtype=torch.float64)
    return A, b


def accuracy(A, x, b, xref=None):
    """Relative residual ||b - A x|| / ||b||, the normwise backward error
    ||A^T r|| / (||A||_F ||r||) and, given xref, ||x - xref|| / ||xref||,
    all in FP64 on the GPU."""
    Ad = A if A.dtype == x.dtype else A.to(x.dtype)
    r = b - Ad @ x
    rn = float(r.norm())
    out = {"rel_residual": rn / float(b.norm()),
           "backward_error": float((Ad.t() @ r).norm()) / (float(Ad.norm()) * rn) if rn > 0 else 0.0}
    if xref is not None:
        out["x_rel_diff"] = float((x - xref).norm() / xref.norm())
    return out


def lapack_solve(A, b):
    """numpy/LAPACK FP64 least squares on the host through Householder QR
    (geqrf/orgqr, all host threads): (x, seconds)."""
    import numpy as np
    Ah = np.asfortranarray(A.double().cpu().numpy())
    bh = b.cpu().numpy()
    t0 = time.perf_counter()
    q, r = np.linalg.qr(Ah, mode="reduced")
    import scipy.linalg
    x = scipy.linalg.solve_triangular(r, q.T @ bh, lower=False)
    return x, time.perf_counter() - t0


def load_peaks():
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        with open(pk) as f:
            return json.load(f), "measured"
    return {}, "fallback"


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
    wl = workload(args)
    m, n, d = wl["m"], wl["n"], wl["d"]
    A, b = make_problem(wl, dev)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    tol = wl["tol"]
    sf = wl["sampling_factor"]
    l = 10 * n
    esz = 4 if wl["f32"] else 8

    o = R.options(precision=R.Precision.BF16X, inner_solver=R.InnerSolver.LSQR, atol=tol, btol=tol, seed=42)
    o_fp64 = R.options(precision=R.Precision.FP64, inner_solver=R.InnerSolver.LSQR, atol=tol, btol=tol,
                       seed=42)
    stream = torch.cuda.current_stream()

    # accuracy of the timed path against the plain FP64 GPU path (same
    # problem, same solver settings); the FP64 solve is also timed
    R.blendenpik_dev(A, b, x, tol, l, sf, o)
    torch.cuda.synchronize()
    x64 = torch.zeros_like(x)
    fp64 = None
    st64 = None
    if not args.no_fp64:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        st64 = R.blendenpik_dev(A, b, x64, tol, l, sf, o_fp64)
        t1.record(stream)
        torch.cuda.synchronize()
        ms64 = t0.elapsed_time(t1)
        if ms64 < 2000.0:                       # short enough to repeat for a steadier figure
            reps = 2
            t0.record(stream)
            for _ in range(reps):
                R.blendenpik_dev(A, b, x64, tol, l, sf, o_fp64)
            t1.record(stream)
            torch.cuda.synchronize()
            ms64 = t0.elapsed_time(t1) / reps
        fp64 = {"value": 1e3 / ms64, "unit": UNIT, "ms_per_solve": ms64,
                "iterations": st64["iterations"], "stages_ms": {k: st64[k] for k in
                                                               ("ms_sketch", "ms_factor", "ms_solve")}}

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

    acc = accuracy(A, x, b)
    acc64 = accuracy(A, x64, b) if fp64 else None
    acc["x_rel_diff_vs_fp64_path"] = float((x - x64).norm() / x64.norm()) if fp64 else None
    if fp64:
        acc["rel_residual_fp64_path"] = acc64["rel_residual"]
        acc["backward_error_fp64_path"] = acc64["backward_error"]
        acc["abs_diff_rel_residual_vs_fp64"] = abs(acc["rel_residual"] - acc64["rel_residual"])

    # end to end through the host-pointer entry point with pinned buffers
    e2e = None
    if not args.no_e2e:
        dt = torch.float32 if wl["f32"] else torch.float64
        Ah = torch.empty((n, m), dtype=dt, pin_memory=True).t()   # column-major host
        Ah.copy_(A.cpu())
        bh = torch.empty(m, dtype=torch.float64, pin_memory=True)
        bh.copy_(b.cpu())
        xh = torch.empty(n, dtype=torch.float64, pin_memory=True)
        st_e = R.Stats()
        fn = lib.rnla_blendenpik_overdetermined_f32_ex if wl["f32"] else lib.rnla_blendenpik_overdetermined_ex

        def e2e_call():
            rc = fn(ctypes.c_void_p(Ah.data_ptr()), m, n, m, ctypes.c_void_p(bh.data_ptr()), tol, l, sf,
                    ctypes.byref(o), ctypes.c_void_p(xh.data_ptr()), ctypes.byref(st_e))
            if rc != 0:
                raise RuntimeError(lib.rnla_last_error_message().decode())

        ke = max(5, args.steps)
        t_e2e, call_ms = time_host_calls(e2e_call, ke, args.warmup, ws)
        e2e = {"value": ws * ke / t_e2e, "unit": UNIT, "h2d_bytes_per_step": m * n * esz + m * 8,
               "d2h_bytes_per_step": n * 8, "steps": ke, "call_ms": call_ms,
               # the last call's device-timed stages: the sketch stage includes the wait for the upload
               "stages_ms": {"sketch_and_upload": st_e.ms_sketch, "factor": st_e.ms_factor,
                             "solve": st_e.ms_solve},
               "pinned_h2d_gbs_of_A": pinned_h2d_gbs(Ah, dev)}
        del Ah

    # roofline of the dominant kernel
    ms_solve = sum(s[0] for s in solve_ms) / len(solve_ms)
    ms_sketch = sum(s[2] for s in solve_ms) / len(solve_ms)
    ms_factor = sum(s[3] for s in solve_ms) / len(solve_ms)
    ms_kernel = sum(s[4] for s in solve_ms) / len(solve_ms)
    iters = solve_ms[-1][1]
    peaks, peak_src = load_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    # one lsqr_ff_kernel launch = iters + 1 streamed passes; each reads the
    # row-major copy of A -- FP32 rows of n rounded up to 4 (4 bytes per
    # element) for FP32-stored A, float-float rows of n rounded up to 2 (8
    # bytes) for FP64 A -- and reads + writes u (2 x 8 bytes per row)
    row_bytes = 4.0 * ((n + 3) & ~3) if wl["f32"] else 8.0 * ((n + 1) & ~1)
    passes = iters + 1
    lsqr_bytes = passes * (row_bytes * m + 16.0 * m)
    lsqr_gbs = lsqr_bytes / (ms_kernel / 1e3) / 1e9 if ms_kernel > 0 else None
    # DRAM traffic: the ncu ratio of DRAM bytes to algorithmic bytes of the
    # matching row layout, scaled by rows and passes
    ratio = LSQR_F32_DRAM_RATIO if wl["f32"] else LSQR_DRAM_BYTES_PER_ROW_PASS / LSQR_NCU_ALGO_BYTES_PER_ROW_PASS
    lsqr_traffic = ratio * lsqr_bytes if ratio else None
    sketch_flops = 2.0 * d * m * (n + 1)   # S [A b], algorithmic
    sketch_tflops = sketch_flops / (ms_sketch / 1e3) / 1e12
    stages = {"sketch_ms": ms_sketch, "qr_rinv_ms": ms_factor, "lsqr_ms": ms_solve, "lsqr_kernel_ms": ms_kernel,
              "lsqr_iterations": iters, "sketch_algorithmic_tflops": sketch_tflops}
    roof = {"bound": "hbm",
            "kernel": "lsqr_ff_kernel (one streamed A y / A^T u pass over the row-major copy of A per LSQR "
                      "iteration: FP32 rows for FP32-stored A, float-float rows for FP64 A)",
            "achieved": lsqr_gbs, "peak": hbm_peak, "unit": "GB/s",
            "frac": lsqr_gbs / hbm_peak if lsqr_gbs else None,
            "traffic": lsqr_traffic, "peak_source": peak_src, "kernel_ms_per_launch": ms_kernel,
            "algorithmic_bytes_per_launch": lsqr_bytes}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 digit-sliced sketch + float-float (fp32 pairs) QR/LSQR",
        "data": "synthetic (seeded torch CUDA generator)",
        "config": workload_config(args, wl, ws),
        "path": "BF16X (tcgen05 digit-sliced sketch, float-float QR or FP64 QR, float-float LSQR)",
        "accuracy": acc,
        "stages": stages,
        "fp64_path": fp64,
        "speedup_vs_fp64_path": (value / ws) / fp64["value"] if fp64 else None,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu:
        line["accuracy_lapack"] = None
        try:
            xl, tl = lapack_solve(A, b)
            xl = torch.from_numpy(xl).to(dev)
            al = accuracy(A, xl, b)
            line["accuracy_lapack"] = {"rel_residual": al["rel_residual"], "backward_error": al["backward_error"],
                                       "abs_diff_rel_residual": abs(acc["rel_residual"] - al["rel_residual"]),
                                       "x_rel_diff": float((x - xl).norm() / xl.norm()), "seconds": tl}
        except MemoryError:
            pass
    del A
    return line


# ---------------------------------------------------------------------------
# rand_svd workloads
# ---------------------------------------------------------------------------
def make_svd_problem(wl, dev):
    """A = U diag(sigma) V^T (+ the noise floor noise * G / (sqrt m + sqrt n)),
    U, V orthonormal factors of seeded Gaussian m x r and n x r matrices,
    sigma from the workload's decay law; stored FP32 or FP64, column-major."""
    import torch
    m, n, r = wl["m"], wl["n"], wl["rank"]
    su, sv, se = wl["seeds"]
    i = torch.arange(r, device=dev, dtype=torch.float64)
    sig = torch.exp(-i / 64.0) if wl["decay"].startswith("exp") else 10.0 ** (-i / 100.0)
    g = torch.Generator(device=dev)
    g.manual_seed(su)
    U = torch.linalg.qr(torch.randn(m, r, generator=g, device=dev, dtype=torch.float64))[0]
    g.manual_seed(sv)
    V = torch.linalg.qr(torch.randn(n, r, generator=g, device=dev, dtype=torch.float64))[0]
    At = (V * sig) @ U.t()                            # A^T row-major = A column-major
    del U, V
    if wl["noise"] > 0:
        g.manual_seed(se)
        At += (wl["noise"] / (math.sqrt(m) + math.sqrt(n))) * torch.randn(n, m, generator=g, device=dev,
                                                                        dtype=torch.float64)
    A = (At.float() if wl["f32"] else At).t()
    return A


def run_svd(args, rank, local, ws):
    import torch
    import randnla_gb300 as R
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lib = R.lib()
    wl = workload(args)
    m, n, k, p, q = wl["m"], wl["n"], wl["k"], wl["p"], wl["q"]
    l = min(k + p, m, n)
    A = make_svd_problem(wl, dev)
    stream = torch.cuda.current_stream()

    def outputs():
        U = torch.zeros((l, m), dtype=torch.float64, device=dev).t()
        sg = torch.zeros(l, dtype=torch.float64, device=dev)
        Vt = torch.zeros((n, l), dtype=torch.float64, device=dev).t()
        return U, sg, Vt

    o = R.options(precision=R.Precision.BF16X, mode=R.Mode.RandNLA, power_iters=q, seed=42)
    o64 = R.options(precision=R.Precision.FP64, mode=R.Mode.RandNLA, power_iters=q, seed=42)
    U, sg, Vt = outputs()
    R.rand_svd_dev(A, k, 1e-6, p, U, sg, Vt, o)
    torch.cuda.synchronize()
    U64, sg64, Vt64 = outputs()
    fp64 = None
    if not args.no_fp64:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        _, st64 = R.rand_svd_dev(A, k, 1e-6, p, U64, sg64, Vt64, o64)
        t1.record(stream)
        torch.cuda.synchronize()
        ms64 = t0.elapsed_time(t1)
        fp64 = {"value": 1e3 / ms64, "unit": UNIT, "ms_per_solve": ms64,
                "stages_ms": {"range_finder": st64["ms_sketch"], "projection": st64["ms_factor"],
                              "svd_finish": st64["ms_solve"]}}

    # L2 flush between steps when A fits in L2 (a 512 MB write, outside the per-step events)
    a_bytes = m * n * (4 if wl["f32"] else 8)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev) if a_bytes < (256 << 20) else None
    clocks = ClockSampler(local)
    clocks.start()
    clocks.wait_first()
    for _ in range(args.warmup):
        R.rand_svd_dev(A, k, 1e-6, p, U, sg, Vt, o)
    torch.cuda.synchronize()
    barrier(ws)
    launches0 = lib.rnla_kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stages = []
    for i in range(args.steps):
        if flush is not None:
            flush.fill_(i & 255)
        ev[i][0].record(stream)
        _, st = R.rand_svd_dev(A, k, 1e-6, p, U, sg, Vt, o)
        ev[i][1].record(stream)
        stages.append((st["ms_sketch"], st["ms_factor"], st["ms_solve"], st["svd_sweeps"]))
    torch.cuda.synchronize()
    launches = lib.rnla_kernel_launches() - launches0
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    ms_max = max_over_ranks(ms, ws)
    value = ws * args.steps / (ms_max / 1e3)

    # accuracy: top-k sigma against the FP64 path with the same Omega, and
    # the approximation error ||A - U S V^T||_F of both
    acc = {}
    Ad = A.double()
    err = float((Ad - (U[:, :k] * sg[:k]) @ Vt[:k]).norm())
    acc["approx_error_fro"] = err
    if fp64:
        s1, s0 = sg[:k], sg64[:k]
        acc["topk_sigma_max_rel_err_vs_fp64"] = float(((s1 - s0).abs() / s0).max())
        acc["approx_error_fro_fp64_path"] = float((Ad - (U64[:, :k] * s0) @ Vt64[:k]).norm())
    acc["U_orthonormality"] = float((U[:, :k].t() @ U[:, :k] - torch.eye(k, device=dev, dtype=torch.float64)).abs().max())
    del Ad

    peaks, peak_src = load_peaks()
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    rf = sum(x[0] for x in stages) / len(stages)
    pr = sum(x[1] for x in stages) / len(stages)
    fin = sum(x[2] for x in stages) / len(stages)
    # the range finder streams A (as bf16 planes) 2q + 1 times and the
    # projection once more; algorithmic bytes: A's own size per pass
    passes = 2 * q + 2
    rf_flops = 2.0 * m * n * l * (2 * q + 1)
    esz = 4 if wl["f32"] else 8
    rf_gbs = (2 * q + 1) * m * n * esz / (rf / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "split-bf16 tcgen05 GEMMs (2 planes power iterations, 3 planes projection/Gram) + FP64 Cholesky/SVD",
        "data": "synthetic (seeded torch CUDA generator)",
        "config": workload_config(args, wl, ws),
        "path": "BF16X rand_svd (RandNLA mode): split-bf16 tensor-core range finder, CholeskyQR2, FP64 SVD finish",
        "accuracy": acc,
        "stages": {"range_finder_ms": rf, "projection_ms": pr, "svd_finish_ms": fin, "passes_over_A": passes,
                   "jacobi_sweeps": stages[-1][3]},
        "fp64_path": fp64,
        "speedup_vs_fp64_path": (value / ws) / fp64["value"] if fp64 else None,
        "e2e": None,
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "kernel": "bfx_gemm_kernel (range-finder products, algorithmic 2 m n l "
                                                  "flops each; 3 plane pairs at level 2)",
                     "achieved": rf_flops / (rf / 1e3) / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": rf_flops / (rf / 1e3) / 1e12 / bf16_peak, "traffic": None, "peak_source": peak_src,
                     "range_finder_hbm_gbs_equivalent": rf_gbs, "hbm_peak": hbm_peak},
        "clocks": clk,
    }
    if not args.no_e2e:
        dt = torch.float32 if wl["f32"] else torch.float64
        Ah = torch.empty((n, m), dtype=dt, pin_memory=True).t()
        Ah.copy_(A.cpu())
        Uh = torch.empty((l, m), dtype=torch.float64, pin_memory=True).t()
        sh = torch.empty(l, dtype=torch.float64, pin_memory=True)
        Vh = torch.empty((n, l), dtype=torch.float64, pin_memory=True).t()
        Ad_ = torch.empty_like(A)
        Ud, sd, Vd = outputs()

        def e2e_call():
            Ad_.copy_(Ah, non_blocking=True)
            R.rand_svd_dev(Ad_, k, 1e-6, p, Ud, sd, Vd, o)
            Uh.copy_(Ud, non_blocking=True)
            sh.copy_(sd, non_blocking=True)
            Vh.copy_(Vd, non_blocking=True)
            torch.cuda.synchronize()

        ke = max(5, args.steps)
        t, call_ms = time_host_calls(e2e_call, ke, args.warmup, ws)
        line["e2e"] = {"value": ws * ke / t, "unit": UNIT, "h2d_bytes_per_step": m * n * esz,
                       "d2h_bytes_per_step": 8 * (m * l + l + l * n), "steps": ke, "call_ms": call_ms,
                       "api": "rnla_rand_svd_dev with pinned host copies in and out on the same stream",
                       "pinned_h2d_gbs_of_A": pinned_h2d_gbs(Ah, dev)}
    return line


def svd_cpu_child(args):
    """`bench.py --cpu-leg port --workload *_svd`: the oracle restatement of the
    reference rand_svd (lora_drivers.rs:30-69, reference semantics: the
    tsog1 data flow of lora_helpers.rs:58-105) at full size, one JSON line per
    solve, at most --steps solves or four minutes."""
    import numpy as np
    from oracle import oracle as O
    wl = workload(args)
    m, n, r = wl["m"], wl["n"], wl["rank"]
    su, sv, se = wl["seeds"]
    U = np.linalg.qr(np.random.default_rng(su).standard_normal((m, r)))[0]
    V = np.linalg.qr(np.random.default_rng(sv).standard_normal((n, r)))[0]
    i = np.arange(r)
    sig = np.exp(-i / 64.0) if wl["decay"].startswith("exp") else 10.0 ** (-i / 100.0)
    A = (U * sig) @ V.T
    del U, V
    if wl["noise"] > 0:
        A += (wl["noise"] / (math.sqrt(m) + math.sqrt(n))) * np.random.default_rng(se).standard_normal((m, n))
    if wl["f32"]:
        A = A.astype(np.float32).astype(np.float64)
    A = np.asfortranarray(A)
    O.rand_svd(A[: max(wl["k"] + wl["p"], m // 64)], wl["k"], 1e-6, wl["p"])     # load libraries
    t_all = time.perf_counter()
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        O.rand_svd(A, wl["k"], 1e-6, wl["p"])
        print(json.dumps({"seconds": time.perf_counter() - t0}), flush=True)
        if time.perf_counter() - t_all > 240.0:
            break


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
    tol, sf = 1e-12, 4.0
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
# CPU legs: the oracle's restatement of the reference path at full size
# ---------------------------------------------------------------------------
def make_problem_host(wl):
    """The workload's construction on the host with numpy (seeded): A =
    U diag(sigma) V^T (FP32-rounded for the FP32 workload, then widened: the
    reference takes FP64 matrices), b = A x* + noise."""
    import numpy as np
    m, n = wl["m"], wl["n"]
    su, sv, sx, sb = wl["seeds"]
    U = np.linalg.qr(np.random.default_rng(su).standard_normal((m, n)))[0]
    V = np.linalg.qr(np.random.default_rng(sv).standard_normal((n, n)))[0]
    A = (U * np.logspace(0, -math.log10(wl["kappa"]), n)) @ V.T
    del U
    if wl["f32"]:
        A = A.astype(np.float32).astype(np.float64)
    A = np.asfortranarray(A)
    b = A @ np.random.default_rng(sx).standard_normal(n) + wl["noise"] * np.random.default_rng(sb).standard_normal(m)
    return A, b


def cpu_child(args):
    if args.workload in SVD_WORKLOADS:
        return svd_cpu_child(args)
    return ls_cpu_child(args)


def ls_cpu_child(args):
    """`bench.py --cpu-leg port`: runs in its own process; prints one JSON
    line per full-size solve of the oracle port (sketch_and_precondition.rs:
    26-59: Gaussian S, S a, Householder QR, R^-1, explicit a R^-1, CGLS to the
    workload's tolerance, x = R^-1 z), stopping after --steps solves or once
    four minutes have passed."""
    import numpy as np
    from oracle import oracle as O
    wl = workload(args)
    m, n = wl["m"], wl["n"]
    A, b = make_problem_host(wl)
    ms = max(4 * int(wl["sampling_factor"] * n), m // 64)
    O.blendenpik_overdetermined_blocked(A[:ms], b[:ms], wl["tol"], 10, wl["sampling_factor"])   # load libraries
    t_all = time.perf_counter()
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        x, it = O.blendenpik_overdetermined_blocked(A, b, wl["tol"], 10 * n, wl["sampling_factor"],
                                                    return_iters=True)
        t = time.perf_counter() - t0
        rr = float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))
        print(json.dumps({"seconds": t, "cgls_iterations": it, "rel_residual": rr}), flush=True)
        if time.perf_counter() - t_all > 240.0:
            break


def cpu_port_runs(args, steps):
    """Full-size oracle-port solves in a child process (capped): returns
    (list of per-solve results, note)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-leg", "port", "--workload", args.workload,
           "--steps", str(steps)]
    if args.m:
        cmd += ["--m", str(args.m)]
    if args.n:
        cmd += ["--n", str(args.n)]
    env = dict(os.environ)
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    env["CUDA_VISIBLE_DEVICES"] = ""
    proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env)
    note = "finished"
    try:
        out, err = proc.communicate(timeout=CPU_CAP_S + 300.0)   # + problem generation
    except subprocess.TimeoutExpired:
        proc.kill()
        out, err = proc.communicate()
        note = "not finished (cap %d s)" % CPU_CAP_S
    runs = [json.loads(ln) for ln in out.splitlines() if ln.startswith("{")]
    if proc.returncode not in (0, None) and note == "finished":
        note = "failed: " + (err.strip().splitlines() or ["?"])[-1][:200]
    return runs, note


def run_reference(args, rank, ws):
    """The reference arm: the oracle's CPU restatement of the reference's
    path at the workload's full size on the host cores, rank 0 only.  A
    step is one full solve; the steps stop after four minutes (at least one
    solve), and the line says how many ran."""
    if rank != 0:
        return None
    wl = workload(args)
    runs, note = cpu_port_runs(args, args.steps)
    cores = os.cpu_count()
    line = {
        "metric": METRIC, "value": None, "unit": UNIT, "n_gpus": ws, "steps": len(runs),
        "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy generator)",
        "impl": "reference", "config": workload_config(args, wl, ws),
        "algorithm": ("the reference rand_svd (lora_drivers.rs:30-69) with its tsog1 / RF1 / QB1 data flow "
                      "(lora_helpers.rs:17-105), k=%d, s=%d" % (wl["k"], wl["p"]))
                     if args.workload in SVD_WORKLOADS else
                     ("the reference's data flow (sketch_and_precondition.rs:26-59): dense Gaussian S "
                      "(generated in column blocks), S a, Householder QR, explicit R^-1 and a R^-1, CGLS to "
                      "tolerance %g, x = R^-1 z" % wl["tol"]),
        "status": note, "runs": runs,
    }
    if runs:
        sec = sum(r["seconds"] for r in runs) / len(runs)
        v = 1.0 / sec
        line.update({"value": v, "ms_per_step": 1e3 * sec})
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "%d full-size solve(s) of the oracle restatement (numpy/LAPACK on "
                                          "all %d host threads, C sketch generator on %d threads); no "
                                          "sampling or extrapolation" % (len(runs), cores, cores)}
        line["e2e"] = {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    return line


def main():
    args = parse()
    if args.cpu_leg:
        cpu_child(args)
        return
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
    if args.workload in SVD_WORKLOADS:
        line = run_svd(args, rank, local, ws)
    else:
        line = run_ours(args, rank, local, ws)
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count()
        runs, note = cpu_port_runs(args, 1)
        cb = {"value": None, "unit": UNIT, "cores": cores, "kind": "port", "status": note}
        if runs:
            cb["value"] = 1.0 / runs[0]["seconds"]
            if args.workload in SVD_WORKLOADS:
                cb["sample"] = ("one full-size rand_svd (%.1f s) of the oracle restatement of lora_drivers.rs:30-69 "
                                "with the reference's tsog1 data flow (numpy/LAPACK on all %d host threads); no "
                                "sampling or extrapolation" % (runs[0]["seconds"], cores))
            else:
                cb["sample"] = ("one full-size solve (%.1f s, %d CGLS iterations) of the oracle restatement of "
                                "sketch_and_precondition.rs:26-59 (numpy/LAPACK on all %d host threads, C sketch "
                                "generator); no sampling or extrapolation"
                                % (runs[0]["seconds"], runs[0]["cgls_iterations"], cores))
        al = line.get("accuracy_lapack")
        if al:
            cb["lapack_qr_lstsq"] = {"value": 1.0 / al["seconds"], "unit": UNIT, "cores": cores,
                                     "sample": "numpy.linalg.qr + triangular solve (LAPACK geqrf/orgqr, FP64, "
                                               "all host threads) on the same A, full size, %.1f s"
                                               % al["seconds"]}
        line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
