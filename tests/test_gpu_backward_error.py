"""Least-squares parity beyond the residual.

The normwise backward error ||A^T r|| / (||A||_F ||r||) of a computed x
cannot fall below the rounding of x itself: with unit roundoff u of the
arithmetic that forms x, its floor is about phi = u ||b|| / ||r||
(~1e-11 for FP64 at these noise levels).  The residual is formed here in
double-double, far below that floor.  Checked, for blendenpik and lsrn,
FP64 and BF16X paths, A stored in FP64 or FP32:
  * FP64 path: backward error <= 1e3 phi_64 (phi_64 = 2^-53 ||b|| / ||r||);
  * BF16X path: its iterate is float-float (~2^-48), so backward error
    <= 1e3 phi_48;
  * where kappa^2 u is far below the tolerance (kappa <= 1e3) the solution
    matches LAPACK's: ||x - x_LAPACK|| / ||x_LAPACK|| <= 1e-9.
At the bench shapes -- the plain workload (100000 x 500 FP64, kappa 1e8) and
the precision workload at its full size (1048576 x 1024 FP32, kappa 1e6,
d = 4096) -- the BF16X solve's relative residual is within 1e-10 of the
plain FP64 GPU path's, the FP64 path's backward error is within 10 x the
LSQR tolerance (or 1e3 phi_64) and the BF16X path's within 64 x the FP64
path's (the ratio of the two unit roundoffs is 32).

The LAPACK reference solves the matrix as stored (FP32 entries widened);
the reference crate itself cannot run here, so these compare against
LAPACK and the FP64 GPU path (which matches the oracle restatement of
sketch_and_precondition.rs:26-59 in test_gpu_blendenpik.py)."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _problem(m, n, kappa, noise, seed):
    A = O.make_lowrank_test_matrix(m, n, np.logspace(0, -np.log10(kappa), n), seed + 1, seed + 2)
    rng = np.random.default_rng(seed + 3)
    b = A @ rng.standard_normal(n) + noise * rng.standard_normal(m)
    return A, b


def _residual_dd(A, x, b):
    """b - A x in double-double (Dekker's TwoProduct and Knuth's TwoSum per
    column of A), rounded to FP64."""
    sh = np.array(b, dtype=np.float64)
    sl = np.zeros_like(sh)
    c = 134217729.0          # 2^27 + 1: Veltkamp split into 26-bit halves

    def split(a):
        t = c * a
        hi = t - (t - a)
        return hi, a - hi

    for j in range(A.shape[1]):
        a = np.ascontiguousarray(A[:, j])
        xj = -float(x[j])
        p = a * xj
        ah, al = split(a)
        xh, xl = split(np.float64(xj))
        e = ((ah * xh - p) + ah * xl + al * xh) + al * xl      # p + e = a xj exactly
        s = sh + p
        bp = s - sh
        t = (sh - (s - bp)) + (p - bp)
        sh = s
        sl = sl + (t + e)
    return sh + sl


def _errors(A, x, b, xl):
    x = np.ravel(x)
    r = _residual_dd(A, x, b)
    rn = np.linalg.norm(r)
    be = np.linalg.norm(A.T @ r) / (np.linalg.norm(A) * rn)
    return be, np.linalg.norm(x - xl) / np.linalg.norm(xl), np.linalg.norm(b) / rn


def _opts(rnla, prec):
    return rnla.options(precision=prec, inner_solver=rnla.InnerSolver.LSQR, atol=1e-14, btol=1e-14, seed=11)


@pytest.mark.parametrize("driver", ["blendenpik", "lsrn"])
@pytest.mark.parametrize("prec", ["FP64", "BF16X"])
@pytest.mark.parametrize("f32", [False, True])
@pytest.mark.parametrize("m,n,kappa", [(20000, 100, 1e2), (30000, 300, 1e3), (40000, 1000, 1e2)])
def test_backward_error_and_solution(rnla, driver, prec, f32, m, n, kappa):
    import torch
    A, b = _problem(m, n, kappa, 1e-6, seed=n)
    if f32:
        A = A.astype(np.float32).astype(np.float64)
    At = torch.from_numpy(A.astype(np.float32) if f32 else A).cuda().t().contiguous().t()
    bt = torch.from_numpy(b).cuda()
    xt = torch.zeros(n, dtype=torch.float64, device="cuda")
    o = _opts(rnla, getattr(rnla.Precision, prec))
    if driver == "blendenpik":
        st = rnla.blendenpik_dev(At, bt, xt, 1e-14, 4 * n, 4.0, o)
    else:
        st = rnla.lsrn_dev(At, bt, xt, 1e-14, 4 * n, 4.0, o)
    assert st["precision_used"] == int(getattr(rnla.Precision, prec))
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    be, xe, b_over_r = _errors(A, xt.cpu().numpy(), b, xl)
    u = 2.0 ** -53 if prec == "FP64" else 2.0 ** -48
    assert be <= 1e3 * u * b_over_r, (be, u * b_over_r)
    assert xe <= 1e-9, xe


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


@pytest.mark.parametrize("name", ["plain_ls", "precision_ls"])
def test_bench_workloads_full_size(rnla, name):
    """The bench's own workloads at full size: BF16X against the plain FP64
    GPU path on the same inputs (the bench line reports the same fields)."""
    import torch
    bench = _bench()
    args = bench.parse(["--workload", name])
    wl = bench.workload(args)
    dev = torch.device("cuda", 0)
    A, b = bench.make_problem(wl, dev)
    n = wl["n"]
    tol = wl["tol"]
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    x64 = torch.zeros_like(x)
    o = rnla.options(precision=rnla.Precision.BF16X, inner_solver=rnla.InnerSolver.LSQR, atol=tol, btol=tol,
                     seed=42)
    o64 = rnla.options(precision=rnla.Precision.FP64, inner_solver=rnla.InnerSolver.LSQR, atol=tol, btol=tol,
                       seed=42)
    st = rnla.blendenpik_dev(A, b, x, tol, 10 * n, wl["sampling_factor"], o)
    st64 = rnla.blendenpik_dev(A, b, x64, tol, 10 * n, wl["sampling_factor"], o64)
    a = bench.accuracy(A, x, b)
    a64 = bench.accuracy(A, x64, b)
    assert abs(a["rel_residual"] - a64["rel_residual"]) < 1e-10, (a, a64)
    # LSQR stops at ||(A M)^T r|| / (||A M|| ||r||) <= tol; on A itself that is within a small factor,
    # or at the rounding floor 2^-53 ||b|| / ||r|| of an FP64 iterate
    floor64 = 2.0 ** -53 / a64["rel_residual"]
    assert a64["backward_error"] <= max(10 * tol, 1e3 * floor64), a64
    # the float-float iterate carries 2^-48 against FP64's 2^-53
    assert a["backward_error"] <= 64 * a64["backward_error"], (a, a64)
    assert 0 < st["iterations"] < 200 and abs(st["iterations"] - st64["iterations"]) <= 3
    assert st["precision_used"] == int(rnla.Precision.BF16X)
    del A
    torch.cuda.empty_cache()
