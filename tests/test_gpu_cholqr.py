"""The blocked cooperative Cholesky and the CholeskyQR factorization of the
sketch.

* rand_svd on the tensor cores with l = k + p >= 128, where every
  CholeskyQR of the range finder, the Gram of the final basis and the
  small-SVD finish run the blocked Cholesky: singular values against the
  oracle's FP64 restatement of lora_drivers.rs:30-69 on the same Omega;
* blendenpik BF16X + LSQR at a shape whose sketch takes the wide-sketch
  branch (n = 1000, d = 4000): the CholeskyQR R (orth = 0) against the
  float-float Householder TSQR R (orth = 1) -- same iteration count within
  2, relative residuals within 1e-12, both solutions at LAPACK's backward
  error; at kappa = 1e8 the CholeskyQR R is refused (its Gram's rounding
  would reach the sketch's smallest singular value) and the TSQR runs.
Reference: sketch_and_precondition.rs:50-58 (QR of S a, z_0 = Q^T S b,
R^-1, the preconditioned solve)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_rand_svd_tensor_core_wide_basis(rnla):
    import torch
    m, n, k, p = 6000, 3000, 150, 20
    l = k + p
    sig = np.exp(-np.arange(n) / 40.0)
    A = O.make_lowrank_test_matrix(m, n, sig, 22, 23)
    At = torch.from_numpy(A).cuda().t().contiguous().t()
    o = rnla.options(precision=rnla.Precision.BF16X, mode=rnla.Mode.RandNLA, power_iters=2, seed=5)
    U = torch.zeros((l, m), dtype=torch.float64, device="cuda").t()
    sg = torch.zeros(l, dtype=torch.float64, device="cuda")
    Vt = torch.zeros((n, l), dtype=torch.float64, device="cuda").t()
    r, _ = rnla.rand_svd_dev(At, k, 1e-6, p, U, sg, Vt, o)
    assert r == k
    _, so, _ = O.rand_svd_randnla(A, k, p, 2, seed=5)
    s = sg[:k].cpu().numpy()
    assert np.max(np.abs(s - so) / so) < 1e-6
    Uk = U[:, :k].cpu().numpy()
    assert np.linalg.norm(Uk.T @ Uk - np.eye(k)) < 1e-5


def _ls_problem(m, n, kappa, seed):
    A = O.make_lowrank_test_matrix(m, n, np.logspace(0, -np.log10(kappa), n), seed + 1, seed + 2)
    rng = np.random.default_rng(seed + 3)
    b = A @ rng.standard_normal(n) + 1e-8 * rng.standard_normal(m)
    return A, b


def _solve(rnla, At, bt, n, orth):
    import torch
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    o = rnla.options(precision=rnla.Precision.BF16X, inner_solver=rnla.InnerSolver.LSQR, atol=1e-10, btol=1e-10,
                     seed=42, orth=orth)
    st = rnla.blendenpik_dev(At, bt, x, 1e-10, 10 * n, 4.0, o)
    return x.cpu().numpy(), st


def _backward_error(A, x, b):
    r = b - A @ x
    return np.linalg.norm(A.T @ r) / (np.linalg.norm(A) * np.linalg.norm(r)), np.linalg.norm(r) / np.linalg.norm(b)


@pytest.mark.parametrize("f32", [False, True])
def test_blendenpik_cholqr_matches_tsqr(rnla, f32):
    import torch
    m, n = 40000, 1000
    A, b = _ls_problem(m, n, 1e6, 7)
    if f32:
        A = A.astype(np.float32).astype(np.float64)
    At = torch.from_numpy(A.astype(np.float32) if f32 else A).cuda().t().contiguous().t()
    bt = torch.from_numpy(b).cuda()
    xc, stc = _solve(rnla, At, bt, n, 0)
    xh, sth = _solve(rnla, At, bt, n, 1)
    assert stc["orth_fallbacks"] == 0 and sth["orth_fallbacks"] == 0
    assert stc["sketch_rows"] == 4000
    assert abs(stc["iterations"] - sth["iterations"]) <= 2, (stc["iterations"], sth["iterations"])
    bec, rc = _backward_error(A, xc, b)
    beh, rh = _backward_error(A, xh, b)
    assert abs(rc - rh) < 1e-12, (rc, rh)
    # both at the float-float iterate's rounding floor (2^-48 ||b|| / ||r||)
    floor = 2.0 ** -48 / rh
    assert bec <= 1e3 * floor and beh <= 1e3 * floor, (bec, beh, floor)


def test_blendenpik_cholqr_refused_when_ill_conditioned(rnla):
    import torch
    m, n = 40000, 1000
    A, b = _ls_problem(m, n, 1e8, 9)
    At = torch.from_numpy(A).cuda().t().contiguous().t()
    bt = torch.from_numpy(b).cuda()
    x, st = _solve(rnla, At, bt, n, 0)
    assert st["orth_fallbacks"] == 1
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    _, r = _backward_error(A, x, b)
    _, rl = _backward_error(A, xl, b)
    assert abs(r - rl) < 1e-10, (r, rl)
