"""The BF16X fast path of blendenpik_overdetermined (tensor-core sketch,
float-float QR and R^-1, float-float LSQR) against LAPACK's least-squares
solution, over the shapes that select different kernel variants:

  n <= 64       LSQR fused roles, one column chunk per lane, 8 rows per warp
  n <= 128      two chunks per lane
  n <= 256      four chunks, 4 rows per warp
  n <= 512      eight chunks, 2 rows per warp (the bench shape)
  512 < n       LSQR split roles; at n = 650 the QR's CTAs own two column
                blocks each, at n = 1000 the sketch no longer fits shared memory
                and the FP64 Householder QR takes over

and the host-pointer entry, whose matrix arrives in column chunks that the
sketch consumes tile by tile (including a padded leading dimension and a
column count that is not a multiple of the 64-column tile).  Tolerance: the
relative residual within 1e-10 (absolute) of LAPACK's."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _problem(m, n, kappa, noise, seed=0):
    A = O.make_lowrank_test_matrix(m, n, np.logspace(0, -np.log10(kappa), n), seed + 1, seed + 2)
    rng = np.random.default_rng(seed + 3)
    b = A @ rng.standard_normal(n) + noise * rng.standard_normal(m)
    return A, b


def _relres(A, x, b):
    return np.linalg.norm(A @ np.ravel(x) - b) / np.linalg.norm(b)


def _fast(rnla, solver=None, seed=42):
    return rnla.options(precision=rnla.Precision.BF16X,
                        inner_solver=solver if solver is not None else rnla.InnerSolver.LSQR,
                        atol=1e-14, btol=1e-14, seed=seed)


@pytest.mark.parametrize("m,n,kappa", [
    (5000, 1, 1.0),
    (6000, 33, 1e6),
    (8000, 100, 1e8),
    (12000, 250, 1e8),
    (30000, 500, 1e8),
    (30000, 650, 1e6),
    (40000, 1000, 1e4),
])
def test_bf16x_lsqr_vs_lapack(rnla, m, n, kappa):
    A, b = _problem(m, n, kappa, 1e-6)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-12, 2000, 4.0, _fast(rnla), return_stats=True)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    assert abs(_relres(A, x, b) - _relres(A, xl, b)) < 1e-10
    assert st["precision_used"] == int(rnla.Precision.BF16X)
    assert 0 < st["iterations"] < 500


def test_bf16x_matches_fp64_path_iterations(rnla):
    """The float-float solver follows the FP64 LSQR: same stopping rule, the
    iteration count within one of the FP64 path on the same sketch seed."""
    A, b = _problem(20000, 300, 1e8, 1e-6)
    _, st = rnla.blendenpik_overdetermined(A, b, 1e-12, 2000, 4.0, _fast(rnla), return_stats=True)
    o64 = rnla.options(precision=rnla.Precision.FP64, inner_solver=rnla.InnerSolver.LSQR,
                       atol=1e-14, btol=1e-14, seed=42)
    _, st64 = rnla.blendenpik_overdetermined(A, b, 1e-12, 2000, 4.0, o64, return_stats=True)
    assert abs(st["iterations"] - st64["iterations"]) <= 1


def test_bf16x_cgls_inner_solver(rnla):
    A, b = _problem(20000, 150, 1e6, 1e-6)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-12, 2000, 4.0, _fast(rnla, rnla.InnerSolver.CGLS),
                                           return_stats=True)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    assert abs(_relres(A, x, b) - _relres(A, xl, b)) < 1e-10


def test_bf16x_host_entry_padded_lda(rnla):
    """rnla_blendenpik_overdetermined_ex with lda > m and n = 130 (three column
    chunks, the last one partial): the chunked upload feeds the sketch."""
    m, n, lda = 9000, 130, 9013
    A, b = _problem(m, n, 1e6, 1e-6)
    Ap = np.zeros((n, lda))                   # column-major storage with padding rows
    Ap[:, :m] = A.T
    Ap[:, m:] = np.nan                        # padding must never be read
    x = np.zeros(n)
    st = rnla.Stats()
    o = _fast(rnla)
    L = rnla.lib()
    rc = L.rnla_blendenpik_overdetermined_ex(
        ctypes.c_void_p(Ap.ctypes.data), m, n, lda, ctypes.c_void_p(np.ascontiguousarray(b).ctypes.data),
        1e-12, 2000, 4.0, ctypes.byref(o), ctypes.c_void_p(x.ctypes.data), ctypes.byref(st))
    assert rc == 0, L.rnla_last_error_message()
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    assert abs(_relres(A, x, b) - _relres(A, xl, b)) < 1e-10


def test_bf16x_host_and_device_entries_agree(rnla):
    """Same seed, same data: the chunked host-pointer path and the
    device-resident path compute the same sketch and the same solution."""
    import torch
    A, b = _problem(10000, 200, 1e8, 1e-6)
    o = _fast(rnla)
    xh, sth = rnla.blendenpik_overdetermined(A, b, 1e-12, 2000, 4.0, o, return_stats=True)
    At = torch.from_numpy(np.asfortranarray(A)).cuda().t().contiguous().t()
    bt = torch.from_numpy(b).cuda()
    xt = torch.zeros(200, dtype=torch.float64, device="cuda")
    std = rnla.blendenpik_dev(At, bt, xt, 1e-12, 2000, 4.0, o)
    assert sth["iterations"] == std["iterations"]
    np.testing.assert_array_equal(np.ravel(xh), xt.cpu().numpy())


@pytest.mark.parametrize("m,n,kappa", [(5000, 1, 1.0), (9000, 77, 1e6), (12000, 200, 1e6), (20000, 511, 1e4),
                                       (40000, 1024, 1e6)])
def test_bf16x_lsqr_fp32_storage(rnla, m, n, kappa):
    """A stored in FP32: the LSQR streams a row-major FP32 copy (4 bytes per
    element; kernel variants with 1, 2, 4 and 8 column chunks per lane)."""
    import torch
    A, b = _problem(m, n, kappa, 1e-6)
    A32 = A.astype(np.float32)
    A64 = A32.astype(np.float64)
    At = torch.from_numpy(A32).cuda().t().contiguous().t()
    bt = torch.from_numpy(b).cuda()
    xt = torch.zeros(n, dtype=torch.float64, device="cuda")
    st = rnla.blendenpik_dev(At, bt, xt, 1e-12, 2000, 4.0, _fast(rnla))
    x = xt.cpu().numpy()
    xl = np.linalg.lstsq(A64, b, rcond=None)[0]
    assert abs(_relres(A64, x, b) - _relres(A64, xl, b)) < 1e-10
    # backward error against its floor 2^-48 ||b|| / ||r|| for a float-float iterate
    r = b - A64 @ x
    be = np.linalg.norm(A64.T @ r) / (np.linalg.norm(A64) * np.linalg.norm(r))
    assert be <= 1e3 * 2.0 ** -48 * np.linalg.norm(b) / np.linalg.norm(r), be
    assert st["precision_used"] == int(rnla.Precision.BF16X)
    assert 0 < st["iterations"] < 500
