"""sketch_and_precondition::blendenpik_overdetermined on the GPU."""
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


def test_errors(rnla):
    A, b = _problem(100, 10, 1e3, 1e-4)
    with pytest.raises(rnla.NotOverdetermined):
        rnla.blendenpik_overdetermined(A[:5], b[:5], 1e-4, 1000, 1.5)
    for eps, l, sf in ((1e-4, 1000, 0.5), (-1e-4, 1000, 1.5), (0.0, 1000, 1.5), (1e-4, 0, 0.5)):
        with pytest.raises(rnla.InvalidParameters):
            rnla.blendenpik_overdetermined(A, b, eps, l, sf)


def test_reference_cgls_matches_oracle(rnla):
    """Same sketch (Philox key 0), same CGLS rule: same iterate count and solution."""
    A, b = _problem(2000, 40, 1e6, 1e-6)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-10, 1000, 4.0, return_stats=True)
    xo, it = O.blendenpik_overdetermined(A, b, 1e-10, 1000, 4.0, return_iters=True)
    assert abs(st["iterations"] - it) <= 1
    assert abs(_relres(A, x, b) - _relres(A, xo, b)) < 1e-10


def test_reference_test_shape(rnla):
    """sketch_and_precondition.rs:229-276 shape: m = 100, n = 10, sf = 1.5."""
    A, b = _problem(100, 10, 1e6, 1e-4)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-4, 1000, 1.5, return_stats=True)
    xo, it = O.blendenpik_overdetermined(A, b, 1e-4, 1000, 1.5, return_iters=True)
    assert x.shape == (10, 1)
    assert st["iterations"] == it
    np.testing.assert_allclose(x.ravel(), xo, rtol=1e-6)


@pytest.mark.parametrize("m,n,kappa", [(3000, 50, 1e8), (20000, 200, 1e6), (5000, 1, 1.0)])
def test_lsqr_inner_solver_vs_lapack(rnla, m, n, kappa):
    A, b = _problem(m, n, kappa, 1e-6)
    o = rnla.options(inner_solver=rnla.InnerSolver.LSQR, atol=1e-14, btol=1e-14, seed=42)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-12, 1000, 4.0, o, return_stats=True)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    assert abs(_relres(A, x, b) - _relres(A, xl, b)) < 1e-10
    assert st["iterations"] < 200


def test_lsqr_matches_oracle_iterates(rnla):
    A, b = _problem(4000, 60, 1e8, 1e-6)
    o = rnla.options(inner_solver=rnla.InnerSolver.LSQR, atol=1e-12, btol=1e-12, seed=3)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-12, 500, 4.0, o, return_stats=True)
    xo, res = O.blendenpik_lsqr(A, b, 4.0, 1e-12, 1e-12, 500, seed=3)
    assert st["istop"] == res[1]
    assert abs(st["iterations"] - res[2]) <= 1
    assert abs(_relres(A, x, b) - _relres(A, xo, b)) < 1e-10


def test_device_float32_input(rnla):
    import torch
    A, b = _problem(8000, 64, 1e4, 1e-6)
    A32 = A.astype(np.float32)
    At = torch.from_numpy(A32).cuda().t().contiguous().t()
    bt = torch.from_numpy(b).cuda()
    xt = torch.zeros(64, dtype=torch.float64, device="cuda")
    o = rnla.options(inner_solver=rnla.InnerSolver.LSQR, atol=1e-14, btol=1e-14)
    st = rnla.blendenpik_dev(At, bt, xt, 1e-12, 1000, 4.0, o)
    x = xt.cpu().numpy()
    A64 = A32.astype(np.float64)
    xl = np.linalg.lstsq(A64, b, rcond=None)[0]
    assert abs(_relres(A64, x, b) - _relres(A64, xl, b)) < 1e-10
