"""sketch_and_precondition::lsrn_overdetermined on the GPU.  The FP64 path
uses the same sketch (Philox key 0) as the oracle restatement, whose
preconditioner is V Sigma^+ from the SVD of S a; the GPU forms it as
R^-1 U_R and runs CGLS on A R^-1 from 0 (the same iterates rotated), so the
iteration counts agree within one and the residuals within 1e-10."""
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


@pytest.mark.parametrize("m,n,kappa", [(2000, 40, 1e6), (100, 10, 1e4), (5000, 120, 1e8)])
def test_cgls_matches_oracle(rnla, m, n, kappa):
    A, b = _problem(m, n, kappa, 1e-6)
    x, st = rnla.lsrn_overdetermined(A, b, 1e-10, 1000, 4.0 if m > 100 else 1.5, return_stats=True)
    xo, it = O.lsrn_overdetermined(A, b, 1e-10, 1000, 4.0 if m > 100 else 1.5, return_iters=True)
    assert x.shape == (n, 1)
    assert abs(st["iterations"] - it) <= 1
    assert abs(_relres(A, x, b) - _relres(A, xo, b)) < 1e-10


def test_bf16x_lsqr_vs_lapack(rnla):
    A, b = _problem(30000, 300, 1e8, 1e-6)
    o = rnla.options(precision=rnla.Precision.BF16X, inner_solver=rnla.InnerSolver.LSQR,
                     atol=1e-14, btol=1e-14, seed=7)
    x, st = rnla.lsrn_overdetermined(A, b, 1e-12, 2000, 4.0, o, return_stats=True)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    assert abs(_relres(A, x, b) - _relres(A, xl, b)) < 1e-10
    assert 0 < st["iterations"] < 500


def test_errors(rnla):
    A, b = _problem(100, 10, 1e3, 1e-4)
    with pytest.raises(rnla.NotOverdetermined):
        rnla.lsrn_overdetermined(A[:5], b[:5], 1e-4, 1000, 1.5)
    # the reference's own error cases (sketch_and_precondition.rs:369-378)
    for eps, l, sf in ((1e-4, 1000, 0.5), (-1e-4, 1000, 1.5), (0.0, 1000, 1.5), (1e-4, 0, 0.5)):
        with pytest.raises(rnla.InvalidParameters):
            rnla.lsrn_overdetermined(A, b, eps, l, sf)


def test_singular_sketch_is_an_error(rnla):
    """A zero column makes the sketch exactly singular: the reference would
    drop that singular direction; this library reports SingularMatrix."""
    A, b = _problem(800, 12, 1e3, 1e-4)
    A[:, 3] = 0.0
    with pytest.raises(rnla.SingularMatrix):
        rnla.lsrn_overdetermined(A, b, 1e-8, 1000, 4.0)
