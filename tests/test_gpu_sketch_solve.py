"""sketch_and_solve::sketched_least_squares_qr / _svd on the GPU against the
oracle restatement with the same Gaussian sketch (Philox key 0): the FP64
path solves the same sketched problem, so x agrees to 1e-8 relative; the
tensor-core (BF16X) path uses the quantised sketch, so it is held to the
sketch-and-solve guarantee against LAPACK's least-squares residual."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _problem(m, n, noise, seed):
    """The reference tests' construction (sketch_and_solve.rs:82-97): a
    random hypothesis, y = data hypothesis, then noise added to the data."""
    rng = np.random.default_rng(seed)
    data = rng.standard_normal((m, n))
    hyp = rng.uniform(-100, 100, n)
    y = data @ hyp
    data = data + noise * rng.standard_normal((m, n))
    return data, y


@pytest.mark.parametrize("m,n", [(400, 20), (301, 29), (4000, 100)])
@pytest.mark.parametrize("svd", [False, True])
def test_fp64_matches_oracle(rnla, m, n, svd):
    A, y = _problem(m, n, 0.01, m + n)
    f = rnla.sketched_least_squares_svd if svd else rnla.sketched_least_squares_qr
    g = O.sketched_least_squares_svd if svd else O.sketched_least_squares_qr
    x = f(A, y)
    xo = g(A, y)
    assert x.shape == (n, 1)
    assert np.linalg.norm(x.ravel() - xo) <= 1e-8 * np.linalg.norm(xo)


@pytest.mark.parametrize("svd", [False, True])
def test_bf16x_residual(rnla, svd):
    A, y = _problem(40000, 200, 0.01, 7)
    o = rnla.options(precision=rnla.Precision.BF16X)
    f = rnla.sketched_least_squares_svd if svd else rnla.sketched_least_squares_qr
    x = f(A, y, o)
    xl = np.linalg.lstsq(A, y, rcond=None)[0]
    r = np.linalg.norm(A @ x.ravel() - y)
    rl = np.linalg.norm(A @ xl - y)
    # d = m/4 = 10000 rows for n = 200: subspace distortion sqrt(n/d) ~ 0.14
    assert r <= 1.5 * rl


def _zero_column_problem():
    A, y = _problem(800, 12, 0.01, 3)
    A[:, 5] = 0.0
    xl = np.linalg.lstsq(A, y, rcond=None)[0]
    return A, y, np.linalg.norm(A @ xl - y)


def test_qr_zero_pivot_rule(rnla):
    """An all-zero column of A: its sketch column is exactly zero, the
    Householder step leaves it zero (tau = 0), so R has an exactly zero
    pivot and the back substitution (solvers.rs:22-41) gives that component
    0; the rest is the sketched least-squares solution of the other columns."""
    A, y, rl = _zero_column_problem()
    x = rnla.sketched_least_squares_qr(A, y).ravel()
    assert np.all(np.isfinite(x))
    assert x[5] == 0.0
    assert np.linalg.norm(A @ x - y) <= 1.6 * rl


def test_device_entry_matches_host(rnla):
    import torch
    A, y = _problem(2000, 40, 0.01, 11)
    At = torch.from_numpy(np.asfortranarray(A)).cuda().t().contiguous().t()
    yt = torch.from_numpy(y).cuda()
    for svd in (False, True):
        xt = torch.zeros(40, dtype=torch.float64, device="cuda")
        rnla.sketched_least_squares_dev(At, yt, xt, use_svd=svd)
        xh = (rnla.sketched_least_squares_svd if svd else rnla.sketched_least_squares_qr)(A, y)
        np.testing.assert_array_equal(xt.cpu().numpy(), xh.ravel())


def test_too_few_sketch_rows(rnla):
    A, y = _problem(40, 11, 0.01, 1)      # m / 4 = 10 < n
    with pytest.raises(rnla.InvalidDimensions):
        rnla.sketched_least_squares_qr(A, y)
    with pytest.raises(rnla.InvalidDimensions):
        rnla.sketched_least_squares_svd(A, y)
