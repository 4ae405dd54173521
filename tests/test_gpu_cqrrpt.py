"""cqrrpt::sap_chol_qrcp on the GPU.  The FP64 path uses the same Gaussian
sketch (Philox key 0) as the oracle restatement, so the pivot order is the
same and Q, R agree to 1e-8; every path gives orthonormal Q and
a[:, j] = Q R (the reference test's checks, cqrrpt.rs:80-115, with tighter
tolerances)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _check_factorization(a, q, r, j, tol):
    n = a.shape[1]
    assert sorted(j) == list(range(n))
    np.testing.assert_allclose(q.T @ q, np.eye(n), atol=tol)
    np.testing.assert_allclose(q @ r, a[:, j], atol=tol * max(1.0, np.abs(a).max()))
    assert np.allclose(np.tril(r, -1), 0.0)


@pytest.mark.parametrize("m,n,d", [(100, 10, 50), (2000, 40, 200), (5000, 64, 64)])
def test_fp64_matches_oracle(rnla, m, n, d):
    rng = np.random.default_rng(m + n)
    a = rng.standard_normal((m, n)) * np.logspace(0, -4, n)
    q, r, j = rnla.sap_chol_qrcp(a, d)
    qo, ro, jo = O.sap_chol_qrcp(a, d)
    assert j == jo
    np.testing.assert_allclose(r, ro, rtol=0, atol=1e-8 * np.abs(ro).max())
    np.testing.assert_allclose(q, qo, rtol=0, atol=1e-8)
    _check_factorization(a, q, r, j, 1e-10)


def test_reference_test_shape(rnla):
    """cqrrpt.rs:82-85: m = 100, n = 10, uniform data (the crate's
    sketching_operator with the Uniform distribution)."""
    a = rnla.sketching_operator(rnla.DistributionType.Uniform, 100, 10)
    q, r, j = rnla.sap_chol_qrcp(a, 37)
    _check_factorization(np.asarray(a), q, r, j, 1e-6)


def test_bf16x_sketch(rnla):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((20000, 96)) * np.logspace(0, -6, 96)
    q, r, j = rnla.sap_chol_qrcp(a, 400, rnla.options(precision=rnla.Precision.BF16X))
    _check_factorization(a, q, r, j, 1e-9)


def test_errors(rnla):
    rng = np.random.default_rng(1)
    a = rng.standard_normal((100, 10))
    with pytest.raises(rnla.InvalidParameters):          # d < n (cqrrpt.rs:117-126)
        rnla.sap_chol_qrcp(a, 5)
    with pytest.raises(rnla.InvalidParameters):          # wide matrix (cqrrpt.rs:127-136)
        rnla.sap_chol_qrcp(a.T.copy(), 50)
    b = a.copy()
    b[:, 3] = 0.0                                         # numerical rank below n
    with pytest.raises(rnla.SingularMatrix):
        rnla.sap_chol_qrcp(b, 50)
