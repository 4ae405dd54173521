"""lora_drivers::rand_evd1 / rand_evd2 on the GPU against the oracle
restatements (same tsog1 / QB1 data flow, numpy's eigh and SVD for the small
eigenproblems): eigenvalues to 1e-8 relative of the largest, eigenvectors up
to sign, plus the reference tests' error cases."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sym(n, eigs, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Q * np.asarray(eigs)) @ Q.T
    return (A + A.T) / 2


def _same_columns_up_to_sign(V, Vo, tol):
    for j in range(V.shape[1]):
        c = abs(float(V[:, j] @ Vo[:, j]))
        assert c > 1.0 - tol, (j, c)


def test_evd1_indefinite(rnla):
    n = 120
    eigs = np.concatenate([[50, -40, 30, -20, 10], 1e-3 * np.linspace(1, -1, n - 5)])
    A = _sym(n, eigs, 1)
    V, lam = rnla.rand_evd1(A, 5, 1e-6, 10)
    Vo, lamo = O.rand_evd1(A, 5, 1e-6, 10)
    assert len(lam) == 5
    np.testing.assert_allclose(lam, lamo, rtol=0, atol=1e-8 * abs(lamo[0]))
    np.testing.assert_allclose(sorted(lam, key=abs, reverse=True), [50, -40, 30, -20, 10], atol=1e-2)
    _same_columns_up_to_sign(V, Vo, 1e-8)


def test_evd2_psd(rnla):
    n = 150
    eigs = np.concatenate([[100, 60, 30, 10, 5, 2], np.full(n - 6, 1e-6)])
    A = _sym(n, eigs, 2)
    V, lam = rnla.rand_evd2(A, 6, 6)
    Vo, lamo = O.rand_evd2(A, 6, 6)
    assert len(lam) == len(lamo) == 6
    np.testing.assert_allclose(lam, lamo, rtol=0, atol=1e-8 * lamo[0])
    np.testing.assert_allclose(lam, [100, 60, 30, 10, 5, 2], rtol=1e-3)
    _same_columns_up_to_sign(V, Vo, 1e-8)


def test_errors(rnla):
    A = _sym(30, np.linspace(1, 2, 30), 3)
    for k, eps, s in ((0, 1e-6, 2), (3, 0.0, 2), (3, -1.0, 2), (3, 1e-6, 0)):
        with pytest.raises(rnla.InvalidParameters):
            rnla.rand_evd1(A, k, eps, s)
    B = A.copy()
    B[0, 1] += 1e-3
    with pytest.raises(rnla.NotHermitian):
        rnla.rand_evd1(B, 3, 1e-6, 2)
    with pytest.raises(rnla.InvalidParameters):
        rnla.rand_evd2(A, 0, 2)
    C = _sym(30, np.linspace(-1, 2, 30), 4)
    with pytest.raises(rnla.NotPositiveSemiDefinite):
        rnla.rand_evd2(C, 3, 2)


def test_reference_known_answers(rnla, golden):
    """The reference's rand_evd tests with fixed answers
    (lora_drivers.rs:506-514, 532-563, 702-710, 725-746, 748-776)."""
    Z = np.zeros((5, 5))
    V, lam = rnla.rand_evd1(Z, 3, 1e-6, 2)
    np.testing.assert_allclose(V, np.eye(5)[:, :3], atol=1e-6)   # symmetric_eigen(0) vectors
    assert all(x == 0.0 for x in lam)
    with pytest.raises(rnla.MatrixDecompositionError):
        rnla.rand_evd2(Z, 3, 2)                                   # Cholesky of S^T 0 fails
    V, lam = rnla.rand_evd1(np.eye(5), 3, 1e-6, 2)
    assert V.shape == (5, 3) and len(lam) == 3
    V, lam = rnla.rand_evd2(np.eye(5), 3, 2)
    assert V.shape == (5, 3) and len(lam) == 3
    W = np.array(golden["solvers"]["rand_evd_reject"]["test_wrong_hermitian"])
    with pytest.raises(rnla.NotHermitian):
        rnla.rand_evd1(W, 3, 1e-6, 2)
    with pytest.raises(rnla.RandNLAError):
        rnla.rand_evd2(W, 3, 2)
    # 5 x 5 PSD, k + s = n: the exact dominant eigenpairs
    G = np.random.default_rng(3).standard_normal((5, 5))
    P = G @ G.T
    V, lam = rnla.rand_evd2(P, 3, 2)
    w, U = np.linalg.eigh(P)
    top = np.argsort(-np.abs(w))[:3]
    np.testing.assert_allclose(lam, w[top], atol=1e-6)
    np.testing.assert_allclose(V.T @ V, np.eye(3), atol=1e-6)
    np.testing.assert_allclose(V @ V.T @ P, U[:, top] @ U[:, top].T @ P, atol=1e-6)


def test_evd1_order_orthogonality_and_error(rnla):
    """lora_drivers.rs:631-686: |lambda| non-increasing, V^T V = I, and the
    relative Frobenius error of V diag(lambda) V^T within epsilon."""
    G = np.random.default_rng(5).standard_normal((100, 100))
    A = 0.5 * (G + G.T)
    V, lam = rnla.rand_evd1(A, 3, 2.0, 2)
    assert list(np.abs(lam)) == sorted(np.abs(lam), reverse=True)
    np.testing.assert_allclose(V.T @ V, np.eye(3), atol=1e-6)
    err = np.linalg.norm(A - (V * lam) @ V.T) / np.linalg.norm(A)
    assert err <= 2.0
