"""The oracle's restatements against the reference's own known answers
(src/solvers.rs:290-410, src/cg.rs:130-184, src/lora_helpers.rs:325-366,
src/lora_drivers.rs:341-357,447-460) and against LAPACK."""
import numpy as np
import pytest

from oracle import oracle as O


def _rm(vals, r, c):
    return np.array(vals, dtype=float).reshape(r, c)


def test_upper_triangular(golden):
    for case in golden["solvers"]["upper_triangular"]:
        n = case["n"]
        u = _rm(case["u_rowmajor"], n, n)
        x = O.solve_upper_triangular_system(u, case["y"])
        if "expected" in case:
            np.testing.assert_allclose(x, case["expected"], atol=1e-10)
        else:   # zero diagonal: the last equation still holds (solvers.rs:323-324)
            assert abs((u @ x)[2] - case["y"][2]) < 1e-10


def test_lsqr_known_solution(golden):
    c = golden["solvers"]["lsqr_simple"]
    a = _rm(c["a_rowmajor"], c["m"], c["n"])
    x = O.lsqr(a, c["b_known"], c["damp"], c["atol"], c["btol"], c["conlim"])[0]
    np.testing.assert_allclose(x, c["x_known"], atol=c["abs_tol"])
    x0 = O.lsqr(a, c["b_zero"], c["damp"], c["atol"], c["btol"], c["conlim"])
    assert np.all(x0[0] == 0) and x0[1] == 0 and x0[2] == 0


def test_lsqr_matches_lstsq():
    rng = np.random.default_rng(5)
    a = rng.standard_normal((200, 40))
    b = rng.standard_normal(200)
    x = O.lsqr(a, b, 0.0, 1e-12, 1e-12, 1e12, 500)[0]
    np.testing.assert_allclose(x, np.linalg.lstsq(a, b, rcond=None)[0], rtol=1e-8, atol=1e-10)


def test_cgls_cases(golden):
    for c in golden["solvers"]["cgls"]:
        a = _rm(c["a_rowmajor"], 3, 3)
        x = O.cgls(a, c["b"], c["tolerance"], c["num_iterations"], c["x0"])
        if c["name"] == "test_cgls_does_not_converge":
            assert np.linalg.norm(x) > c["tolerance"]
        else:
            assert np.linalg.norm(x) < c["tolerance"]


def test_orth_and_stabilizer_known_answers():
    assert np.allclose(O.orth(np.zeros((5, 5))), np.eye(5), atol=1e-6)
    assert np.allclose(O.orth(np.eye(5)), np.eye(5), atol=1e-6)
    assert np.allclose(O.stabilizer(np.zeros((5, 5))), np.eye(5), atol=1e-6)
    X = np.random.default_rng(0).standard_normal((10, 5))
    assert O.stabilizer(X).shape == (10, 5)


def test_full_piv_lu_reconstructs():
    """L of P X Q = L U: range(L) = P range(X); |L| <= 1 (complete pivoting)."""
    X = np.random.default_rng(1).standard_normal((30, 8))
    L = O.full_piv_lu_l(X)
    assert np.all(np.abs(L) <= 1.0 + 1e-15)
    assert np.allclose(np.diag(L), 1.0)
    # rows of L are a permutation of rows of X (up to the column transform):
    # the projector onto range(L) equals a row/column permutation of that of X
    PL = L @ np.linalg.pinv(L)
    PX = X @ np.linalg.pinv(X)
    assert np.isclose(np.trace(PL), np.trace(PX))


def test_rand_svd_zero_matrix():
    U, S, Vt = O.rand_svd(np.zeros((10, 5)), 3, 1e-6, 2)
    assert np.allclose(U, np.eye(10, 3), atol=1e-6)
    assert np.allclose(S, 0)
    assert np.allclose(Vt.T, np.eye(5, 3), atol=1e-6)


def test_rand_svd_errors_and_shapes():
    A = np.random.default_rng(2).standard_normal((100, 50))
    for bad in ((0, 1e-6, 2), (3, 0.0, 2), (3, 1e-6, 0)):
        with pytest.raises(O.InvalidParameters):
            O.rand_svd(A, *bad)
    U, S, Vt = O.rand_svd(A, 45, 1e-6, 2)
    assert U.shape == (100, 45) and S.shape == (45, 45) and Vt.shape == (45, 50)
    sv = np.diag(S)
    assert np.all(np.diff(sv) <= 0)
    U, S, Vt = O.rand_svd(np.random.default_rng(3).standard_normal((5, 20)), 3, 1e-6, 2)
    assert U.shape == (5, 3) and Vt.shape == (3, 20)


def test_reference_rand_svd_ignores_gaussian():
    """lora_helpers.rs:70-99: the result depends on A only."""
    A = np.random.default_rng(4).standard_normal((40, 20))
    s1 = O.tsog1(A, 6, 2, 1, gaussian=lambda r, c: np.ones((r, c)))
    s2 = O.tsog1(A, 6, 2, 1, gaussian=lambda r, c: np.zeros((r, c)))
    assert np.array_equal(s1, s2)


def test_blendenpik_matches_lstsq():
    m, n = 3000, 40
    A = O.make_lowrank_test_matrix(m, n, np.logspace(0, -6, n), 1, 2)
    xs = np.random.default_rng(3).standard_normal(n)
    b = A @ xs + 1e-6 * np.random.default_rng(4).standard_normal(m)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    rl = np.linalg.norm(A @ xl - b) / np.linalg.norm(b)
    x = O.blendenpik_overdetermined(A, b, 1e-10, 1000, 4.0)
    assert abs(np.linalg.norm(A @ x - b) / np.linalg.norm(b) - rl) < 1e-10
    x2, res = O.blendenpik_lsqr(A, b, 4.0, 1e-14, 1e-14)
    assert abs(np.linalg.norm(A @ x2 - b) / np.linalg.norm(b) - rl) < 1e-10
    assert res[2] < 60


def test_blendenpik_errors():
    A = np.ones((10, 20))
    with pytest.raises(ValueError):
        O.blendenpik_overdetermined(A, np.ones(10), 1e-4, 10, 2.0)
    A = np.random.default_rng(0).standard_normal((100, 10))
    for eps, l, sf in ((1e-4, 1000, 0.5), (-1e-4, 1000, 1.5), (0.0, 1000, 1.5), (1e-4, 0, 1.5)):
        with pytest.raises(O.InvalidParameters):
            O.blendenpik_overdetermined(A, np.ones(100), eps, l, sf)


def test_sketch_rows_rule():
    assert O.sketch_rows(100, 10, 1.5) == 15
    assert O.sketch_rows(100, 80, 1.5) == 100
    assert O.sketch_rows(100000, 500, 4.0) == 2000


def test_sketched_least_squares_restatements_agree():
    """sketch_and_solve.rs:24-33 and :53-65 solve the same sketched problem:
    with the same sketch, QR and SVD give the same x; both come close to the
    full least-squares residual (d = m/4 = 250 rows for n = 20)."""
    rng = np.random.default_rng(5)
    A = rng.standard_normal((1000, 20))
    y = A @ rng.uniform(-100, 100, 20)
    A = A + 0.01 * rng.standard_normal(A.shape)
    xq = O.sketched_least_squares_qr(A, y)
    xs = O.sketched_least_squares_svd(A, y)
    assert np.linalg.norm(xq - xs) <= 1e-9 * np.linalg.norm(xq)
    xl = np.linalg.lstsq(A, y, rcond=None)[0]
    assert np.linalg.norm(A @ xq - y) <= 1.6 * np.linalg.norm(A @ xl - y)
    with pytest.raises(ValueError):
        O.sketched_least_squares_qr(A[:40], y[:40])


def test_lsrn_restatement_converges():
    """sketch_and_precondition.rs:82-119 restated: on a well-posed problem the
    V Sigma^+ preconditioned CGLS reaches the least-squares residual."""
    rng = np.random.default_rng(9)
    A = O.make_lowrank_test_matrix(1500, 30, np.logspace(0, -6, 30), 1, 2)
    b = A @ rng.standard_normal(30) + 1e-6 * rng.standard_normal(1500)
    x, it = O.lsrn_overdetermined(A, b, 1e-12, 500, 4.0, return_iters=True)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    r = np.linalg.norm(A @ x - b) / np.linalg.norm(b)
    rl = np.linalg.norm(A @ xl - b) / np.linalg.norm(b)
    assert abs(r - rl) < 1e-10
    assert it < 100


def test_qrcp_and_cqrrpt_restatements():
    """pivot_decompositions.rs:106-174 and cqrrpt.rs:27-58 restated: the
    pivoted R has non-increasing |R_kk| and R^T R = (a P)^T (a P); CQRRPT
    gives orthonormal q with a[:, p] = q r."""
    rng = np.random.default_rng(4)
    a = rng.standard_normal((300, 12)) * np.logspace(0, -3, 12)
    r, p = O.qrcp(a)
    R = np.triu(r[:12, :12])
    assert sorted(p) == list(range(12))
    assert np.all(np.diff(np.abs(np.diag(R))) <= 1e-12)
    ap = a[:, p]
    np.testing.assert_allclose(R.T @ R, ap.T @ ap, rtol=0, atol=1e-10)
    q, rr, pp = O.sap_chol_qrcp(a, 60)
    np.testing.assert_allclose(q.T @ q, np.eye(12), atol=1e-10)
    np.testing.assert_allclose(q @ rr, a[:, pp], atol=1e-10)
    assert np.allclose(np.tril(rr, -1), 0.0)
    with pytest.raises(O.InvalidParameters):
        O.sap_chol_qrcp(a, 5)


def test_rand_evd_restatements():
    """lora_drivers.rs:84-213 restated: the dominant eigenpairs of a
    symmetric matrix with a clear gap come out of both drivers."""
    rng = np.random.default_rng(8)
    Q, _ = np.linalg.qr(rng.standard_normal((80, 80)))
    eigs = np.concatenate([[20.0, -10.0, 5.0], 1e-4 * np.ones(77)])
    A = (Q * eigs) @ Q.T
    A = (A + A.T) / 2
    V, lam = O.rand_evd1(A, 3, 1e-6, 8)
    np.testing.assert_allclose(lam, [20.0, -10.0, 5.0], atol=1e-3)
    P = (Q * np.abs(eigs)) @ Q.T
    P = (P + P.T) / 2
    V2, lam2 = O.rand_evd2(P, 3, 8)
    np.testing.assert_allclose(lam2, [20.0, 10.0, 5.0], rtol=1e-3)


def test_rand_evd_reference_known_answers(golden):
    """The reference's rand_evd tests with fixed answers
    (lora_drivers.rs:506-514, 532-563, 702-710, 725-746, 748-776)."""
    Z = np.zeros((5, 5))
    V, lam = O.rand_evd1(Z, 3, 1e-6, 2)
    np.testing.assert_array_equal(V, np.eye(5)[:, :3])        # symmetric_eigen(0) vectors
    assert all(x == 0.0 for x in lam)
    with pytest.raises(O.MatrixDecompositionError):
        O.rand_evd2(Z, 3, 2)                                   # Cholesky of S^T 0 fails
    assert len(O.rand_evd1(np.eye(5), 3, 1e-6, 2)[1]) == 3
    assert len(O.rand_evd2(np.eye(5), 3, 2)[1]) == 3
    W = np.array(golden["solvers"]["rand_evd_reject"]["test_wrong_hermitian"])
    with pytest.raises(O.NotHermitian):
        O.rand_evd1(W, 3, 1e-6, 2)
    with pytest.raises(ValueError):
        O.rand_evd2(W, 3, 2)
    # 5 x 5 PSD, k + s = n: the exact dominant eigenpairs
    G = np.random.default_rng(3).standard_normal((5, 5))
    P = G @ G.T
    V, lam = O.rand_evd2(P, 3, 2)
    w, U = np.linalg.eigh(P)
    top = np.argsort(-np.abs(w))[:3]
    np.testing.assert_allclose(lam, w[top], atol=1e-6)
    np.testing.assert_allclose(V.T @ V, np.eye(3), atol=1e-6)
    np.testing.assert_allclose(V @ V.T @ P, U[:, top] @ U[:, top].T @ P, atol=1e-6)
