"""solvers.rs / cg.rs on the GPU against the reference's known answers and
the oracle's restatement."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rm(vals, r, c):
    return np.array(vals, dtype=float).reshape(r, c)


def test_upper_triangular_kats(rnla, golden):
    for case in golden["solvers"]["upper_triangular"]:
        n = case["n"]
        u = _rm(case["u_rowmajor"], n, n)
        x = rnla.solve_upper_triangular_system(u, case["y"]).ravel()
        np.testing.assert_allclose(x, O.solve_upper_triangular_system(u, case["y"]), atol=1e-14)
        if "expected" in case:
            np.testing.assert_allclose(x, case["expected"], atol=1e-10)


def test_upper_triangular_random(rnla):
    rng = np.random.default_rng(0)
    for n in (1, 5, 64, 300):
        u = np.triu(rng.standard_normal((n, n))) + n * np.eye(n)
        if n > 4:
            u[3, 3] = 0.0
        y = rng.standard_normal(n)
        np.testing.assert_allclose(rnla.solve_upper_triangular_system(u, y).ravel(),
                                   O.solve_upper_triangular_system(u, y), rtol=1e-12, atol=1e-12)


def test_lsqr_kat(rnla, golden):
    c = golden["solvers"]["lsqr_simple"]
    a = _rm(c["a_rowmajor"], c["m"], c["n"])
    got = rnla.lsqr(a, c["b_known"], c["damp"], c["atol"], c["btol"], c["conlim"])
    np.testing.assert_allclose(got[0], c["x_known"], atol=c["abs_tol"])
    ref = O.lsqr(a, c["b_known"], c["damp"], c["atol"], c["btol"], c["conlim"])
    assert got[1] == ref[1] and got[2] == ref[2]
    z = rnla.lsqr(a, c["b_zero"], c["damp"], c["atol"], c["btol"], c["conlim"])
    assert np.all(z[0] == 0) and z[1] == 0 and z[2] == 0


@pytest.mark.parametrize("shape,damp,x0,calc_var", [((200, 40), 0.0, False, False),
                                                     ((500, 30), 0.3, True, True),
                                                     ((1000, 300), 0.0, True, False),
                                                     ((64, 64), 0.0, False, True)])
def test_lsqr_matches_oracle(rnla, shape, damp, x0, calc_var):
    rng = np.random.default_rng(1)
    m, n = shape
    a = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    xx = rng.standard_normal(n) if x0 else None
    got = rnla.lsqr(a, b, damp, 1e-10, 1e-10, 1e8, 3 * n, calc_var, xx)
    ref = O.lsqr(a, b, damp, 1e-10, 1e-10, 1e8, 3 * n, calc_var, xx)
    # iteration counts near a stopping threshold move by a few steps with rounding
    assert got[1] == ref[1]
    assert abs(got[2] - ref[2]) <= max(1, ref[2] // 20)
    np.testing.assert_allclose(got[0], ref[0], rtol=1e-7, atol=1e-9)
    # anorm, acond, xnorm are running estimates: they agree tightly only at equal counts
    # (on the square system they accumulate rounding over ~90 steps)
    rt = (1e-6 if m > n else 1e-2) if got[2] == ref[2] else 5e-2
    for i in (5, 6, 8):
        np.testing.assert_allclose(got[i], ref[i], rtol=rt)
    for i in (3, 4):   # residual norms: absolute scale ||b|| (a square system drives them to 0)
        np.testing.assert_allclose(got[i], ref[i], rtol=1e-6, atol=1e-6 * np.linalg.norm(b))
    if calc_var:
        np.testing.assert_allclose(got[9], ref[9], rtol=rt)
    # the ||A^T r|| history: finite-precision LSQR trajectories on an ill-conditioned
    # system separate after some tens of steps (different summation orders)
    k = min(len(got[7]), len(ref[7]), 20)
    np.testing.assert_allclose(got[7][:k], ref[7][:k], rtol=1e-6)


def test_cgls_kats(rnla, golden):
    for c in golden["solvers"]["cgls"]:
        a = _rm(c["a_rowmajor"], 3, 3)
        got, it = rnla.cgls(a, c["b"], c["tolerance"], c["num_iterations"], c["x0"], return_iterations=True)
        ref, rit = O.cgls(a, c["b"], c["tolerance"], c["num_iterations"], c["x0"], return_iters=True)
        np.testing.assert_allclose(got.ravel(), ref, rtol=1e-12, atol=1e-14)
        assert it == rit


def test_cgls_matches_oracle(rnla):
    rng = np.random.default_rng(2)
    a = rng.standard_normal((700, 90))
    b = rng.standard_normal(700)
    got, it = rnla.cgls(a, b, 1e-9, 500, None, return_iterations=True)
    ref, rit = O.cgls(a, b, 1e-9, 500, None, return_iters=True)
    assert abs(it - rit) <= 1
    np.testing.assert_allclose(got.ravel(), ref, rtol=1e-8, atol=1e-10)


def test_cgls_zero_rhs_propagates_nan(rnla):
    """cg.rs:39: alpha = 0/0 for b = 0, kept as in the reference."""
    a = np.random.default_rng(3).standard_normal((20, 4))
    got = rnla.cgls(a, np.zeros(20), 1e-8, 5)
    ref = O.cgls(a, np.zeros(20), 1e-8, 5)
    assert np.isnan(got).all() and np.isnan(ref).all()


@pytest.mark.parametrize("m,n,x0", [(3000, 1100, False), (2500, 2049, True)])
def test_lsqr_wide_columns_staged_pass(rnla, m, n, x0):
    """n > 1024 takes the staged (mode 0) pass of the FP64 solver kernels."""
    rng = np.random.default_rng(n)
    a = rng.standard_normal((m, n))
    b = rng.standard_normal(m)
    xx = rng.standard_normal(n) if x0 else None
    got = rnla.lsqr(a, b, 0.0, 1e-12, 1e-12, 1e8, 4 * n, False, xx)
    ref = O.lsqr(a, b, 0.0, 1e-12, 1e-12, 1e8, 4 * n, False, xx)
    assert got[1] == ref[1] == 2
    assert abs(got[2] - ref[2]) <= 1
    xl = np.linalg.lstsq(a, b, rcond=None)[0]
    np.testing.assert_allclose(got[0], xl, rtol=1e-9, atol=1e-10)
    r = b - a @ got[0]
    assert np.linalg.norm(a.T @ r) / (np.linalg.norm(a) * np.linalg.norm(r)) < 1e-12


def test_cgls_wide_columns_staged_pass(rnla):
    rng = np.random.default_rng(5)
    a = rng.standard_normal((3000, 1100))
    b = rng.standard_normal(3000)
    got, it = rnla.cgls(a, b, 1e-9, 500, None, return_iterations=True)
    ref, rit = O.cgls(a, b, 1e-9, 500, None, return_iters=True)
    assert abs(it - rit) <= 1
    np.testing.assert_allclose(got.ravel(), np.linalg.lstsq(a, b, rcond=None)[0], rtol=1e-7, atol=1e-9)
