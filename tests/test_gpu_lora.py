"""lora_helpers.rs / lora_drivers.rs on the GPU against the oracle and the
reference's known answers."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_orth_known_answers(rnla):
    assert np.allclose(rnla.Orth(np.zeros((5, 5))), np.eye(5), atol=1e-6)
    assert np.allclose(rnla.Orth(np.eye(5)), np.eye(5), atol=1e-6)


@pytest.mark.parametrize("shape", [(10, 5), (5, 5), (100, 37), (7, 12)])
def test_orth_spans_same_space(rnla, shape):
    X = np.random.default_rng(0).standard_normal(shape)
    q = rnla.Orth(X)
    qo = O.orth(X)
    assert q.shape == qo.shape
    assert np.allclose(q.T @ q, np.eye(q.shape[1]), atol=1e-12)
    assert np.allclose(q @ q.T, qo @ qo.T, atol=1e-12)
    assert np.allclose(np.abs(q), np.abs(qo), atol=1e-12)   # same Householder convention


def test_stabilizer_known_answers(rnla):
    assert np.allclose(rnla.Stabilizer(np.zeros((5, 5))), np.eye(5), atol=1e-6)
    assert rnla.Stabilizer(np.eye(5)).shape == (5, 5)


@pytest.mark.parametrize("shape", [(10, 5), (5, 5), (200, 60), (1000, 60), (8, 20)])
def test_stabilizer_bit_exact(rnla, shape):
    X = np.random.default_rng(1).standard_normal(shape)
    assert np.array_equal(rnla.Stabilizer(X), O.stabilizer(X))


@pytest.mark.parametrize("passes,pps", [(2, 1), (4, 2), (4, 3), (2, 2)])
def test_tsog1_even_passes(rnla, passes, pps):
    A = np.random.default_rng(2).standard_normal((40, 25))
    S = rnla.tsog1(A, 6, passes, pps)
    So = O.tsog1(A, 6, passes, pps)
    assert S.shape == So.shape
    np.testing.assert_allclose(S, So, rtol=1e-12, atol=1e-12)


def test_rf1_qb1(rnla):
    A = np.random.default_rng(3).standard_normal((100, 50))
    Q = rnla.RF1(A, 3)
    Qo = O.rf1(A, 3)
    assert Q.shape == Qo.shape == (100, 3)
    assert np.allclose(Q @ Q.T, Qo @ Qo.T, atol=1e-11)
    Q, B = rnla.QB1(A, 3, 1e-6)
    assert B.shape == (3, 50)
    assert np.allclose(Q @ B, Qo @ (Qo.T @ A), atol=1e-10)


def test_rand_svd_zero_matrix(rnla):
    """lora_drivers.rs:341-357."""
    U, S, Vt = rnla.rand_svd(np.zeros((10, 5)), 3, 1e-6, 2)
    assert np.allclose(U, np.eye(10, 3), atol=1e-6)
    assert np.allclose(S, np.zeros((3, 3)), atol=1e-6)
    assert np.allclose(Vt.T, np.eye(5, 3), atol=1e-6)


def test_rand_svd_errors(rnla):
    A = np.random.default_rng(4).standard_normal((100, 50))
    for bad in ((0, 1e-6, 2), (3, 0.0, 2), (3, -1.0, 2), (3, 1e-6, 0)):
        with pytest.raises(rnla.InvalidParameters):
            rnla.rand_svd(A, *bad)


@pytest.mark.parametrize("shape,k,s", [((100, 50), 45, 2), ((20, 5), 3, 2), ((5, 20), 3, 2),
                                       ((10, 5), 3, 2), ((3, 3), 2, 2), ((300, 200), 30, 10)])
def test_rand_svd_reference_mode(rnla, shape, k, s):
    A = np.random.default_rng(5).standard_normal(shape)
    U, S, Vt = rnla.rand_svd(A, k, 1e-6, s)
    Uo, So, Vto = O.rand_svd(A, k, 1e-6, s)
    assert U.shape == Uo.shape and S.shape == So.shape and Vt.shape == Vto.shape
    sv, so = np.diag(S), np.diag(So)
    assert np.all(np.diff(sv) <= 0)                     # lora_drivers.rs:447-460
    np.testing.assert_allclose(sv, so, rtol=1e-10, atol=1e-12 * so[0])
    np.testing.assert_allclose(U @ S @ Vt, Uo @ So @ Vto, atol=1e-9 * so[0])


def test_rand_svd_config1_reference_mode(rnla):
    """2000 x 1000, sigma_i = 10^(-i/100), k = 50, s = 10: singular values
    within 1e-10 relative of the oracle's restatement."""
    sig = 10.0 ** (-np.arange(1000) / 100.0)
    A = O.make_lowrank_test_matrix(2000, 1000, sig, 1, 2)
    U, S, Vt = rnla.rand_svd(A, 50, 1e-6, 10)
    Uo, So, Vto = O.rand_svd(A, 50, 1e-6, 10)
    np.testing.assert_allclose(np.diag(S), np.diag(So), rtol=1e-10)


def test_rand_svd_randnla_fp64(rnla):
    sig = 10.0 ** (-np.arange(1000) / 100.0)
    A = O.make_lowrank_test_matrix(2000, 1000, sig, 1, 2)
    o = rnla.options(mode=rnla.Mode.RandNLA, power_iters=2, seed=42)
    U, S, Vt = rnla.rand_svd(A, 50, 1e-6, 10, o)
    Uo, so, Vto = O.rand_svd_randnla(A, 50, 10, 2, seed=42)
    np.testing.assert_allclose(np.diag(S), so, rtol=1e-10)
    assert np.allclose(U.T @ U, np.eye(50), atol=1e-12)
    # the figures of the randomized range finder: ||A - U S Vt||_F against the
    # oracle's and the optimal rank-50 error, the top-k sigma against the
    # construction (oracle on this matrix: 1.0068 x optimal, 2.4% worst sigma)
    err = np.linalg.norm(A - U @ S @ Vt)
    err_o = np.linalg.norm(A - (Uo * so) @ Vto)
    tail = np.sqrt(np.sum(sig[50:] ** 2))
    assert abs(err - err_o) < 1e-8
    assert err < 1.01 * tail
    rel = np.abs(np.diag(S) - sig[:50]) / sig[:50]
    assert rel.max() < 0.03 and rel[0] < 1e-6


def test_rand_svd_randnla_tensor_core_vs_oracle(rnla):
    """The tensor-core (BF16X) range finder on the oracle's FP64 pipeline with
    the same Omega: the top-k singular values within 1e-6 relative, the
    approximation error ||A - U S Vt||_F and U's orthonormality at the level
    of the split-bf16 products (~1e-7)."""
    sig = 10.0 ** (-np.arange(1000) / 100.0)
    A = O.make_lowrank_test_matrix(2000, 1000, sig, 1, 2)
    o = rnla.options(precision=rnla.Precision.BF16X, mode=rnla.Mode.RandNLA, power_iters=2, seed=42)
    U, S, Vt, st = rnla.rand_svd(A, 50, 1e-6, 10, o, return_stats=True)
    Uo, so, Vto = O.rand_svd_randnla(A, 50, 10, 2, seed=42)
    s = np.diag(S)
    assert np.max(np.abs(s - so) / so) < 1e-6
    assert np.allclose(U.T @ U, np.eye(50), atol=1e-6)
    assert np.allclose(Vt @ Vt.T, np.eye(50), atol=1e-6)
    err = np.linalg.norm(A - U @ S @ Vt)
    err_o = np.linalg.norm(A - (Uo * so) @ Vto)
    assert abs(err - err_o) <= 1e-6 * err_o
    assert st["precision_used"] == int(rnla.Precision.BF16X)


def test_rand_svd_randnla_tensor_core_fp32_storage(rnla):
    """A stored in FP32 (read by the plane builder directly, no FP64 copy)."""
    import torch
    rng = np.random.default_rng(8)
    m, n, k, p = 3000, 1500, 64, 16
    sig = np.exp(-np.arange(n) / 16.0)
    A = O.make_lowrank_test_matrix(m, n, sig, 3, 4).astype(np.float32)
    A64 = A.astype(np.float64)
    At = torch.from_numpy(A).cuda().t().contiguous().t()
    l = k + p
    U = torch.zeros((l, m), dtype=torch.float64, device="cuda").t()
    sg = torch.zeros(l, dtype=torch.float64, device="cuda")
    Vt = torch.zeros((n, l), dtype=torch.float64, device="cuda").t()
    o = rnla.options(precision=rnla.Precision.BF16X, mode=rnla.Mode.RandNLA, power_iters=2, seed=5)
    r, _ = rnla.rand_svd_dev(At, k, 1e-6, p, U, sg, Vt, o)
    assert r == k
    _, so, _ = O.rand_svd_randnla(A64, k, p, 2, seed=5)
    s = sg[:k].cpu().numpy()
    assert np.max(np.abs(s - so) / so) < 1e-6
    del rng


@pytest.mark.parametrize("K,MM,NN", [(5000, 300, 200), (700, 130, 97), (64, 16, 8)])
def test_gemm_tn_split_bf16_levels(rnla, K, MM, NN):
    """rnla_gemm_tn_dev on the tensor cores: level 1 (plain bf16), 2 and 3
    planes (the digits arguments) and 4 (exact integer digit products)
    against the FP64 product."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(K + MM)
    x = torch.randn((MM, K), generator=g, dtype=torch.float64, device="cuda").t()
    y = torch.randn((NN, K), generator=g, dtype=torch.float64, device="cuda").t()
    ref = x.t() @ y
    scale = (x.abs().t() @ y.abs()).max().item()
    for level, bound in ((1, 2e-2), (2, 2e-4), (3, 2e-6), (4, 1e-8)):
        c = torch.full((NN, MM), float("nan"), dtype=torch.float64, device="cuda").t()
        rnla.gemm_tn_dev(x, y, c, precision=rnla.Precision.BF16X, digits_x=level, digits_y=level)
        torch.cuda.synchronize()
        err = (c - ref).abs().max().item() / scale
        assert err < bound, (level, err)


def test_gemm_tn_split_bf16_exact_on_small_integers(rnla):
    """Integers |v| <= 16 are exact in bf16 and the sums stay below 2^24, so
    every level returns the exact product."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(3)
    K, MM, NN = 3000, 150, 100
    x = torch.randint(-16, 17, (MM, K), generator=g, device="cuda").double().t()
    y = torch.randint(-16, 17, (NN, K), generator=g, device="cuda").double().t()
    ref = x.t() @ y
    for level in (1, 2, 3, 4):
        c = torch.zeros((NN, MM), dtype=torch.float64, device="cuda").t()
        rnla.gemm_tn_dev(x, y, c, precision=rnla.Precision.BF16X, digits_x=level, digits_y=level)
        torch.cuda.synchronize()
        assert torch.equal(c, ref), level
