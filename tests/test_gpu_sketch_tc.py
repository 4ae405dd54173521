"""Tensor-core (tcgen05) sketch S [A] against an FP64 product with the same
quantised sketch.  Integer data makes every product and partial sum exactly
representable, so there the result must be bit-identical: that pins the
exact-window accumulation, both swizzled shared-memory layouts, the split-K
reduction and the ragged edge tiles."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _quantized_sketch(d, m, seed, dist=0):
    import torch
    import randnla_gb300 as R
    S = torch.empty((m, d), dtype=torch.float32, device="cuda").t()     # column-major d x m
    R.sketching_operator_dev(S, dist_type=R.DistributionType(dist), quantized=True, seed=seed)
    return S.double()


def _tc(Y, d, seed, digits=0, dist=0):
    import torch
    import randnla_gb300 as R
    C = torch.empty((Y.shape[1], d), dtype=torch.float64, device="cuda").t()
    R.sketch_apply_dev(Y, d, C, precision=R.Precision.BF16X, digits=digits, seed=seed,
                       dist_type=R.DistributionType(dist))
    torch.cuda.synchronize()
    return C


@pytest.mark.parametrize("d,m,n", [(200, 5000, 100), (128, 64, 96), (37, 4099, 5), (256, 2048, 1)])
def test_integer_data_bit_exact(rnla, d, m, n):
    import torch
    g = torch.Generator(device="cuda").manual_seed(d + m + n)
    Y = torch.randint(-1000, 1001, (n, m), generator=g, device="cuda").double().t()
    C = _tc(Y, d, seed=11)
    ref = _quantized_sketch(d, m, 11) @ Y
    assert torch.equal(C, ref), (C - ref).abs().max().item()


@pytest.mark.parametrize("digits,vmax", [(3, 1000), (2, 1000), (1, 127)])
@pytest.mark.parametrize("n", [1, 79, 80, 81, 159, 161])
def test_integer_fp32_data_80_column_tiles_bit_exact(rnla, digits, vmax, n):
    """FP32 data with up to three digits runs on 80-column digit tiles (one
    MMA of N = 80 x digits); integers that the digits hold exactly give the
    exact product, for column counts on both sides of the tile edges."""
    import torch
    d, m = 136, 3001
    g = torch.Generator(device="cuda").manual_seed(31 * n + digits)
    Y = torch.randint(-vmax, vmax + 1, (n, m), generator=g, device="cuda").float().t()
    C = _tc(Y, d, seed=21, digits=digits)
    ref = _quantized_sketch(d, m, 21) @ Y.double()
    assert torch.equal(C, ref), (C - ref).abs().max().item()


@pytest.mark.parametrize("dist", [1, 2])
@pytest.mark.parametrize("d,m,n", [(200, 5000, 100), (37, 4099, 5)])
def test_uniform_and_rademacher_bit_exact(rnla, dist, d, m, n):
    import torch
    g = torch.Generator(device="cuda").manual_seed(d + m + n + dist)
    Y = torch.randint(-1000, 1001, (n, m), generator=g, device="cuda").double().t()
    C = _tc(Y, d, seed=13, dist=dist)
    S = _quantized_sketch(d, m, 13, dist)
    assert torch.equal(C, S @ Y), (C - S @ Y).abs().max().item()
    # the device quantised operator is the oracle's, word for word
    ref = O.sketch(dist, d, 64, key0=13, quantized=True)
    assert np.array_equal(S[:, :64].cpu().numpy(), ref)


@pytest.mark.parametrize("dist", [1, 2])
def test_uniform_and_rademacher_fp64_data(rnla, dist):
    import torch
    g = torch.Generator(device="cuda").manual_seed(17)
    d, m, n = 160, 12000, 70
    Y = torch.randn((n, m), generator=g, device="cuda", dtype=torch.float64).t()
    C = _tc(Y, d, seed=5, dist=dist)
    ref = _quantized_sketch(d, m, 5, dist) @ Y
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-9, err


def test_gaussian_fp64_data(rnla):
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    d, m, n = 300, 20000, 130
    Y = torch.randn((n, m), generator=g, device="cuda", dtype=torch.float64).t()
    C = _tc(Y, d, seed=3)
    ref = _quantized_sketch(d, m, 3) @ Y
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-9, err


def test_float32_data_default_digits(rnla):
    import torch
    g = torch.Generator(device="cuda").manual_seed(6)
    d, m, n = 256, 9000, 200
    Y = torch.randn((n, m), generator=g, device="cuda", dtype=torch.float32).t()
    C = _tc(Y, d, seed=4)
    ref = _quantized_sketch(d, m, 4) @ Y.double()
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    # FP32 data default to 3 digits: 24 bits below each column's maximum
    assert err < 1e-6, err


@pytest.mark.parametrize("digits,bound", [(1, 2e-2), (2, 4e-4), (3, 4e-6), (4, 1e-9)])
def test_digit_count_controls_accuracy(rnla, digits, bound):
    import torch
    g = torch.Generator(device="cuda").manual_seed(7)
    d, m, n = 128, 6000, 64
    Y = torch.randn((n, m), generator=g, device="cuda", dtype=torch.float64).t()
    C = _tc(Y, d, seed=9, digits=digits)
    ref = _quantized_sketch(d, m, 9) @ Y
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert err < bound, (digits, err)


def test_digit_count_out_of_range_is_an_error(rnla):
    import torch
    Y = torch.randn((8, 256), device="cuda", dtype=torch.float64).t()
    with pytest.raises(rnla.RandNLAError):
        _tc(Y, 16, seed=1, digits=5)


def test_blendenpik_bf16x_vs_lapack(rnla):
    from oracle import oracle as O
    A = O.make_lowrank_test_matrix(20000, 120, np.logspace(0, -8, 120), 1, 2)
    rng = np.random.default_rng(3)
    b = A @ rng.standard_normal(120) + 1e-6 * rng.standard_normal(20000)
    o = rnla.options(precision=rnla.Precision.BF16X, inner_solver=rnla.InnerSolver.LSQR,
                     atol=1e-14, btol=1e-14, seed=42)
    x, st = rnla.blendenpik_overdetermined(A, b, 1e-12, 1000, 4.0, o, return_stats=True)
    xl = np.linalg.lstsq(A, b, rcond=None)[0]
    rr = np.linalg.norm(A @ x.ravel() - b) / np.linalg.norm(b)
    rl = np.linalg.norm(A @ xl - b) / np.linalg.norm(b)
    assert abs(rr - rl) < 1e-10
    o64 = rnla.options(precision=rnla.Precision.FP64, inner_solver=rnla.InnerSolver.LSQR,
                       atol=1e-14, btol=1e-14, seed=42)
    _, st64 = rnla.blendenpik_overdetermined(A, b, 1e-12, 1000, 4.0, o64, return_stats=True)
    assert st["iterations"] <= st64["iterations"] + 5
