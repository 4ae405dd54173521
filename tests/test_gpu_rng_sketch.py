"""GPU generators and sketch operators against the oracle: bit-exact
word streams (pinned to the reference KATs) and bit-exact sketch entries."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_philox_stream_kat(rnla, golden):
    k = golden["rng"]
    key = k["philox_key_seed1"] | (k["philox_key_seed2"] << 32)
    w = rnla.rng_words(0, 40, rnla.Generator.Philox4x32, key)
    assert list(w) == k["philox4x32"]


def test_threefry_stream_kat(rnla, golden):
    k = golden["rng"]
    w = rnla.rng_words(0, 40, rnla.Generator.ThreeFry2x64, k["threefry_key0"], k["threefry_key1"])
    joined = [int(w[2 * i]) | (int(w[2 * i + 1]) << 32) for i in range(20)]
    assert joined == k["threefry2x64"]


@pytest.mark.parametrize("gen", [0, 1])
def test_streams_match_oracle_at_offsets(rnla, gen):
    for first, n in ((0, 1), (3, 9), (12345, 1000), (4 * (1 << 32) - 5, 17)):
        g = rnla.rng_words(first, n, gen, 0xDEADBEEF12345678, 99)
        o = O.word_stream(gen, 0xDEADBEEF12345678, 99, first, n)
        assert np.array_equal(g, o)


@pytest.mark.parametrize("gen", [0, 1])
def test_stream_checksums_over_1e8_counters(rnla, gen):
    """1e8 generator counters (4e8 words) against the oracle's C generator:
    the sum of the words and the sum of word xor offset, both exact."""
    import ctypes
    import torch
    n = 400_000_000
    key0, key1 = 0x0123456789ABCDEF, 77
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    r = rnla._rng(gen, key0, key1)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert rnla.lib().rnla_rng_words_dev(ctypes.byref(r), 0, n, ctypes.c_void_p(out.data_ptr()), stream) == 0
    s1 = s2 = 0
    chunk = 50_000_000
    for c0 in range(0, n, chunk):
        w = out[c0:c0 + chunk]
        idx = torch.arange(c0, c0 + w.numel(), dtype=torch.int32, device="cuda")
        s1 += int((w.long() & 0xFFFFFFFF).sum())
        s2 += int(((w ^ idx).long() & 0xFFFFFFFF).sum())
    del out
    assert (s1, s2) == O.word_checksums(gen, key0, key1, 0, n)


@pytest.mark.parametrize("dist", [0, 1, 2])
@pytest.mark.parametrize("gen", [0, 1])
def test_sketching_operator_bit_exact(rnla, dist, gen):
    for rows, cols in ((1, 1), (7, 5), (100, 50), (257, 33)):
        S = rnla.sketching_operator(dist, rows, cols, gen, seed=42)
        ref = O.sketch(dist, rows, cols, gen, key0=42)
        assert S.shape == (rows, cols)
        assert np.array_equal(S, ref), (dist, gen, rows, cols, np.abs(S - ref).max())


def test_sketching_operator_default_seed(rnla):
    S = rnla.sketching_operator(rnla.DistributionType.Gaussian, 100, 50)
    assert np.array_equal(S, O.sketch(0, 100, 50))


def test_sketching_operator_errors(rnla):
    with pytest.raises(rnla.InvalidDimensions):
        rnla.sketching_operator(rnla.DistributionType.Gaussian, 0, 50)
    with pytest.raises(rnla.InvalidDimensions):
        rnla.sketching_operator(rnla.DistributionType.Gaussian, 100, 0)


def test_quantized_f32_operator(rnla):
    import torch
    out = torch.empty((96, 131), dtype=torch.float32, device="cuda").t().contiguous().t()
    rnla.sketching_operator_dev(out, quantized=True, seed=7)
    torch.cuda.synchronize()
    ref = O.sketch(0, 96, 131, key0=7, quantized=True)
    assert np.array_equal(out.cpu().numpy().astype(np.float64), ref)
