"""The oracle's generators against the reference's own known-answer vectors
(rust-random123/src/philox.rs:242-363, threefry.rs:97-127)."""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O


def test_philox_kats(golden):
    k = golden["rng"]
    s1, s2 = k["philox_key_seed1"], k["philox_key_seed2"]
    for i in range(10):
        assert O.philox4x32([i, 0, 0, 0], [s1, s2]) == k["philox4x32"][4 * i:4 * i + 4]
        assert O.philox2x32([i, 0], [s1]) == k["philox2x32"][2 * i:2 * i + 2]
        assert O.philox2x64([i, 0], [s1]) == k["philox2x64"][2 * i:2 * i + 2]
        assert O.philox4x64([i, 0, 0, 0], [s1, s2]) == k["philox4x64"][4 * i:4 * i + 4]


def test_threefry_kat(golden):
    k = golden["rng"]
    for i in range(10):
        assert O.threefry2x64([i, 0], [k["threefry_key0"], k["threefry_key1"]]) == \
            k["threefry2x64"][2 * i:2 * i + 2]


def test_word_stream_is_block_sequence(golden):
    """Word t = word t%4 of block t//4 (philox.rs:87-99 counter order)."""
    k = golden["rng"]
    key = k["philox_key_seed1"] | (k["philox_key_seed2"] << 32)
    w = O.word_stream(O.GEN_PHILOX4X32, key, 0, 0, 40)
    assert list(w) == k["philox4x32"]
    w = O.word_stream(O.GEN_THREEFRY2X64, k["threefry_key0"], k["threefry_key1"], 0, 40)
    joined = [int(w[2 * i]) | (int(w[2 * i + 1]) << 32) for i in range(20)]
    assert joined == k["threefry2x64"]
    # offsets: a window equals the slice of a longer stream
    full = O.word_stream(O.GEN_PHILOX4X32, 7, 0, 0, 1000)
    part = O.word_stream(O.GEN_PHILOX4X32, 7, 0, 333, 101)
    assert np.array_equal(full[333:434], part)


@pytest.mark.parametrize("gen", [0, 1])
def test_word_checksums_match_the_stream(gen):
    first, n = 5, 100003
    w = O.word_stream(gen, 0x0123456789ABCDEF, 77, first, n)
    s1, s2 = O.word_checksums(gen, 0x0123456789ABCDEF, 77, first, n)
    assert s1 == int(w.astype(np.uint64).sum())
    assert s2 == int((w ^ np.arange(n, dtype=np.uint32)).astype(np.uint64).sum())


def test_counter_carry():
    """Block 2^32 carries into the second counter word (philox.rs:89-91)."""
    w = O.word_stream(O.GEN_PHILOX4X32, 5, 0, 4 * (1 << 32), 4)
    assert list(w) == O.philox4x32([0, 1, 0, 0], [5, 0])


def test_transforms_accuracy():
    lib = O.lib()
    import ctypes
    lib.oracle_log_unit.restype = ctypes.c_float
    lib.oracle_log_unit.argtypes = [ctypes.c_float]
    us = np.random.default_rng(0).integers(1, 2 ** 24 + 1, 5000) * 2.0 ** -24
    err = max(abs(lib.oracle_log_unit(float(u)) - np.log(u)) / max(1.0, abs(np.log(u))) for u in us)
    assert err < 4e-7


def test_gaussian_statistics():
    S = O.sketch(O.DIST_GAUSSIAN, 256, 1000, key0=42)
    assert abs(S.mean()) < 0.01 and abs(S.var() - 1.0) < 0.01
    kurt = ((S - S.mean()) ** 4).mean() / S.var() ** 2
    assert abs(kurt - 3.0) < 0.05
    U = O.sketch(O.DIST_UNIFORM, 256, 1000, key0=42)
    assert U.min() > -1 and U.max() < 1 and abs(U.var() - 1 / 3) < 0.01
    R = O.sketch(O.DIST_RADEMACHER, 256, 1000, key0=42)
    assert set(np.unique(R)) == {-1.0, 1.0} and abs(R.mean()) < 0.01


def _qgauss_table():
    import re
    path = os.path.join(os.path.dirname(__file__), "..", "randnla_gb300", "csrc", "rnla_qgauss_table.h")
    return [int(v, 16) for v in re.findall(r"0x([0-9a-f]{8})u", open(path).read())]


def test_qgauss_table_is_the_discretised_gaussian():
    """The alias table reproduces P(t) = Phi((t+1/2)/8) - Phi((t-1/2)/8)
    (tails clamped at |t| = 63) to within the 2^-25 weight resolution."""
    tab = _qgauss_table()
    assert len(tab) == 128
    cap = 1 << 18
    got = [0] * 128
    for b, e in enumerate(tab):
        thr, own, ali = e & (cap - 1), (e >> 18) & 127, e >> 25
        assert own == b
        got[own] += thr
        got[ali] += cap - thr
    assert sum(got) == 1 << 25 and got[127] == 0
    phi = lambda x: 0.5 * math.erfc(-x / math.sqrt(2.0))
    for o in range(127):
        t = o - 63
        lo = -math.inf if t == -63 else (t - 0.5) / 8
        hi = math.inf if t == 63 else (t + 0.5) / 8
        p = (1.0 if hi == math.inf else phi(hi)) - (0.0 if lo == -math.inf else phi(lo))
        assert abs(got[o] / 2.0 ** 25 - p) <= 2.0 ** -25


def test_qgauss_lookup_matches_restatement():
    """The C oracle's lookup against a numpy restatement on random words."""
    tab = np.array(_qgauss_table(), dtype=np.uint64)
    rng = np.random.default_rng(5)
    u = rng.integers(0, 2 ** 32, size=4000, dtype=np.uint64)
    e = tab[u >> 25]
    x = (u >> 7) & 0x3FFFF
    o = np.where(x < (e & 0x3FFFF), (e >> 18) & 127, e >> 25).astype(np.int64) - 63
    got = np.array([O.lib().oracle_qgauss_t(int(v)) for v in u])
    assert np.array_equal(got, o)


def test_qgauss_64bit_entries_select_the_same_sample():
    """The tensor-core generator holds the alias table as 64-bit entries
    {threshold << 7, bf16(own t) | bf16(alias t) << 16} and selects with the
    masked word, (u & 0x01FFFF80) < threshold << 7, keeping the low or high
    half: a restatement of that rule gives the bf16 bits of qgauss_t(u) for
    every bucket and threshold edge."""
    tab = np.array(_qgauss_table(), dtype=np.uint64)
    thr, own, ali = tab & 0x3FFFF, ((tab >> 18) & 127).astype(np.int64) - 63, (tab >> 25).astype(np.int64) - 63

    def bf16_bits(t):
        return (np.asarray(t, dtype=np.float32).view(np.uint32) >> 16).astype(np.uint64)

    lo = thr << np.uint64(7)
    hi = bf16_bits(own) | (bf16_bits(ali) << np.uint64(16))
    rng = np.random.default_rng(9)
    u = rng.integers(0, 2 ** 32, size=20000, dtype=np.uint64)
    # the words at each bucket's threshold edge (x = thr - 1, thr) as well
    b = np.arange(128, dtype=np.uint64)
    for dx in (0, 1):
        x = np.maximum(thr.astype(np.int64) - dx, 0).astype(np.uint64)
        u = np.concatenate([u, (b << np.uint64(25)) | (x << np.uint64(7)) | np.uint64(0x55)])
    idx = (u >> np.uint64(25)).astype(np.int64)
    sel = np.where((u & np.uint64(0x01FFFF80)) < lo[idx], hi[idx], hi[idx] >> np.uint64(16)) & np.uint64(0xFFFF)
    x = (u >> np.uint64(7)) & np.uint64(0x3FFFF)
    t = np.where(x < thr[idx], own[idx], ali[idx])
    assert np.array_equal(sel, bf16_bits(t))


def test_quantized_sketch_grid():
    Q = O.sketch(O.DIST_GAUSSIAN, 64, 2000, key0=1, quantized=True)
    assert np.all(np.abs(Q * 8 - np.rint(Q * 8)) == 0) and np.abs(Q).max() <= 63 / 8
    # moments of round(8 g) / 8: mean 0, variance 1 + 1/768
    assert abs(Q.mean()) < 0.01 and abs(Q.var() - (1 + 1 / 768)) < 0.02
    # entry (i, j) is the alias sample of word i + j * rows4
    w = O.word_stream(O.GEN_PHILOX4X32, 1, 0, 0, 64 * 3)
    col = np.array([O.lib().oracle_qgauss_t(int(v)) for v in w[128:192]]) / 8
    assert np.array_equal(Q[:, 2], col)


def test_quantized_uniform_and_rademacher_grid():
    w = O.word_stream(O.GEN_PHILOX4X32, 3, 0, 0, 64 * 3).astype(np.int64)
    U = O.sketch(O.DIST_UNIFORM, 64, 3, key0=3, quantized=True)
    assert np.array_equal(U[:, 1], (2 * (w[64:128] >> 26) - 63) / 64)
    assert np.abs(U).max() <= 63 / 64 and np.all(np.abs(U * 64 - np.rint(U * 64)) == 0)
    Rm = O.sketch(O.DIST_RADEMACHER, 64, 3, key0=3, quantized=True)
    assert np.array_equal(Rm[:, 2], np.where(w[128:192] >> 31, 1.0, -1.0))
    big = O.sketch(O.DIST_UNIFORM, 64, 2000, key0=1, quantized=True)
    # midpoints of 64 equal cells of [-1, 1): mean 0, variance 1/3 - 1/(3 * 64^2)
    assert abs(big.mean()) < 0.01 and abs(big.var() - (1 / 3 - 1 / 12288)) < 0.01


def test_sketch_shape_errors():
    with pytest.raises(ValueError):
        O.sketch(O.DIST_GAUSSIAN, 0, 5)
    with pytest.raises(ValueError):
        O.sketch(O.DIST_GAUSSIAN, 5, 0)
