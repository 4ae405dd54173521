// Counter-based generators and sketch-entry transforms, device side.
//
// Philox4x32-10 and ThreeFry2x64-20 reproduce the block functions of the
// reference's vendored rust-random123 (philox.rs:150-154,174-176,211-223;
// threefry.rs:30-93) bit for bit; the block index is the counter value, as
// in the stateful `next()` of philox.rs:87-99 / threefry.rs:13-21.
//
// The Gaussian transform is this library's own: Box-Muller in binary32 with
// log and sin/cos evaluated from their Taylor series using only correctly
// rounded operations (__fadd_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn and
// explicit __fmaf_rn), so host checkers compiled without contraction
// reproduce every value exactly.
#pragma once
#include <cstdint>
#include "rnla_qgauss_table.h"

namespace rnla {

enum { GEN_PHILOX4X32 = 0, GEN_THREEFRY2X64 = 1 };
enum { DIST_GAUSSIAN = 0, DIST_UNIFORM = 1, DIST_RADEMACHER = 2 };

struct RngKey {
    int gen;
    uint64_t k0, k1;
};

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    }
}

__device__ __forceinline__ uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

__device__ __forceinline__ void threefry2x64_20(uint64_t& x0, uint64_t& x1, uint64_t key0, uint64_t key1) {
    const uint64_t ks2 = 0x1BD11BDAA9FC1A22ULL ^ key0 ^ key1;
    const uint64_t ks[3] = {key0, key1, ks2};
    const int R0[4] = {16, 42, 12, 31}, R1[4] = {16, 32, 24, 21};
#pragma unroll
    for (int inj = 0; inj <= 5; ++inj) {
        x0 += ks[inj % 3];
        x1 += ks[(inj + 1) % 3] + (uint64_t)inj;
        if (inj == 5) break;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            x0 += x1;
            x1 = rotl64(x1, (inj & 1) ? R1[r] : R0[r]);
            x1 ^= x0;
        }
    }
}

// Four 32-bit words of block g.
__device__ __forceinline__ void block_words(const RngKey& k, uint64_t g, uint32_t w[4]) {
    if (k.gen == GEN_PHILOX4X32) {
        w[0] = (uint32_t)g; w[1] = (uint32_t)(g >> 32); w[2] = 0u; w[3] = 0u;
        philox4x32_10(w, (uint32_t)k.k0, (uint32_t)(k.k0 >> 32));
    } else {
        uint64_t x0 = g, x1 = 0;
        threefry2x64_20(x0, x1, k.k0, k.k1);
        w[0] = (uint32_t)x0; w[1] = (uint32_t)(x0 >> 32);
        w[2] = (uint32_t)x1; w[3] = (uint32_t)(x1 >> 32);
    }
}

// ln(u) for u in (0, 1] (normal binary32): u = 2^e f, f in [sqrt(1/2), sqrt(2)),
// ln f = 2 atanh(s) with s = (f-1)/(f+1), atanh series through s^13.
__device__ __forceinline__ float log_unit(float u) {
    const uint32_t b = __float_as_uint(u);
    int e = (int)((b >> 23) & 0xffu) - 127;
    const uint32_t fb = (b & 0x7fffffu) | 0x3f800000u;
    float f = __uint_as_float(fb);
    if (fb > 0x3fb504f3u) { f = __fmul_rn(f, 0.5f); e += 1; }
    const float s = __fdiv_rn(__fsub_rn(f, 1.0f), __fadd_rn(f, 1.0f));
    const float z = __fmul_rn(s, s);
    float p = 0x1.3b13b2p-3f;
    p = __fmaf_rn(p, z, 0x1.745d18p-3f);
    p = __fmaf_rn(p, z, 0x1.c71c72p-3f);
    p = __fmaf_rn(p, z, 0x1.24924ap-2f);
    p = __fmaf_rn(p, z, 0x1.99999ap-2f);
    p = __fmaf_rn(p, z, 0x1.555556p-1f);
    const float lnf = __fmaf_rn(__fmul_rn(s, z), p, __fmul_rn(2.0f, s));
    const float ef = (float)e;
    const float t = __fmaf_rn(ef, 0x1.7f7d1cp-20f, lnf);
    return __fmaf_rn(ef, 0x1.62e4p-1f, t);
}

// (cos 2 pi u, sin 2 pi u) for u in [0, 1): quadrant q = rint(4u),
// w = 4u - q in [-1/2, 1/2], series of sin/cos(w pi/2).
__device__ __forceinline__ void sincos_2pi(float u, float& c_out, float& s_out) {
    const float t = __fmul_rn(u, 4.0f);
    const float q = rintf(t);
    const float w = __fsub_rn(t, q);
    const float z = __fmul_rn(w, w);
    float sp = 0x1.507834p-13f;
    sp = __fmaf_rn(sp, z, -0x1.32d2ccp-8f);
    sp = __fmaf_rn(sp, z, 0x1.466bc6p-4f);
    sp = __fmaf_rn(sp, z, -0x1.4abbcep-1f);
    sp = __fmaf_rn(sp, z, 0x1.921fb6p+0f);
    const float sn = __fmul_rn(w, sp);
    float cp = -0x1.a6d1f2p-16f;
    cp = __fmaf_rn(cp, z, 0x1.e1f506p-11f);
    cp = __fmaf_rn(cp, z, -0x1.55d3c8p-6f);
    cp = __fmaf_rn(cp, z, 0x1.03c1f0p-2f);
    cp = __fmaf_rn(cp, z, -0x1.3bd3ccp+0f);
    const float cs = __fmaf_rn(cp, z, 1.0f);
    switch (((int)q) & 3) {
        case 0: c_out = cs;  s_out = sn;  break;
        case 1: c_out = -sn; s_out = cs;  break;
        case 2: c_out = -cs; s_out = -sn; break;
        default: c_out = sn; s_out = -cs; break;
    }
}

__device__ __forceinline__ void gauss_pair(uint32_t a, uint32_t b, float& g0, float& g1) {
    const float u1 = __fmul_rn((float)((a >> 8) + 1u), 0x1p-24f);
    const float u2 = __fmul_rn((float)(b >> 8), 0x1p-24f);
    const float r = __fsqrt_rn(__fmul_rn(-2.0f, log_unit(u1)));
    float c, s;
    sincos_2pi(u2, c, s);
    g0 = __fmul_rn(r, c);
    g1 = __fmul_rn(r, s);
}

__device__ __forceinline__ float uniform_pm1(uint32_t a) {
    return __fadd_rn(__fmul_rn((float)((int32_t)(a >> 8) - 0x800000), 0x1p-23f), 0x1p-24f);
}

// Quantised Gaussian of the tensor-core sketch: t = round(8 g) clamped to
// [-63, 63] for g ~ N(0, 1), drawn from one 32-bit word through the alias
// table of rnla_qgauss_table.h (P(t) = W_t / 2^25).  t / 8 is exact in bf16
// and the digit products of the tensor-core sketch stay below 2^13.
static __device__ const uint32_t k_qgauss_table[128] = RNLA_QGAUSS_INIT;

__device__ __forceinline__ int qgauss_t(uint32_t u, const uint32_t* tab) {
    const uint32_t e = tab[u >> 25];
    const uint32_t x = (u >> 7) & 0x3FFFFu;
    const uint32_t o = (x < (e & 0x3FFFFu)) ? ((e >> 18) & 0x7Fu) : (e >> 25);
    return (int)o - 63;
}

// Quantised entries of the tensor-core sketch for each distribution: an
// integer t with |t| <= 63 (so t is exact in bf16 and the digit products stay
// below 2^14) and the scale 2^-qshift(dist) that makes t 2^-qshift the entry.
//   Gaussian    t = qgauss_t(u), entry t / 8
//   Uniform     t = 2 (u >> 26) - 63 (odd, -63..63), entry t / 64: the midpoint
//               of the 1/32-wide bin holding the unquantised U(-1, 1) value
//               uniform_pm1(u) (both come from the top bits of u)
//   Rademacher  t = +-1 from the top bit, entry t (already exact)
__device__ __forceinline__ int quant_t(int dist, uint32_t u, const uint32_t* tab) {
    if (dist == DIST_GAUSSIAN) return qgauss_t(u, tab);
    if (dist == DIST_UNIFORM) return 2 * (int)(u >> 26) - 63;
    return (u >> 31) ? 1 : -1;
}
__host__ __device__ constexpr int quant_shift(int dist) {
    return dist == DIST_GAUSSIAN ? 3 : dist == DIST_UNIFORM ? 6 : 0;
}

// The four entries generated by block g for distribution `dist`.
__device__ __forceinline__ void block_entries(const RngKey& k, int dist, uint64_t g, float v[4]) {
    uint32_t w[4];
    block_words(k, g, w);
    if (dist == DIST_GAUSSIAN) {
        gauss_pair(w[0], w[1], v[0], v[1]);
        gauss_pair(w[2], w[3], v[2], v[3]);
    } else if (dist == DIST_UNIFORM) {
#pragma unroll
        for (int i = 0; i < 4; ++i) v[i] = uniform_pm1(w[i]);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) v[i] = (w[i] >> 31) ? 1.0f : -1.0f;
    }
}

}  // namespace rnla
