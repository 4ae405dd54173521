/*
 * ORACLE — test infrastructure only.  This file is the CPU restatement of the
 * counter-based generators used by the reference crate (divijkhaitan/randnla,
 * vendored `rust-random123`) plus the sketch-entry transform this project
 * defines on top of them.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it, and only as the checker: the product library
 * never links or calls it.
 *
 * Parity status
 *   - Philox2x32/2x64/4x32/4x64-10 and ThreeFry2x64-20 block functions:
 *     PINNED by the reference's own known-answer vectors
 *     (rust-random123/src/philox.rs:242-292,301-363;
 *      rust-random123/src/threefry.rs:97-127), copied into
 *     tests/golden/rng_kat.json and checked by tests/test_oracle_rng.py.
 *   - Stream order (block g = counter g, 128-bit little-endian counter with
 *     carry) follows philox.rs:87-99 and threefry.rs:13-21; words of a block
 *     are consumed in order, as rand_core's BlockRng does for 32-bit draws
 *     (rust-random123/src/rng.rs:15-21,85,93).
 *   - Key from seed: the little-endian bytes of the seed (philox.rs:101-105,
 *     threefry.rs:23-27).  rand_core's `seed_from_u64` expansion lives in the
 *     absent third-party crate rand_core 0.6.4 and is NOT reproduced.
 *   - Gaussian / Uniform / Rademacher transforms: the reference draws through
 *     rand_distr 0.4.3 (sketch.rs:114-126), which is absent here, so sketch
 *     VALUES are parity-unpinned against the reference.  This project defines
 *     its own transform (Box-Muller in binary32 using only correctly rounded
 *     +,-,*,/,sqrt and fma, with series for log and sin/cos written from
 *     their Taylor expansions), so the GPU generator and this oracle agree
 *     bit for bit.
 *   - Quantised Gaussian of the tensor-core sketch: this project's own
 *     definition, an alias-table sample of round(8 g) clamped to [-63, 63]
 *     per 32-bit word; the table (rnla_qgauss_table.h, shared data) is
 *     checked against the exact discretised-Gaussian probabilities by
 *     tests/test_oracle_rng.py, and the lookup below is written separately
 *     from the CUDA one.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (see oracle/build_oracle.sh).
 * -ffp-contract=off matters: every fused multiply-add below is an explicit
 * fmaf() call, and no other a*b+c may be contracted.
 */
#include "../randnla_gb300/csrc/rnla_qgauss_table.h"
#include <stdint.h>
#include <string.h>
#include <math.h>

/* ------------------------------------------------------------------ */
/* Philox (rust-random123/src/philox.rs:16-27 constants)               */
/* ------------------------------------------------------------------ */
#define PHILOX_M2X64_0 0xD2B74407B1CE6E93ULL
#define PHILOX_M4X64_0 0xD2E7470EE14C6C93ULL
#define PHILOX_M4X64_1 0xCA5A826395121157ULL
#define PHILOX_W64_0   0x9E3779B97F4A7C15ULL
#define PHILOX_W64_1   0xBB67AE8584CAA73BULL
#define PHILOX_M2X32_0 0xd256d193U
#define PHILOX_M4X32_0 0xD2511F53U
#define PHILOX_M4X32_1 0xCD9E8D57U
#define PHILOX_W32_0   0x9E3779B9U
#define PHILOX_W32_1   0xBB67AE85U

static void mul32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}
static void mul64(uint64_t a, uint64_t b, uint64_t *hi, uint64_t *lo) {
    unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
    *hi = (uint64_t)(p >> 64);
    *lo = (uint64_t)p;
}

/* philox.rs:183-195 — ten rounds, key bumped by the Weyl constant between rounds */
void oracle_philox2x32(const uint32_t ctr_in[2], const uint32_t key_in[1], uint32_t out[2]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], k0 = key_in[0];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) k0 += PHILOX_W32_0;
        uint32_t hi, lo;
        mul32(PHILOX_M2X32_0, c0, &hi, &lo);          /* philox.rs:138-141 */
        c0 = hi ^ k0 ^ c1;
        c1 = lo;
    }
    out[0] = c0; out[1] = c1;
}

/* philox.rs:197-209 */
void oracle_philox2x64(const uint64_t ctr_in[2], const uint64_t key_in[1], uint64_t out[2]) {
    uint64_t c0 = ctr_in[0], c1 = ctr_in[1], k0 = key_in[0];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) k0 += PHILOX_W64_0;
        uint64_t hi, lo;
        mul64(PHILOX_M2X64_0, c0, &hi, &lo);          /* philox.rs:144-147 */
        c0 = hi ^ k0 ^ c1;
        c1 = lo;
    }
    out[0] = c0; out[1] = c1;
}

/* philox.rs:211-223 with the round of philox.rs:150-154 */
void oracle_philox4x32(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr_in[0], ctr_in[1], ctr_in[2], ctr_in[3]};
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += PHILOX_W32_0; k1 += PHILOX_W32_1; }   /* philox.rs:174-176 */
        uint32_t hi0, lo0, hi1, lo1;
        mul32(PHILOX_M4X32_0, c[0], &hi0, &lo0);
        mul32(PHILOX_M4X32_1, c[2], &hi1, &lo1);
        uint32_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    }
    memcpy(out, c, sizeof c);
}

/* philox.rs:225-237 with the round of philox.rs:157-161 */
void oracle_philox4x64(const uint64_t ctr_in[4], const uint64_t key_in[2], uint64_t out[4]) {
    uint64_t c[4] = {ctr_in[0], ctr_in[1], ctr_in[2], ctr_in[3]};
    uint64_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += PHILOX_W64_0; k1 += PHILOX_W64_1; }   /* philox.rs:178-181 */
        uint64_t hi0, lo0, hi1, lo1;
        mul64(PHILOX_M4X64_0, c[0], &hi0, &lo0);
        mul64(PHILOX_M4X64_1, c[2], &hi1, &lo1);
        uint64_t n0 = hi1 ^ c[1] ^ k0, n1 = lo1, n2 = hi0 ^ c[3] ^ k1, n3 = lo0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
    }
    memcpy(out, c, sizeof c);
}

/* ------------------------------------------------------------------ */
/* ThreeFry2x64-20 (rust-random123/src/threefry.rs:30-93)              */
/* ------------------------------------------------------------------ */
static uint64_t rotl64(uint64_t x, unsigned r) { return (x << r) | (x >> (64 - r)); }

void oracle_threefry2x64(const uint64_t ctr[2], const uint64_t key[2], uint64_t out[2]) {
    static const unsigned R[8] = {16, 42, 12, 31, 16, 32, 24, 21};   /* threefry.rs:34-41 */
    const uint64_t parity = 0x1BD11BDAA9FC1A22ULL;                   /* threefry.rs:30-32 */
    uint64_t ks[3] = {key[0], key[1], parity ^ key[0] ^ key[1]};
    uint64_t x0 = ctr[0], x1 = ctr[1];
    /* five groups of four mix rounds, a key injection after each group (threefry.rs:77-92) */
    for (int inj = 0; inj <= 5; ++inj) {
        x0 += ks[inj % 3];
        x1 += ks[(inj + 1) % 3];
        x1 += (uint64_t)inj;
        if (inj == 5) break;
        const unsigned *rot = (inj % 2 == 0) ? &R[0] : &R[4];
        for (int r = 0; r < 4; ++r) {
            x0 += x1; x1 = rotl64(x1, rot[r]); x1 ^= x0;
        }
    }
    out[0] = x0; out[1] = x1;
}

/* ------------------------------------------------------------------ */
/* Streams: block g of a generator = its output at counter value g       */
/* ------------------------------------------------------------------ */
enum { GEN_PHILOX4X32 = 0, GEN_THREEFRY2X64 = 1 };

/* Four 32-bit words of block g.  Philox4x32: the four output words
   (key = little-endian halves of key0, philox.rs:101-105).  ThreeFry2x64:
   the low then high half of each 64-bit output word. */
static void block_words(int gen, uint64_t key0, uint64_t key1, uint64_t g, uint32_t w[4]) {
    if (gen == GEN_PHILOX4X32) {
        uint32_t ctr[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0, 0};
        uint32_t key[2] = {(uint32_t)key0, (uint32_t)(key0 >> 32)};
        oracle_philox4x32(ctr, key, w);
    } else {
        uint64_t ctr[2] = {g, 0}, key[2] = {key0, key1}, o[2];
        oracle_threefry2x64(ctr, key, o);
        w[0] = (uint32_t)o[0]; w[1] = (uint32_t)(o[0] >> 32);
        w[2] = (uint32_t)o[1]; w[3] = (uint32_t)(o[1] >> 32);
    }
}

/* The 32-bit word stream x_0, x_1, ... with x_{4g+k} = word k of block g
   (the next_u32 sequence of Philox4x32Rng, rng.rs:85,93). */
void oracle_word_stream(int gen, uint64_t key0, uint64_t key1, uint64_t first_word,
                        int64_t n, uint32_t *out) {
    for (int64_t t = 0; t < n; ++t) {
        uint64_t L = first_word + (uint64_t)t;
        uint32_t w[4];
        block_words(gen, key0, key1, L >> 2, w);
        out[t] = w[L & 3];
    }
}

/* Checksums of n stream words from first_word, one block evaluation per
 * four words: s1 = sum of the words, s2 = sum of (word xor the low 32 bits
 * of its offset t), both mod 2^64.  s2 changes when words trade places. */
void oracle_word_checksums(int gen, uint64_t key0, uint64_t key1, uint64_t first_word,
                           int64_t n, uint64_t *s1, uint64_t *s2) {
    uint64_t a = 0, b = 0;
    int64_t t = 0;
    while (t < n) {
        uint64_t L = first_word + (uint64_t)t;
        uint32_t w[4];
        block_words(gen, key0, key1, L >> 2, w);
        for (unsigned j = (unsigned)(L & 3); j < 4 && t < n; ++j, ++t) {
            a += w[j];
            b += (uint64_t)(w[j] ^ (uint32_t)t);
        }
    }
    *s1 = a;
    *s2 = b;
}

/* ------------------------------------------------------------------ */
/* Sketch-entry transforms (this project's definition; see header)     */
/* ------------------------------------------------------------------ */
static float u32_as_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t f_as_u32(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

/* natural log of u in (0, 1], u a normal binary32 number.
   ln u = e ln2 + 2 atanh(s), s = (f-1)/(f+1), f in [sqrt(1/2), sqrt(2)). */
float oracle_log_unit(float u) {
    uint32_t b = f_as_u32(u);
    int e = (int)((b >> 23) & 0xffu) - 127;
    uint32_t fb = (b & 0x7fffffu) | 0x3f800000u;
    float f = u32_as_f(fb);
    if (fb > 0x3fb504f3u) { f = f * 0.5f; e += 1; }
    float s = (f - 1.0f) / (f + 1.0f);
    float z = s * s;
    float p = 0x1.3b13b2p-3f;                 /* 2/13 */
    p = fmaf(p, z, 0x1.745d18p-3f);           /* 2/11 */
    p = fmaf(p, z, 0x1.c71c72p-3f);           /* 2/9  */
    p = fmaf(p, z, 0x1.24924ap-2f);           /* 2/7  */
    p = fmaf(p, z, 0x1.99999ap-2f);           /* 2/5  */
    p = fmaf(p, z, 0x1.555556p-1f);           /* 2/3  */
    float sz = s * z;
    float lnf = fmaf(sz, p, 2.0f * s);
    float ef = (float)e;
    float t = fmaf(ef, 0x1.7f7d1cp-20f, lnf); /* e * (ln2 - hi) */
    return fmaf(ef, 0x1.62e4p-1f, t);         /* e * hi, exact product */
}

/* cos(2 pi u), sin(2 pi u) for u in [0, 1): quadrant q = rint(4u), w = 4u - q
   in [-1/2, 1/2], Taylor series of sin/cos(w pi/2). */
void oracle_sincos_2pi(float u, float *c_out, float *s_out) {
    float t = u * 4.0f;
    float q = rintf(t);
    float w = t - q;
    float z = w * w;
    float sp = 0x1.507834p-13f;
    sp = fmaf(sp, z, -0x1.32d2ccp-8f);
    sp = fmaf(sp, z, 0x1.466bc6p-4f);
    sp = fmaf(sp, z, -0x1.4abbcep-1f);
    sp = fmaf(sp, z, 0x1.921fb6p+0f);
    float sn = w * sp;
    float cp = -0x1.a6d1f2p-16f;
    cp = fmaf(cp, z, 0x1.e1f506p-11f);
    cp = fmaf(cp, z, -0x1.55d3c8p-6f);
    cp = fmaf(cp, z, 0x1.03c1f0p-2f);
    cp = fmaf(cp, z, -0x1.3bd3ccp+0f);
    float cs = fmaf(cp, z, 1.0f);
    int qi = ((int)q) & 3;
    switch (qi) {
        case 0: *c_out = cs;  *s_out = sn;  break;
        case 1: *c_out = -sn; *s_out = cs;  break;
        case 2: *c_out = -cs; *s_out = -sn; break;
        default: *c_out = sn; *s_out = -cs; break;
    }
}

/* Box-Muller on two words: u1 in (0,1], u2 in [0,1), 24-bit resolution. */
void oracle_gauss_pair(uint32_t a, uint32_t b, float *g0, float *g1) {
    float u1 = (float)((a >> 8) + 1u) * 0x1p-24f;
    float u2 = (float)(b >> 8) * 0x1p-24f;
    float r = sqrtf(-2.0f * oracle_log_unit(u1));
    float c, s;
    oracle_sincos_2pi(u2, &c, &s);
    *g0 = r * c;
    *g1 = r * s;
}

/* U(-1,1): (k - 2^23) 2^-23 + 2^-24, k = word >> 8; every value is exact. */
float oracle_uniform_pm1(uint32_t a) {
    return (float)((int32_t)(a >> 8) - 0x800000) * 0x1p-23f + 0x1p-24f;
}

enum { DIST_GAUSSIAN = 0, DIST_UNIFORM = 1, DIST_RADEMACHER = 2 };

/* Sketch entry (i, j) of a rows x cols operator uses word L = i + j*rows4,
   rows4 = rows rounded up to a multiple of 4; Gaussian entries come in
   Box-Muller pairs (words 0,1 and 2,3 of a block). */
float oracle_sketch_entry(int dist, int gen, uint64_t key0, uint64_t key1,
                          int64_t rows, int64_t i, int64_t j) {
    int64_t rows4 = (rows + 3) & ~(int64_t)3;
    uint64_t L = (uint64_t)(i + j * rows4);
    uint32_t w[4];
    block_words(gen, key0, key1, L >> 2, w);
    unsigned lane = (unsigned)(L & 3);
    if (dist == DIST_GAUSSIAN) {
        float g0, g1;
        unsigned p = lane >> 1;
        oracle_gauss_pair(w[2 * p], w[2 * p + 1], &g0, &g1);
        return (lane & 1) ? g1 : g0;
    } else if (dist == DIST_UNIFORM) {
        return oracle_uniform_pm1(w[lane]);
    } else {
        return (w[lane] >> 31) ? 1.0f : -1.0f;
    }
}

/* Dense column-major fill, ld >= rows. */
void oracle_sketch_fill(int dist, int gen, uint64_t key0, uint64_t key1,
                        int64_t rows, int64_t cols, float *out, int64_t ld) {
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i)
            out[i + j * ld] = oracle_sketch_entry(dist, gen, key0, key1, rows, i, j);
}

/* Columns [j0, j1) of the same dense operator into out (column j - j0), so
   callers can generate a large sketch in column blocks (and in parallel,
   one block per thread) without holding all of it. */
void oracle_sketch_fill_cols(int dist, int gen, uint64_t key0, uint64_t key1,
                             int64_t rows, int64_t j0, int64_t j1, float *out, int64_t ld) {
    for (int64_t j = j0; j < j1; ++j)
        for (int64_t i = 0; i < rows; ++i)
            out[i + (j - j0) * ld] = oracle_sketch_entry(dist, gen, key0, key1, rows, i, j);
}

/* Quantised Gaussian used by the tensor-core sketch: t = round(8 g) clamped
   to [-63, 63], g ~ N(0, 1), drawn from one 32-bit word with the Walker
   alias table of rnla_qgauss_table.h (generated by make_qgauss_table.py:
   P(t) = W_t / 2^25).  Entry (i, j) uses word L = i + j*rows4, like every
   other distribution.  Returns t / 8. */
static const uint32_t QGAUSS[128] = RNLA_QGAUSS_INIT;

int oracle_qgauss_t(uint32_t u) {
    uint32_t e = QGAUSS[u >> 25];
    uint32_t x = (u >> 7) & 0x3FFFFu;
    uint32_t o = (x < (e & 0x3FFFFu)) ? ((e >> 18) & 0x7Fu) : (e >> 25);
    return (int)o - 63;
}

void oracle_sketch_fill_quantized(int gen, uint64_t key0, uint64_t key1,
                                  int64_t rows, int64_t cols, float *out, int64_t ld) {
    int64_t rows4 = (rows + 3) & ~(int64_t)3;
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) {
            uint64_t L = (uint64_t)(i + j * rows4);
            uint32_t w[4];
            block_words(gen, key0, key1, L >> 2, w);
            out[i + j * ld] = (float)oracle_qgauss_t(w[L & 3]) * 0.125f;
        }
}

/* The quantised uniform and Rademacher sketches (this library's own
 * definitions, restated from the word): dist 1 gives (2 (u >> 26) - 63) / 64,
 * dist 2 gives +-1 from the top bit; dist 0 is the Gaussian above. */
void oracle_sketch_fill_quantized_dist(int dist, int gen, uint64_t key0, uint64_t key1,
                                       int64_t rows, int64_t cols, float *out, int64_t ld) {
    if (dist == 0) {
        oracle_sketch_fill_quantized(gen, key0, key1, rows, cols, out, ld);
        return;
    }
    int64_t rows4 = (rows + 3) & ~(int64_t)3;
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) {
            uint64_t L = (uint64_t)(i + j * rows4);
            uint32_t w[4];
            block_words(gen, key0, key1, L >> 2, w);
            uint32_t u = w[L & 3];
            out[i + j * ld] = (dist == 1) ? (float)(2 * (int)(u >> 26) - 63) / 64.0f : ((u >> 31) ? 1.0f : -1.0f);
        }
}
