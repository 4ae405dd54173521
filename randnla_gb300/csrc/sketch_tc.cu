// Tensor-core sketch application for sm_103a (tcgen05 + TMEM + bulk async copies).
//
//   C (M x N, FP64) = S Y,   S (M x K) the quantised Gaussian sketch t / 8
//   (t = round(8 g) clamped to [-63, 63], drawn per Philox word through the
//   alias table of rnla_qgauss_table.h; exact in bf16), Y (K x N) an FP64 or
//   FP32 matrix, K = rows of the data (the sketch_and_precondition.rs:51-52
//   products S a and S b, and A Omega of the range finder).
//
// Exactness.  Y is cut into P <= 4 bf16 "digits" per element: with E_j the
// exponent of the largest |Y[:, j]| (|y| < 2^E_j), T = round(|y| 2^(8P-E_j))
// <= 2^(8P) is split into base-256 digits d_1..d_P (d_1 <= 256), each
// carrying the sign of y (an integer of at most 8 significant bits: exact in
// bf16).  A digit times a sketch entry is an integer of magnitude
// <= 256*63 < 2^14, so the FP32 tensor-core accumulation of 1024 consecutive
// K (one "window") is an integer below 2^24: exact.  After each window the
// drain warps read the P accumulators from TMEM and fold
// D_1 2^(8(P-1)) + ... + D_P exactly into int64 accumulators held in their
// registers (|window| < 2^48.01); a work unit ends with one store of its
// int64 tile.  The split-K partials are added in a fixed order (in int64
// when all windows together fit) and scaled once by 2^(E_j - 8P - 3).  The
// only roundings are the digit truncation (|error| <= 2^(E_j - 8P - 1) per
// entry of Y) and the final conversion to FP64; S is applied exactly.
//
// Pipeline.
//   sketch_gen_gauss_kernel (sketch_gen_kernel for the other distributions
//                      and ThreeFry keys) writes S once as bf16 tile images
//                      [m tile][K stage] (128 x 64, the exact SWIZZLE_128B
//                      K-major shared-memory layout), 16 KB each: 2 bytes per
//                      entry of HBM traffic instead of generating S inside
//                      the GEMM;
//   colexp_kernel      the column exponents E_j;
//   slice_kernel       writes the digit planes of Y as tile images
//                      [n tile][K stage][digit] (W x 64 bf16, W = 80 for
//                      P <= 3 and 64 for P = 4); slice_rowmajor_kernel the
//                      same for FP32 data together with the solver's
//                      row-major copy of Y from the same reads;
//   sketch_mma_kernel  persistent: one CTA per SM walks the work units
//                      (m tile, n tile, K chunk) u = blockIdx.x, + gridDim.x,
//                      ...; 192 threads: warp 0 streams the S tile and the P
//                      digit tiles of each stage with cp.async.bulk into a
//                      4- or 5-stage mbarrier ring that runs on across units;
//                      warp 1 allocates TMEM and issues tcgen05.mma
//                      (M = 128, N = W P, K = 16, bf16 x bf16 -> f32: the
//                      P digit tiles are one operand, so digit p accumulates
//                      in TMEM columns [W p, W p + W); two sets so the MMAs
//                      of a window overlap the drain of the previous one)
//                      from one lane; warps 2-5 drain TMEM after each
//                      window.  Units that share an S tile are adjacent in
//                      the walk, so S is read from HBM about once and served
//                      from L2 to the other column tiles;
//   splitk_sum_kernel  adds the K chunks and scales.
//
// Every mbarrier wait is bounded (2 s of globaltimer); on timeout the CTA
// records an error, drains its own bulk copies and MMAs, frees TMEM and exits.
#include "rnla_internal.h"
#include "rnla_async.cuh"
#include "rnla_tc.cuh"
#include <cuda_bf16.h>
#include <vector>
#include <algorithm>
#include <cstring>
#include <functional>

namespace rnla {

namespace tc {

constexpr int BM = 128;           // sketch rows per CTA tile (TMEM lanes)
constexpr int BN = (int)TC_TILE_COLS; // data columns per CTA tile
constexpr int BK = 64;            // K per pipeline stage (one 128-byte bf16 row)
constexpr int WIN = 16;           // stages per exact window (1024 K values)
constexpr int MAXP = 4;           // digits
constexpr int ACC_COLS = MAXP * BN;                  // TMEM columns of one accumulator set
// Column tile width of a launch's digit planes: one MMA covers the P planes
// of a tile (N = P x width), so the sketch's own launches use 80 columns for
// P <= 3 (N = 240: fewer operand bytes per MMA flop than 64-column tiles, and
// 13 tiles for 1025 columns instead of 17 with 6% padding) and 64 for P = 4
// (N = 256); the exact X^T Y product keeps 64-column planes for every P.
__host__ __device__ constexpr int bn_for(int P) { return P <= 3 ? 80 : 64; }
// ring depth: as many 16 KB + P x (width x 128 B) stages as fit in ~200 KB
// (4 for P = 4 at 64 columns and for every P at 80, 5 for P <= 3 at 64), the
// operand stream from L2 being latency-bound
__host__ __device__ constexpr int stages_for(int P, int BNT) { return BNT == 64 ? (P >= 4 ? 4 : 5) : 4; }
constexpr int DRAIN_WARPS = 4;
constexpr int THREADS = 64 + 32 * DRAIN_WARPS;       // loader warp + MMA warp + drain warps
constexpr int S_BYTES = BM * BK * 2;                 // 16 KB sketch tile
constexpr int ROW_BYTES = BK * 2;                    // 128
constexpr int YD_BYTES = BN * ROW_BYTES;             // one 64-column digit tile, 8 KB
constexpr unsigned long long WAIT_NS = 2000000000ull;

// acc += (integer value of the FP32 word f) * 2^sh, exact in int64 (sh < 31)
__device__ __forceinline__ void acc_digit(long long& acc, uint32_t f, int sh) {
    const int d = __float2int_rn(__uint_as_float(f));
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(acc) : "r"(d), "r"(1 << sh));
}

struct Params {
    int64_t M, N, K;          // C is M x N, reduction length K
    int tiles_m, tiles_n, Ks, kc_count, stages_per_kc;
    int units;                // work units of this launch
    int jt0, jt_count;        // the column tiles [jt0, jt0 + jt_count) of this launch
    int it0, it_count;        // the row tiles [it0, it0 + it_count) of this launch
    const uint8_t* sk;        // sketch tiles [it][stage] (SW128 images, 16 KB)
    const uint16_t* ydig;     // digit planes [jt][stage][p][width rows][64] bf16 (SW128 images)
    int ypl;                  // planes stored per stage in ydig (>= P; the first P are used)
    long long* partial;       // [kc][tile][width][BM] exact integer sums (row fastest)
    unsigned int* status;
};

// The four quantised entries t (integers, |t| <= 63) of block g.
__device__ __forceinline__ void sketch_block(const RngKey& key, int dist, uint64_t g, const uint32_t* tab,
                                             float v[4]) {
    uint32_t w[4];
    block_words(key, g, w);
#pragma unroll
    for (int t = 0; t < 4; ++t) v[t] = (float)quant_t(dist, w[t], tab);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    // both values are integers with |t| <= 63: exact in bf16 (truncation is exact)
    return (__float_as_uint(lo) >> 16) | (__float_as_uint(hi) & 0xFFFF0000u);
}

// S tile images.  Block (x, y = m tile): a thread per (4 rows, 2 consecutive
// K) unit of a stage; a warp covers 4 rows x 64 K, i.e. four whole 128-byte
// rows of the image, so stores are coalesced.  Entry (i, k) is word
// i + k * round_up(M, 4) of the stream (block (i >> 2) + k * M4 / 4).
__global__ void __launch_bounds__(256) sketch_gen_kernel(RngKey key, int dist, int64_t M, int64_t K, int Ks,
                                                         int it0, uint8_t* __restrict__ S) {
    __shared__ uint32_t qtab[128];
    if (threadIdx.x < 128) qtab[threadIdx.x] = k_qgauss_table[threadIdx.x];
    __syncthreads();
    const int it = it0 + blockIdx.y;
    const uint64_t gstride = (uint64_t)(((M + 3) & ~3LL) >> 2);
    const int64_t units = (int64_t)Ks * 1024;            // 32 row groups x 32 K pairs per stage
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < units;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int kp = (int)(u & 31), ig = (int)((u >> 5) & 31);
        const int64_t s = u >> 10;
        const int64_t row0 = (int64_t)it * BM + 4 * ig;
        const int64_t k = s * BK + 2 * kp;
        float v0[4] = {0.f, 0.f, 0.f, 0.f}, v1[4] = {0.f, 0.f, 0.f, 0.f};
        if (row0 < M && k < K) sketch_block(key, dist, (uint64_t)(row0 >> 2) + (uint64_t)k * gstride, qtab, v0);
        if (row0 < M && k + 1 < K)
            sketch_block(key, dist, (uint64_t)(row0 >> 2) + (uint64_t)(k + 1) * gstride, qtab, v1);
        uint8_t* tile = S + ((size_t)it * Ks + (size_t)s) * S_BYTES;
        const int kl = 2 * kp;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int r = 4 * ig + t;
            const bool rv = row0 + t < M;
            uint32_t* qd = (uint32_t*)(tile + r * ROW_BYTES + ((((kl >> 3) ^ (r & 7))) << 4) + ((kl & 7) << 1));
            *qd = pack_bf16(rv ? v0[t] : 0.f, rv ? v1[t] : 0.f);
        }
    }
}

// The same S tile images for Gaussian entries of a Philox key, bit for bit,
// with fewer instructions on the integer ALU pipe, which bounds the
// generator (and which the digit-plane kernels running beside it need too):
//  * block x takes the whole stages x, x + gridDim.x, ... of m tile it, so a
//    thread keeps its K pair kp and row groups igq + 8 q (q = 0..3) from
//    stage to stage, and with them the swizzled store offsets;
//  * the alias table sits in shared memory as 64-bit entries
//    {threshold << 7, bf16(own t) | bf16(alias t) << 16}: an entry is a
//    shift, a 64-bit load, a masked compare and a select -- the masked word
//    (u & 0x01FFFF80) < threshold << 7 is the x < threshold of qgauss_t --
//    and no integer-to-float conversion; two entries pack with one byte
//    permute.
__device__ __forceinline__ void gauss_block_bf16(const RngKey& key, uint64_t g, const uint2* qt, uint32_t r[4]) {
    uint32_t w[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u};
    philox4x32_10(w, (uint32_t)key.k0, (uint32_t)(key.k0 >> 32));
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint2 e = qt[w[i] >> 25];
        r[i] = ((w[i] & 0x01FFFF80u) < e.x) ? e.y : (e.y >> 16);     // low 16 bits: bf16 of t
    }
}

__global__ void __launch_bounds__(256) sketch_gen_gauss_kernel(RngKey key, int64_t M, int64_t K, int Ks, int it0,
                                                               uint8_t* __restrict__ S) {
    __shared__ uint2 qt[128];
    if (threadIdx.x < 128) {
        const uint32_t e = k_qgauss_table[threadIdx.x];
        const float own = (float)((int)((e >> 18) & 0x7Fu) - 63), ali = (float)((int)(e >> 25) - 63);
        qt[threadIdx.x] = make_uint2((e & 0x3FFFFu) << 7, pack_bf16(own, ali));
    }
    __syncthreads();
    const int it = it0 + blockIdx.y;
    const uint64_t gstride = (uint64_t)(((M + 3) & ~3LL) >> 2);
    const int kp = threadIdx.x & 31, igq = threadIdx.x >> 5;
    // rows 4 igq + t of the first 32-row slab; slab q adds 32 rows (4096 bytes)
    // and leaves the swizzle (row & 7) unchanged
    uint32_t off[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
        const int r = 4 * igq + t;
        off[t] = (uint32_t)(r * ROW_BYTES + ((((kp >> 2) ^ (r & 7))) << 4) + ((kp & 3) << 2));
    }
    // block counter of (row group igq, K column 2 kp) in stage 0
    const uint64_t g0 = (uint64_t)it * (BM / 4) + (uint64_t)igq + (uint64_t)(2 * kp) * gstride;
    for (int s = blockIdx.x; s < Ks; s += gridDim.x) {
        uint8_t* tile = S + ((size_t)it * Ks + (size_t)s) * S_BYTES;
        const int64_t k0 = (int64_t)s * BK + 2 * kp;
        const uint64_t gs = g0 + (uint64_t)s * BK * gstride;
        // all four slabs unrolled: eight independent Philox chains per thread
        // (4.47 ms at the full precision least-squares sketch against 4.68
        // one slab at a time)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t row0 = (int64_t)it * BM + 4 * (igq + 8 * q);
            uint32_t r0[4] = {0u, 0u, 0u, 0u}, r1[4] = {0u, 0u, 0u, 0u};
            if (row0 < M) {
                if (k0 < K) gauss_block_bf16(key, gs + 8 * q, qt, r0);
                if (k0 + 1 < K) gauss_block_bf16(key, gs + 8 * q + gstride, qt, r1);
            }
#pragma unroll
            for (int t = 0; t < 4; ++t)
                *(uint32_t*)(tile + 4096 * q + off[t]) = (row0 + t < M) ? __byte_perm(r0[t], r1[t], 0x5410) : 0u;
        }
    }
}

// Work unit u: C tile (it, jt) partial over K chunk kc, with jt fastest:
// the column tiles sharing an S tile are processed side by side.
struct Unit {
    int jt, it, kc, s_begin, nst;
};
__device__ __forceinline__ Unit unit_of(const Params& prm, int u) {
    Unit w;
    w.jt = prm.jt0 + u % prm.jt_count;
    const int rest = u / prm.jt_count;
    w.it = prm.it0 + rest % prm.it_count;
    w.kc = rest / prm.it_count;
    w.s_begin = w.kc * prm.stages_per_kc;
    w.nst = min(prm.Ks, w.s_begin + prm.stages_per_kc) - w.s_begin;
    return w;
}

template <int P, int BNT>
__global__ void __launch_bounds__(THREADS, 1) sketch_mma_kernel(const Params prm) {
    static_assert(P * BNT <= ACC_COLS && BNT % 16 == 0, "accumulator width");
    constexpr int STAGES = stages_for(P, BNT);
    constexpr int YDB = BNT * ROW_BYTES;                           // one digit tile
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sS = smem;                                           // STAGES x 16 KB
    uint8_t* sY = smem + STAGES * S_BYTES;                        // STAGES x P digit tiles
    uint64_t* bars = (uint64_t*)(sY + STAGES * P * YDB);
    uint64_t* full = bars;                                        // stage landed (tx)
    uint64_t* empty = bars + STAGES;                              // MMAs done with the stage
    uint64_t* accFull = bars + 2 * STAGES;                        // [2] window accumulated
    uint64_t* accEmpty = accFull + 2;                             // [2] window drained
    uint64_t* drain = accEmpty + 2;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    volatile int* err = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accFull[b], 1);
            mbar_init(&accEmpty[b], DRAIN_WARPS);
        }
        mbar_init(drain, 1);
        *err = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                         smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- loader: S tile + P digit tiles per stage ----------------
        if (lane == 0) {
            int g = 0;                    // stages issued
            bool ok = true;
            for (int u = blockIdx.x; u < prm.units && ok; u += gridDim.x) {
                const Unit w = unit_of(prm, u);
                const uint8_t* sk = prm.sk + ((size_t)w.it * prm.Ks + w.s_begin) * S_BYTES;
                const uint8_t* yd = (const uint8_t*)prm.ydig + ((size_t)w.jt * prm.Ks + w.s_begin) * (size_t)(prm.ypl * YDB);
                for (int i = 0; i < w.nst; ++i) {
                    const int slot = g % STAGES;
                    if (g >= STAGES && !mbar_wait(&empty[slot], (uint32_t)((g / STAGES) - 1) & 1u, err)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&full[slot], (uint32_t)(S_BYTES + P * YDB));
                    bulk_g2s(sS + slot * S_BYTES, sk + (size_t)i * S_BYTES, S_BYTES, &full[slot]);
#pragma unroll
                    for (int p = 0; p < P; ++p)
                        bulk_g2s(sY + (slot * P + p) * YDB, yd + ((size_t)i * prm.ypl + p) * YDB, YDB,
                                 &full[slot]);
                    ++g;
                }
            }
            // let every copy this warp issued land before the CTA can exit
            for (int i = (g > STAGES ? g - STAGES : 0); i < g; ++i) {
                const int sl = i % STAGES;
                const uint32_t ph = (uint32_t)(i / STAGES) & 1u;
                if (!mbar_try(&full[sl], ph)) {
                    const unsigned long long t0 = globaltimer_ns();
                    while (!mbar_try(&full[sl], ph))
                        if (globaltimer_ns() - t0 > WAIT_NS) break;
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            // the P digit tiles of a stage are contiguous rows of one K-major
            // operand, so one MMA of N = P * BNT covers every digit: the S tile
            // is read from shared memory once per K step, not P times
            constexpr uint32_t idesc = idesc_bf16(BM, P * BNT);
            int g = 0, slot = 0;          // stages consumed; ring slot
            uint32_t fph = 0;             // full-barrier parity of slot
            int win = 0;                  // windows started
            bool ok = true;
            for (int u = blockIdx.x; u < prm.units && ok; u += gridDim.x) {
                const Unit w = unit_of(prm, u);
                int in_win = 0;
                uint32_t acc = 0;
                for (int i = 0; i < w.nst; ++i) {
                    if (in_win == 0) {
                        const int b = win & 1;
                        acc = tmem + (uint32_t)(b * ACC_COLS);
                        if (win >= 2) {
                            if (!mbar_wait(&accEmpty[b], (uint32_t)((win >> 1) - 1) & 1u, err)) { ok = false; break; }
                            tc_after();
                        }
                    }
                    if (!mbar_wait(&full[slot], fph, err)) { ok = false; break; }
                    tc_after();
                    const uint32_t a0 = smem_u32(sS + slot * S_BYTES);
                    const uint32_t b0 = smem_u32(sY + slot * P * YDB);
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk)
                        mma_bf16(acc, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc,
                                 (in_win > 0 || kk > 0) ? 1u : 0u);
                    mma_commit(&empty[slot]);
                    if (++slot == STAGES) { slot = 0; fph ^= 1u; }
                    ++g;
                    if (++in_win == WIN || i == w.nst - 1) {
                        mma_commit(&accFull[win & 1]);
                        ++win;
                        in_win = 0;
                    }
                }
            }
            mma_commit(drain);
            const unsigned long long t0 = globaltimer_ns();
            while (!mbar_try(drain, 0))
                if (globaltimer_ns() - t0 > WAIT_NS) { *err = 1; break; }
        }
    } else {
        // ---------------- drain: TMEM lane quarter (warp & 3), all BNT columns ----------------
        const int q = warp & 3;
        const int row = 32 * q + lane;
        int win = 0;
        bool ok = true;
        for (int u = blockIdx.x; u < prm.units && ok; u += gridDim.x) {
            const Unit w = unit_of(prm, u);
            const int tile = w.it + prm.tiles_m * w.jt;
            long long v[BNT];
#pragma unroll
            for (int c = 0; c < BNT; ++c) v[c] = 0;
            const int nwin = (w.nst + WIN - 1) / WIN;
            for (int wi = 0; wi < nwin; ++wi, ++win) {
                const int b = win & 1;
                if (!mbar_wait(&accFull[b], (uint32_t)(win >> 1) & 1u, err)) { ok = false; break; }
                tc_after();
                const uint32_t base = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * ACC_COLS);
                // two digit planes per TMEM round trip (registers: v holds the
                // unit's int64 tile row)
#pragma unroll
                for (int c16 = 0; c16 < BNT; c16 += 16) {
#pragma unroll
                    for (int p0 = 0; p0 < P; p0 += 2) {
                        uint32_t r0[16], r1[16];
                        tmem_ld16(base + (uint32_t)(p0 * BNT + c16), r0);
                        if (p0 + 1 < P) tmem_ld16(base + (uint32_t)((p0 + 1) * BNT + c16), r1);
                        tmem_ld_wait();
#pragma unroll
                        for (int c = 0; c < 16; ++c) {
                            acc_digit(v[c16 + c], r0[c], 8 * (P - 1 - p0));
                            if (p0 + 1 < P) acc_digit(v[c16 + c], r1[c], 8 * (P - 2 - p0));
                        }
                    }
                }
                tc_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&accEmpty[b]);
            }
            if (!ok) break;
            long long* out = prm.partial + ((size_t)w.kc * prm.tiles_m * prm.tiles_n + tile) * (size_t)(BM * BNT);
#pragma unroll
            for (int c = 0; c < BNT; ++c) out[(size_t)c * BM + row] = v[c];
        }
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
    if (threadIdx.x == 0 && *err) atomicCAS(prm.status, 0u, (unsigned int)KSTATUS_MBAR_TIMEOUT);
}

// ---------------------------------------------------------------------------
// Digit planes of Y
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mant_exp(double y, uint64_t& M, int& e2) {
    const uint64_t b = (uint64_t)__double_as_longlong(y);
    const int e = (int)((b >> 52) & 0x7ff);
    M = b & 0xFFFFFFFFFFFFFull;
    if (e) { M |= 1ull << 52; e2 = e - 1075; }
    else e2 = -1074;
}
__device__ __forceinline__ void mant_exp(float y, uint64_t& M, int& e2) {
    const uint32_t b = __float_as_uint(y);
    const int e = (int)((b >> 23) & 0xff);
    M = b & 0x7FFFFFu;
    if (e) { M |= 1u << 23; e2 = e - 150; }
    else e2 = -149;
}

// E_j = max over the column of (e2 + bitlength(M)): |y| < 2^E_j.  Zero column -> -1074.
// Column N (when `extra` is given) is the double vector extra[0..K).
template <typename T>
__device__ __forceinline__ void load_elem(const T* __restrict__ Y, int64_t ldy, int64_t N,
                                          const double* __restrict__ extra, int64_t k, int64_t j,
                                          uint64_t& M, int& e2, bool& neg) {
    if (j < N) {
        const T y = Y[k + j * ldy];
        mant_exp(y, M, e2);
        neg = (sizeof(T) == 8) ? (__double_as_longlong((double)y) < 0) : ((__float_as_uint((float)y) >> 31) != 0);
    } else {
        const double y = extra[k];
        mant_exp(y, M, e2);
        neg = __double_as_longlong(y) < 0;
    }
}

// E[j] = -1074 (the exponent of an all-zero column) before colexp_kernel.
__global__ void exp_init_kernel(int* __restrict__ E, int64_t n) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        E[j] = -1074;
}

// Block (x, y): rows [x * rows_per_block, ...) of column j0 + y; the block
// maximum goes into E[j] with atomicMax (the maximum is order independent).
// The largest |y| is the largest bit pattern with the sign cleared (IEEE
// order), so the loop is a load, a mask and an unsigned max per element, with
// eight loads in flight per thread; the exponent is formed once per thread.
__device__ __forceinline__ int exp_of_bits(uint32_t b) {          // FP32 |y| bits -> E with |y| < 2^E
    const int e = (int)(b >> 23);
    return e ? e - 126 : -149 + (32 - __clz((int)(b & 0x7FFFFFu)));
}
__device__ __forceinline__ int exp_of_bits(uint64_t b) {          // FP64
    const int e = (int)(b >> 52);
    return e ? e - 1022 : -1074 + (64 - __clzll((long long)(b & 0xFFFFFFFFFFFFFull)));
}
__device__ __forceinline__ uint32_t abs_bits(float y) { return __float_as_uint(y) & 0x7FFFFFFFu; }
__device__ __forceinline__ uint64_t abs_bits(double y) {
    return (uint64_t)__double_as_longlong(y) & 0x7FFFFFFFFFFFFFFFull;
}

template <typename T>
__device__ __forceinline__ int column_max_exp(const T* __restrict__ col, int64_t k0, int64_t k1) {
    using U = decltype(abs_bits(T(0)));
    U best = 0;
    constexpr int Q = 8;
    int64_t k = k0 + threadIdx.x;
    for (; k + (Q - 1) * (int64_t)blockDim.x < k1; k += Q * (int64_t)blockDim.x) {
        T v[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) v[q] = col[k + q * (int64_t)blockDim.x];
#pragma unroll
        for (int q = 0; q < Q; ++q) best = max(best, abs_bits(v[q]));
    }
    for (; k < k1; k += blockDim.x) best = max(best, abs_bits(col[k]));
    return best ? exp_of_bits(best) : -1074;
}

template <typename T>
__global__ void colexp_kernel(const T* __restrict__ Y, int64_t K, int64_t N, int64_t ldy,
                              const double* __restrict__ extra, int* __restrict__ E, int64_t j0,
                              int64_t rows_per_block) {
    const int64_t j = j0 + blockIdx.y;
    const int64_t k0 = (int64_t)blockIdx.x * rows_per_block;
    const int64_t k1 = min(K, k0 + rows_per_block);
    int best = (j < N) ? column_max_exp(Y + j * ldy, k0, k1) : column_max_exp(extra, k0, k1);
    __shared__ int red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x < 32) {
        best = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : -1074;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
        if (threadIdx.x == 0 && best > -1074) atomicMax(&E[j], best);
    }
}

__device__ __forceinline__ uint16_t digit_bf16(uint32_t d, bool neg) {
    // d <= 256: the float of d has at most 8 significant bits, so its top 16 bits are the bf16
    const float f = (float)d;
    return (uint16_t)((__float_as_uint(f) >> 16) | (neg && d ? 0x8000u : 0u));
}

// One thread per (column j, 8 consecutive k): reads 8 values, writes P 16-byte
// chunks into the SW128 images [jt][stage][p][BN][64].  Ntot = N (+1 with extra).
// The P bf16 digits of the 8 values k = s BK + 8 c8 .. + 7 of column j
// (zeros beyond K or Ntot) and, for the row-major copy, the 8 FP32 values of
// A's columns (zero for the appended column and beyond N).
template <typename T, int P>
__device__ __forceinline__ void slice_unit(const T* __restrict__ Y, int64_t K, int64_t N, int64_t ldy,
                                           const double* __restrict__ extra, int64_t Ntot,
                                           const int* __restrict__ E, int64_t j, int s, int c8,
                                           uint16_t dg[P][8], float xs[8]) {
    const int Ej = (j < Ntot) ? E[j] : 0;
    const int ksc = 8 - Ej;                      // x 2^(8 - E_j) lies in (-256, 256)
#pragma unroll
    for (int t = 0; t < 8; ++t) xs[t] = 0.f;
    if (sizeof(T) == 4 && j < N && ksc >= -126 && ksc <= 127) {
        // FP32 data in FP32 arithmetic: scaling by a power of two is exact,
        // each digit is the nearest integer of what the earlier ones leave
        // (|d| <= 256, balanced), times 256 for the next -- a handful of
        // FP32 operations per element instead of 64-bit integer work.  The
        // bf16 of an integer of at most 9 bits is its float's top half.
        const float scale = __int_as_float((127 + ksc) << 23);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int64_t k = (int64_t)s * BK + c8 * 8 + t;
            xs[t] = k < K ? (float)Y[k + j * ldy] : 0.f;
            float x = xs[t] * scale;
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const float d = rintf(x);
                dg[p][t] = (uint16_t)(__float_as_uint(d) >> 16);
                x = (x - d) * 256.f;
            }
        }
    } else {
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int64_t k = (int64_t)s * BK + c8 * 8 + t;
            uint64_t M = 0;
            int e2 = 0;
            bool neg = false;
            if (j < Ntot && k < K) {
                load_elem(Y, ldy, N, extra, k, j, M, e2, neg);
                if (sizeof(T) == 4 && j < N) xs[t] = (float)Y[k + j * ldy];
            }
            uint64_t Tq = 0;
            if (M) {
                const int sh = Ej - 8 * P - e2;
                if (sh <= 0) Tq = M << (-sh);
                else if (sh < 64) Tq = (M + (1ull << (sh - 1))) >> sh;
            }
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const uint32_t d = (p == 0) ? (uint32_t)(Tq >> (8 * (P - 1)))
                                            : (uint32_t)((Tq >> (8 * (P - 1 - p))) & 255u);
                dg[p][t] = digit_bf16(d, neg);
            }
        }
    }
}

// The unit's digits into row jl of the P digit tile images (BNT rows each)
// of (jt, s).
template <int P, int BNT>
__device__ __forceinline__ void store_digits(uint16_t* __restrict__ out, int Ks, int jt, int s, int jl, int c8,
                                             const uint16_t dg[P][8]) {
    const size_t blk = ((size_t)jt * Ks + s) * P;
#pragma unroll
    for (int p = 0; p < P; ++p) {
        uint4 v;
        v.x = dg[p][0] | ((uint32_t)dg[p][1] << 16);
        v.y = dg[p][2] | ((uint32_t)dg[p][3] << 16);
        v.z = dg[p][4] | ((uint32_t)dg[p][5] << 16);
        v.w = dg[p][6] | ((uint32_t)dg[p][7] << 16);
        uint8_t* base = (uint8_t*)out + (blk + p) * (size_t)(BNT * ROW_BYTES);
        *(uint4*)(base + jl * ROW_BYTES + ((c8 ^ (jl & 7)) << 4)) = v;
    }
}

// Digit planes of column tiles [jt0, jt0 + jt_count) of width BNT: a thread
// per (column j, 8 consecutive k); consecutive threads take consecutive k of
// one column.
template <typename T, int P, int BNT>
__global__ void slice_kernel(const T* __restrict__ Y, int64_t K, int64_t N, int64_t ldy,
                             const double* __restrict__ extra, int64_t Ntot, const int* __restrict__ E,
                             int Ks, int jt0, int jt_count, uint16_t* __restrict__ out) {
    const int64_t chunks_per_col = (int64_t)Ks * 8;
    const int64_t total = chunks_per_col * (int64_t)jt_count * BNT;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < total;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = (int64_t)jt0 * BNT + u / chunks_per_col;
        const int64_t cc = u % chunks_per_col;
        const int s = (int)(cc >> 3), c8 = (int)(cc & 7);
        uint16_t dg[P][8];
        float xs[8];
        slice_unit<T, P>(Y, K, N, ldy, extra, Ntot, E, j, s, c8, dg, xs);
        store_digits<P, BNT>(out, Ks, (int)(j / BNT), s, (int)(j % BNT), c8, dg);
    }
}

// The same digit planes for FP32 data together with the solver's row-major
// FP32 copy of A (rows of ldq floats, zero from column N on), so that A is
// read once for both: a block per (column tile, stage) tile of 64 x BNT
// values (tiles column-tile fastest), the BNT x 8 (column, 8 k) units spread
// over the threads, the values transposed through shared memory and written
// as row segments of BNT floats.
template <int P, int BNT>
__global__ void __launch_bounds__(256) slice_rowmajor_kernel(const float* __restrict__ Y, int64_t K, int64_t N,
                                                             int64_t ldy, const double* __restrict__ extra,
                                                             int64_t Ntot, const int* __restrict__ E, int Ks,
                                                             int jt0, int jt_count, uint16_t* __restrict__ out,
                                                             float* __restrict__ AQ, int64_t ldq) {
    // SPI stages per iteration, so that the iteration's (column, 8 k) units
    // are a whole number per thread (two stages of 80 columns: 1280 units,
    // five each)
    constexpr int SPI = (BNT * 8) % 256 == 0 ? 1 : 2;
    constexpr int UNITS = SPI * BNT * 8;
    static_assert(BK == 64 && UNITS % 256 == 0 && (SPI * BK * BNT) % 256 == 0, "tile shape");
    __shared__ float tile[SPI * BK][BNT + 1];
    const int tid = threadIdx.x;
    const int pairs = (Ks + SPI - 1) / SPI;
    const int64_t tiles = (int64_t)jt_count * pairs;
    for (int64_t u = blockIdx.x; u < tiles; u += gridDim.x) {
        const int jt = jt0 + (int)(u % jt_count);
        const int s0 = (int)(u / jt_count) * SPI;
#pragma unroll
        for (int h = 0; h < UNITS / 256; ++h) {
            const int v = tid + 256 * h;
            const int ss = v / (BNT * 8), w = v % (BNT * 8);
            const int c8 = w & 7, jl = w >> 3;
            const int s = s0 + ss;
            float xs[8];
            if (s < Ks) {
                const int64_t j = (int64_t)jt * BNT + jl;
                uint16_t dg[P][8];
                slice_unit<float, P>(Y, K, N, ldy, extra, Ntot, E, j, s, c8, dg, xs);
                store_digits<P, BNT>(out, Ks, jt, s, jl, c8, dg);
            } else {
#pragma unroll
                for (int t = 0; t < 8; ++t) xs[t] = 0.f;
            }
#pragma unroll
            for (int t = 0; t < 8; ++t) tile[ss * BK + c8 * 8 + t][jl] = xs[t];
        }
        __syncthreads();
        const int64_t k0 = (int64_t)s0 * BK, j0 = (int64_t)jt * BNT;
#pragma unroll 4
        for (int q = 0; q < SPI * BK * BNT / 256; ++q) {
            const int idx = q * 256 + tid;
            const int kk = idx / BNT, jj = idx % BNT;
            if (k0 + kk < K && j0 + jj < ldq) AQ[(k0 + kk) * ldq + j0 + jj] = tile[kk][jj];
        }
        __syncthreads();
    }
}

// C[i, j] = 2^(E_j - shift) * sum over kc of partial[kc][tile][col][row].
// The chunk sums are exact integers; they are added in int64 when the
// caller guarantees no overflow (exact_sum), else in FP64, in a fixed order.
__global__ void splitk_sum_kernel(const long long* __restrict__ part, int kc_count, int tiles_m, int tiles_n, int bn,
                                  int64_t M, int64_t N, const int* __restrict__ colexp, int shift, int exact_sum,
                                  double* __restrict__ C, int64_t ldc) {
    const int64_t total = M * N;
    const size_t tile_elems = (size_t)BM * bn;
    const size_t kc_stride = (size_t)tiles_m * tiles_n * tile_elems;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % M, j = e / M;
        const int it = (int)(i / BM), jt = (int)(j / bn);
        const size_t off = (size_t)(it + (int64_t)tiles_m * jt) * tile_elems + (size_t)(j % bn) * BM + (i % BM);
        double s;
        if (exact_sum) {
            long long t = 0;
            for (int k = 0; k < kc_count; ++k) t += part[k * kc_stride + off];
            s = (double)t;
        } else {
            s = 0.0;
            for (int k = 0; k < kc_count; ++k) s += (double)part[k * kc_stride + off];
        }
        C[i + j * ldc] = ldexp(s, colexp[j] - shift);
    }
}

template <int P, int BNT>
static size_t smem_bytes() {
    constexpr int STAGES = stages_for(P, BNT);
    return 1024 + (size_t)STAGES * S_BYTES + (size_t)STAGES * P * (BNT * ROW_BYTES) + 512;
}

template <int P>
static void run(Ctx& ctx, const RngKey& key, int dist, const void* Y, bool y_f32, int64_t K, int64_t N0,
                int64_t ldy, const double* extra, int64_t M, double* C, int64_t ldc, const ColumnFeed* feed,
                const std::function<void(cudaStream_t)>& before_mma, const SketchRowMajor& rm) {
    constexpr int BNR = bn_for(P);               // column tile width of this launch
    const int64_t N = N0 + (extra ? 1 : 0);      // the extra column is appended as column N0
    const int tiles_m = div_up(M, BM), tiles_n = div_up(N, BNR);
    const size_t smem = smem_bytes<P, BNR>();
    const int Ks = div_up(K, BK);
    const int wins = div_up(Ks, WIN);
    // choose the K split for the persistent walk: about
    //   rounds x stages per unit x (time of one stage)  +  units x (int64 tile
    //   store and reload, 128 KB of HBM traffic)
    // with rounds = ceil(units / SMs); a unit sums at most WIN_MAX windows in
    // int64 (|window value| < 2^48.01, so WIN_MAX windows stay below 2^63)
    constexpr int WIN_MAX = 32000;
    const int sm = ctx.sm_count;
    const int64_t tiles = (int64_t)tiles_m * tiles_n;
    // With a feed (A still arriving from the host) the MMA runs per group of
    // column tiles as their columns land, so it overlaps the rest of the
    // upload; every group re-reads S (from L2 when S is small), so a small S
    // goes tile by tile and a large one in four groups.
    const double s_bytes = (double)tiles_m * Ks * S_BYTES;
    const int groups = !feed ? 1 : (s_bytes * tiles_n <= 4.0e9 ? tiles_n : std::min(tiles_n, 4));
    const int per_group = div_up(tiles_n, groups);
    const int64_t tiles_launch = (int64_t)tiles_m * per_group;
    const double t_stage = 0.09 * P;                 // us per stage per SM (tensor bound)
    const double t_unit = 0.02;                      // us of partial traffic per unit
    int best_kc = div_up(wins, WIN_MAX);
    double best_cost = 1e300;
    for (int kcn = div_up(wins, WIN_MAX); kcn <= Ks && kcn <= 64; ++kcn) {
        const int spk_n = div_up(Ks, kcn);
        const int kc_eff = div_up(Ks, spk_n);
        const int64_t units = tiles_launch * kc_eff;
        const int64_t rounds = (units + sm - 1) / sm;
        const double cost = (double)rounds * spk_n * t_stage + (double)units * t_unit;
        if (cost < best_cost - 1e-9) { best_cost = cost; best_kc = kc_eff; }
    }
    const int spk = div_up(Ks, best_kc);
    const int kc_count = div_up(Ks, spk);
    const int64_t units = tiles_launch * kc_count;

    DevBuf<int> E((size_t)tiles_n * BNR, ctx.stream);
    exp_init_kernel<<<(unsigned)div_up((int64_t)tiles_n * BNR, 256), 256, 0, ctx.stream>>>(E, (int64_t)tiles_n * BNR);
    RNLA_LAUNCH_CHECK();
    DevBuf<uint16_t> dig((size_t)tiles_n * Ks * P * BNR * (ROW_BYTES / 2), ctx.stream);
    DevBuf<uint8_t> sk((size_t)tiles_m * Ks * S_BYTES, ctx.stream);
    DevBuf<long long> part((size_t)kc_count * tiles * BM * BNR, ctx.stream);
    // the sketch generator (integer ALU bound) runs on the side stream while
    // the main stream makes the digit planes (HBM bound)
    const cudaStream_t side = (ctx.side ? ctx.side : side_stream(ctx.device));
    stream_wait(side, ctx.stream);                 // the S buffer exists
    cudaEvent_t s_done;
    RNLA_CUDA(cudaEventCreateWithFlags(&s_done, cudaEventDisableTiming));
    {
        // about four resident blocks per SM in all: the generator is
        // integer-pipe bound, and the main stream's HBM-bound digit planes
        // need the remaining SM slots
        const int cap = std::max(1, 4 * sm / tiles_m);
        if (dist == DIST_GAUSSIAN && key.gen == GEN_PHILOX4X32) {
            const int gx = std::min(Ks, cap);
            sketch_gen_gauss_kernel<<<dim3((unsigned)gx, (unsigned)tiles_m), 256, 0, side>>>(key, M, K, Ks, 0, sk);
        } else {
            int gx = div_up((int64_t)Ks * 1024, 256);
            if (gx > cap) gx = cap;
            sketch_gen_kernel<<<dim3((unsigned)gx, (unsigned)tiles_m), 256, 0, side>>>(key, dist, M, K, Ks, 0, sk);
        }
        RNLA_LAUNCH_CHECK();
        RNLA_CUDA(cudaEventRecord(s_done, side));
    }
    Params prm;
    prm.M = M; prm.N = N; prm.K = K;
    prm.tiles_m = tiles_m; prm.tiles_n = tiles_n; prm.Ks = Ks;
    prm.it0 = 0; prm.it_count = tiles_m;
    prm.jt0 = 0; prm.jt_count = tiles_n;
    prm.kc_count = kc_count; prm.stages_per_kc = spk; prm.units = (int)units;
    prm.sk = sk; prm.ydig = dig; prm.ypl = P; prm.partial = part; prm.status = ctx.status;
    ctx.clear_status();
    auto kfn = sketch_mma_kernel<P, BNR>;
    set_smem_limit((const void*)kfn, smem);
    const unsigned grid = (unsigned)(units < sm ? units : sm);
    // exponents and digit planes of column tiles [jt0, jt0 + cnt)
    auto digits = [&](int jt0, int cnt) {
        const int64_t j0 = (int64_t)jt0 * BNR;
        const int64_t j1 = std::min((int64_t)N, (int64_t)(jt0 + cnt) * BNR);
        // about 16 values per thread: K / 4096 blocks per column
        const int64_t rpb = 4096;
        const dim3 cg((unsigned)div_up(K, rpb), (unsigned)(j1 - j0));
        if (y_f32)
            colexp_kernel<float><<<cg, 256, 0, ctx.stream>>>((const float*)Y, K, N0, ldy, extra, E, j0, rpb);
        else
            colexp_kernel<double><<<cg, 256, 0, ctx.stream>>>((const double*)Y, K, N0, ldy, extra, E, j0, rpb);
        RNLA_LAUNCH_CHECK();
        const int64_t su = (int64_t)Ks * 8 * cnt * BNR;
        int g = div_up(su, 256);
        if (g > 32 * sm) g = 32 * sm;
        if (y_f32 && rm.dst) {
            // every block resident at once (a grid of whole waves)
            static const int occ = [] {
                int o = 0;
                RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, slice_rowmajor_kernel<P, bn_for(P)>, 256, 0));
                return o;
            }();
            const int64_t tl = (int64_t)cnt * div_up(Ks, (BNR * 8) % 256 == 0 ? 1 : 2);
            const int gr = (int)std::min<int64_t>(tl, (int64_t)std::max(occ, 1) * sm);
            slice_rowmajor_kernel<P, BNR><<<gr, 256, 0, ctx.stream>>>((const float*)Y, K, N0, ldy, extra, N, E, Ks, jt0, cnt,
                                                                 dig, rm.dst, rm.ld);
        } else if (y_f32)
            slice_kernel<float, P, BNR><<<g, 256, 0, ctx.stream>>>((const float*)Y, K, N0, ldy, extra, N, E, Ks, jt0, cnt, dig);
        else
            slice_kernel<double, P, BNR><<<g, 256, 0, ctx.stream>>>((const double*)Y, K, N0, ldy, extra, N, E, Ks, jt0, cnt, dig);
        RNLA_LAUNCH_CHECK();
    };
    if (!feed) {
        digits(0, tiles_n);
        // the caller's main-stream work that needs only the inputs (the
        // solver's row-major copy) goes before the MMA: beside the MMA, its
        // HBM traffic slows the L2-bound MMA by more than it saves
        if (before_mma) before_mma(ctx.stream);
        RNLA_CUDA(cudaStreamWaitEvent(ctx.stream, s_done, 0));     // S is written
        kfn<<<grid, THREADS, smem, ctx.stream>>>(prm);
        RNLA_LAUNCH_CHECK();
    } else {
        // each column tile's digit planes as soon as its columns have
        // landed, each group's MMA once the group's last tile is in
        for (int g0 = 0; g0 < tiles_n; g0 += per_group) {
            const int cnt = std::min(per_group, tiles_n - g0);
            for (int jt = g0; jt < g0 + cnt; ++jt) {
                feed->wait_cols(ctx.stream, (int64_t)jt * BNR, std::min(N0, (int64_t)(jt + 1) * BNR));
                digits(jt, 1);
            }
            if (g0 == 0) RNLA_CUDA(cudaStreamWaitEvent(ctx.stream, s_done, 0));   // S is written
            prm.jt0 = g0;
            prm.jt_count = cnt;
            prm.units = (int)((int64_t)cnt * tiles_m * kc_count);
            const unsigned gp = (unsigned)(prm.units < sm ? prm.units : sm);
            kfn<<<gp, THREADS, smem, ctx.stream>>>(prm);
            RNLA_LAUNCH_CHECK();
        }
    }
    int g = div_up(M * N, 256);
    if (g > 8 * sm) g = 8 * sm;
    const int exact_sum = (int64_t)wins + kc_count <= WIN_MAX ? 1 : 0;   // all windows together fit int64
    splitk_sum_kernel<<<g, 256, 0, ctx.stream>>>(part, kc_count, tiles_m, tiles_n, BNR, M, N, E, 8 * P + quant_shift(dist),
                                                 exact_sum, C, ldc);
    RNLA_LAUNCH_CHECK();
    RNLA_CUDA(cudaEventDestroy(s_done));
    ctx.check_status("tensor-core sketch");
}

// ---------------------------------------------------------------------------
// Exact X^T Y for two data operands on the same MMA kernel: X's columns cut
// into signed 6-bit digits below each column's exponent play the sketch
// (integers |t| <= 64, exact in bf16), Y's columns the 8-bit digit planes.
// ---------------------------------------------------------------------------

// One thread per (column j of X, 8 consecutive k): the ND digits (most
// significant first) of T = round(|x| 2^(6 ND - E_j)) as sketch-tile image
// rows j % 128 of tiles [digit][j / 128][stage] (X is read once).
template <typename T>
__global__ void sdigit_kernel(const T* __restrict__ X, int64_t K, int64_t N, int64_t ldx, const int* __restrict__ E,
                              int ND, int Ks, int tiles, uint8_t* __restrict__ out) {
    const size_t digit_stride = (size_t)tiles * Ks * S_BYTES;
    const int64_t chunks_per_col = (int64_t)Ks * 8;
    const int64_t total = chunks_per_col * (int64_t)tiles * BM;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = u / chunks_per_col;
        const int64_t cc = u % chunks_per_col;
        const int st = (int)(cc >> 3), c8 = (int)(cc & 7);
        const int it = (int)(j / BM), r = (int)(j % BM);
        const int Ej = (j < N) ? E[j] : 0;
        uint8_t* tile = out + ((size_t)it * Ks + st) * S_BYTES + r * ROW_BYTES + ((c8 ^ (r & 7)) << 4);
        const int ksc = 6 - Ej;                      // x 2^(6 - E_j) lies in (-64, 64)
        if (sizeof(T) == 4 && j < N && ksc >= -126 && ksc <= 127) {
            // FP32 data in FP32 arithmetic (as slice_kernel): balanced digits
            // |d| <= 64, the bf16 of each the top half of its float
            const float scale = __int_as_float((127 + ksc) << 23);
            float x[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int64_t k = (int64_t)st * BK + c8 * 8 + t;
                x[t] = k < K ? (float)X[k + j * ldx] * scale : 0.f;
            }
            for (int dig = 0; dig < ND; ++dig) {
                uint32_t h[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const float d = rintf(x[t]);
                    h[t] = __float_as_uint(d) >> 16;
                    x[t] = (x[t] - d) * 64.f;
                }
                uint4 v;
                v.x = h[0] | (h[1] << 16);
                v.y = h[2] | (h[3] << 16);
                v.z = h[4] | (h[5] << 16);
                v.w = h[6] | (h[7] << 16);
                *(uint4*)(tile + (size_t)dig * digit_stride) = v;
            }
            continue;
        }
        uint64_t Tq[8];
        bool neg[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int64_t k = (int64_t)st * BK + c8 * 8 + t;
            uint64_t M = 0;
            int e2 = 0;
            neg[t] = false;
            if (j < N && k < K) {
                const T x = X[k + j * ldx];
                mant_exp(x, M, e2);
                neg[t] = (sizeof(T) == 8) ? (__double_as_longlong((double)x) < 0)
                                          : ((__float_as_uint((float)x) >> 31) != 0);
            }
            Tq[t] = 0;
            if (M) {
                const int sh = Ej - 6 * ND - e2;
                if (sh <= 0) Tq[t] = M << (-sh);
                else if (sh < 64) Tq[t] = (M + (1ull << (sh - 1))) >> sh;
            }
        }
        for (int dig = 0; dig < ND; ++dig) {
            uint16_t dg[8];
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const uint32_t d = (dig == 0) ? (uint32_t)(Tq[t] >> (6 * (ND - 1)))
                                              : (uint32_t)((Tq[t] >> (6 * (ND - 1 - dig))) & 63u);
                dg[t] = digit_bf16(d, neg[t]);
            }
            uint4 v;
            v.x = dg[0] | ((uint32_t)dg[1] << 16);
            v.y = dg[2] | ((uint32_t)dg[3] << 16);
            v.z = dg[4] | ((uint32_t)dg[5] << 16);
            v.w = dg[6] | ((uint32_t)dg[7] << 16);
            *(uint4*)(tile + (size_t)dig * digit_stride) = v;
        }
    }
}

// C (+)= 2^(Ex_r + Ey_c - shift) * sum over kc of the partials (row r of the
// product = column r of X, column c = column c of Y); C^T when trans.
__global__ void exact_tn_sum_kernel(const long long* __restrict__ part, int kc_count, int tiles_m, int tiles_n,
                                    int64_t M, int64_t N, const int* __restrict__ Ex, const int* __restrict__ Ey,
                                    int shift, int exact_sum, int accumulate, int trans, double* __restrict__ C,
                                    int64_t ldc) {
    const size_t tile_elems = (size_t)BM * BN;
    const size_t kc_stride = (size_t)tiles_m * tiles_n * tile_elems;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M * N; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % M, j = e / M;
        const size_t off = (size_t)((i / BM) + (int64_t)tiles_m * (j / BN)) * tile_elems + (size_t)(j % BN) * BM + (i % BM);
        double sum;
        if (exact_sum) {
            long long t = 0;
            for (int k = 0; k < kc_count; ++k) t += part[k * kc_stride + off];
            sum = (double)t;
        } else {
            sum = 0.0;
            for (int k = 0; k < kc_count; ++k) sum += (double)part[k * kc_stride + off];
        }
        const double v = ldexp(sum, Ex[i] + Ey[j] - shift);
        double* dst = trans ? &C[j + i * ldc] : &C[i + j * ldc];
        *dst = accumulate ? *dst + v : v;
    }
}

}  // namespace tc

// C (MM x NN, FP64) = X^T Y, X (K x MM, FP32 or FP64) and Y (K x NN, FP64)
// column-major, with exact tensor-core products: Y is cut into 4 planes of
// 8-bit digits below each column's maximum (32 bits), X into xd digits of 6
// bits (24 bits for xd = 4: FP32 data to their own precision below each
// column's maximum); each X digit is one launch of the sketch MMA kernel
// whose 1024-K windows are exact in FP32 and folded into int64, so the only
// roundings are the two digit truncations and the final FP64 sums over the
// xd launches.  All X digit images are built in one pass over X
// (xd x tiles_m x Ks x 16 KB).
template <int P>
static void launch_mma(Ctx& ctx, const tc::Params& prm, unsigned grid) {
    using namespace tc;
    const size_t smem = smem_bytes<P, BN>();
    auto kfn = sketch_mma_kernel<P, BN>;
    set_smem_limit((const void*)kfn, smem);
    kfn<<<grid, THREADS, smem, ctx.stream>>>(prm);
    RNLA_LAUNCH_CHECK();
}

void tc_exact_tn(Ctx& ctx, const void* X, bool x_f32, int64_t K, int64_t MM, int64_t ldx, const double* Y,
                 int64_t NN, int64_t ldy, double* C, int64_t ldc, bool trans, int xd) {
    using namespace tc;
    constexpr int P = 4;
    if (K <= 0 || MM <= 0 || NN <= 0) return;
    if (xd < 1 || xd > 5) fail(RNLA_ERR_INVALID_PARAMETERS, "exact X^T Y: 1..5 digits of X");
    const int tiles_m = div_up(MM, BM), tiles_n = div_up(NN, BN);
    const int Ks = div_up(K, BK);
    const int wins = div_up(Ks, WIN);
    const int sm = ctx.sm_count;
    const int64_t tiles = (int64_t)tiles_m * tiles_n;
    constexpr int WIN_MAX = 32000;
    int best_kc = div_up(wins, WIN_MAX);
    double best_cost = 1e300;
    for (int kcn = div_up(wins, WIN_MAX); kcn <= Ks && kcn <= 64; ++kcn) {
        const int spk_n = div_up(Ks, kcn);
        const int kc_eff = div_up(Ks, spk_n);
        const int64_t units = tiles * kc_eff;
        const int64_t rounds = (units + sm - 1) / sm;
        const double cost = (double)rounds * spk_n * (0.09 * P) + (double)units * 0.02;
        if (cost < best_cost - 1e-9) { best_cost = cost; best_kc = kc_eff; }
    }
    const int spk = div_up(Ks, best_kc);
    const int kc_count = div_up(Ks, spk);
    const int64_t units = tiles * kc_count;
    DevBuf<int> Ex((size_t)tiles_m * BM, ctx.stream), Ey((size_t)tiles_n * BN, ctx.stream);
    exp_init_kernel<<<(unsigned)div_up((int64_t)tiles_m * BM, 256), 256, 0, ctx.stream>>>(Ex, (int64_t)tiles_m * BM);
    RNLA_LAUNCH_CHECK();
    exp_init_kernel<<<(unsigned)div_up((int64_t)tiles_n * BN, 256), 256, 0, ctx.stream>>>(Ey, (int64_t)tiles_n * BN);
    RNLA_LAUNCH_CHECK();
    const int64_t rpb = 4096;
    if (x_f32)
        colexp_kernel<float><<<dim3((unsigned)div_up(K, rpb), (unsigned)MM), 256, 0, ctx.stream>>>(
            static_cast<const float*>(X), K, MM, ldx, nullptr, Ex, 0, rpb);
    else
        colexp_kernel<double><<<dim3((unsigned)div_up(K, rpb), (unsigned)MM), 256, 0, ctx.stream>>>(
            static_cast<const double*>(X), K, MM, ldx, nullptr, Ex, 0, rpb);
    RNLA_LAUNCH_CHECK();
    colexp_kernel<double><<<dim3((unsigned)div_up(K, rpb), (unsigned)NN), 256, 0, ctx.stream>>>(Y, K, NN, ldy, nullptr,
                                                                                              Ey, 0, rpb);
    RNLA_LAUNCH_CHECK();
    DevBuf<uint16_t> dig((size_t)tiles_n * Ks * P * (YD_BYTES / 2), ctx.stream);
    {
        const int64_t su = (int64_t)Ks * 8 * tiles_n * BN;
        int g = div_up(su, 256);
        if (g > 32 * sm) g = 32 * sm;
        slice_kernel<double, P, BN><<<g, 256, 0, ctx.stream>>>(Y, K, NN, ldy, nullptr, NN, Ey, Ks, 0, tiles_n, dig);
        RNLA_LAUNCH_CHECK();
    }
    const size_t digit_bytes = (size_t)tiles_m * Ks * S_BYTES;
    DevBuf<uint8_t> sk(digit_bytes * xd, ctx.stream);
    {
        const int64_t su = (int64_t)Ks * 8 * tiles_m * BM;
        int g = div_up(su, 256);
        if (g > 32 * sm) g = 32 * sm;
        if (x_f32)
            sdigit_kernel<float><<<g, 256, 0, ctx.stream>>>(static_cast<const float*>(X), K, MM, ldx, Ex, xd, Ks, tiles_m,
                                                            sk);
        else
            sdigit_kernel<double><<<g, 256, 0, ctx.stream>>>(static_cast<const double*>(X), K, MM, ldx, Ex, xd, Ks,
                                                             tiles_m, sk);
        RNLA_LAUNCH_CHECK();
    }
    DevBuf<long long> part((size_t)kc_count * tiles * BM * BN, ctx.stream);
    Params prm;
    prm.M = MM; prm.N = NN; prm.K = K;
    prm.tiles_m = tiles_m; prm.tiles_n = tiles_n; prm.Ks = Ks;
    prm.kc_count = kc_count; prm.stages_per_kc = spk; prm.units = (int)units;
    prm.jt0 = 0; prm.jt_count = tiles_n;
    prm.it0 = 0; prm.it_count = tiles_m;
    prm.sk = sk; prm.ydig = dig; prm.ypl = P; prm.partial = part; prm.status = ctx.status;
    ctx.clear_status();
    const unsigned grid = (unsigned)(units < sm ? units : sm);
    const int exact_sum = (int64_t)wins + kc_count <= WIN_MAX ? 1 : 0;
    int gs = div_up(MM * NN, 256);
    if (gs > 8 * sm) gs = 8 * sm;
    for (int d = 0; d < xd; ++d) {
        // digit pair (d, p) weighs 2^-(6 d + 8 p) against the leading pair; X's
        // truncation after xd digits is 2^-6 xd, so pairs below 2^-(6 xd + 4)
        // are left out: the first Pd planes of Y for X digit d
        const int Pd = std::min(P, (6 * xd + 4 - 6 * d) / 8 + 1);
        prm.sk = sk.get() + (size_t)d * digit_bytes;
        switch (Pd) {
            case 1: launch_mma<1>(ctx, prm, grid); break;
            case 2: launch_mma<2>(ctx, prm, grid); break;
            case 3: launch_mma<3>(ctx, prm, grid); break;
            default: launch_mma<4>(ctx, prm, grid); break;
        }
        exact_tn_sum_kernel<<<gs, 256, 0, ctx.stream>>>(part, kc_count, tiles_m, tiles_n, MM, NN, Ex, Ey,
                                                        8 * Pd + 6 * (d + 1), exact_sum, d > 0 ? 1 : 0, trans ? 1 : 0,
                                                        C, ldc);
        RNLA_LAUNCH_CHECK();
    }
    ctx.check_status("exact tensor-core X^T Y");
}

bool tc_available(Ctx& ctx) {
    int major = 0, minor = 0;
    RNLA_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx.device));
    RNLA_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, ctx.device));
    return major == 10 && minor == 3;
}

void tc_sketch_apply(Ctx& ctx, const RngKey& key, const void* X, bool x_f32, int64_t K, int64_t N,
                     int64_t ldx, const double* extra, int64_t M, int digits, double* C, int64_t ldc,
                     const ColumnFeed* feed, int dist, const std::function<void(cudaStream_t)>& before_mma,
                     const SketchRowMajor& rm) {
    if (K <= 0 || (N <= 0 && !extra) || M <= 0) return;
    // default digits: 4 for FP64 data (32 bits below each column's maximum),
    // 3 for FP32 data (its 24-bit significands)
    if (digits <= 0) digits = x_f32 ? 3 : 4;
    switch (digits) {
        case 1: tc::run<1>(ctx, key, dist, X, x_f32, K, N, ldx, extra, M, C, ldc, feed, before_mma, rm); break;
        case 2: tc::run<2>(ctx, key, dist, X, x_f32, K, N, ldx, extra, M, C, ldc, feed, before_mma, rm); break;
        case 3: tc::run<3>(ctx, key, dist, X, x_f32, K, N, ldx, extra, M, C, ldc, feed, before_mma, rm); break;
        case 4: tc::run<4>(ctx, key, dist, X, x_f32, K, N, ldx, extra, M, C, ldc, feed, before_mma, rm); break;
        default: fail(RNLA_ERR_INVALID_PARAMETERS, "digits must be 1..4");
    }
}

// C = X^T Y on the tensor cores: the level is the larger digit count
// requested -- 1..3 on the split-bf16 GEMM (gemm_bfx.cu; 1 = plain bf16,
// default 3, which holds FP32 data exactly), 4 or more on the exact integer
// digit products (tc_exact_tn).
void tc_gemm_tn(Ctx& ctx, const double* X, int64_t K, int64_t MM, int64_t ldx, const double* Y, int64_t NN,
                int64_t ldy, int dx, int dy, double* C, int64_t ldc) {
    if (K <= 0 || MM <= 0 || NN <= 0) return;
    int level = std::max(dx, dy);
    if (level <= 0) level = 3;
    if (level >= 4) {
        // exact digit products (X in five 6-bit digits, Y in four 8-bit digits)
        tc_exact_tn(ctx, X, false, K, MM, ldx, Y, NN, ldy, C, ldc, false, 5);
        return;
    }
    BfxPlanes px, py;
    bfx_planes(ctx, px, X, false, MM, K, ldx, 1, bfx_tile_rows(level, true), level);
    bfx_planes(ctx, py, Y, false, NN, K, ldy, 1, bfx_tile_rows(level, false), level);
    bfx_gemm(ctx, level, px, py, C, ldc, false);
}

}  // namespace rnla
