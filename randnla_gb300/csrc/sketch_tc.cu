// Tensor-core sketch application for sm_103a (tcgen05 + TMEM + bulk async copies).
//
//   C (M x N, FP64) = S Y,   S (M x K) the Philox Gaussian sketch quantised
//   to multiples of 1/8 (|t| <= 63, exact in bf16), Y (K x N) an FP64 or FP32
//   matrix, K = rows of the data (the sketch_and_precondition.rs:51-52
//   products S a and S b, and A Omega of the range finder).
//
// Exactness.  Y is cut into P bf16 "digits" per element: with E_j the
// exponent of the largest |Y[:, j]| (|y| < 2^E_j), T = round(|y| 2^(7P-E_j))
// < 2^(7P)+1 is split into base-128 digits d_1..d_P (d_1 <= 128), each
// carrying the sign of y.  A digit times a sketch entry is an integer of
// magnitude <= 63*128 < 2^13, so the FP32 tensor-core accumulation of 2048
// consecutive K (one "window") is an integer below 2^24: exact.  After each
// window the worker warps read the P accumulators from TMEM, fold
// D_1 2^(7(P-1)) + ... + D_P exactly in int64, scale by 2^(E_j - 7P - 3)
// and add the result into the CTA's FP64 partial tile.  The roundings are
// the digit truncation (|error| <= 2^(E_j - 7P - 1) per entry of Y), one
// FP64 conversion per window, and the FP64 sums of windows and K chunks;
// S is applied exactly.
//
// Kernel structure (one CTA per SM, 576 threads):
//   warp 0      loads the digit tiles of Y with cp.async.bulk into a
//               2-stage ring (mbarrier complete_tx);
//   warp 1      allocates TMEM (512 columns) and issues tcgen05.mma
//               (M = 128, N = 96, K = 16, bf16 x bf16 -> f32) from one lane;
//   warps 2-17  ("workers") generate the 128 x 64 sketch tile of each stage
//               straight into shared memory in the SWIZZLE_128B K-major
//               layout -- S never exists in global memory -- and, after each
//               window, drain TMEM into int64 accumulators (24 columns per
//               warp); at the end they write the FP64 partial tile of the
//               CTA's K range.
// Split-K partials are summed in a fixed order by a second kernel.
//
// Every mbarrier wait is bounded (2 s of globaltimer); on timeout the CTA
// records an error, drains its own bulk copies, frees TMEM and exits.
#include "rnla_internal.h"
#include "rnla_async.cuh"
#include <cuda_bf16.h>
#include <vector>
#include <cstring>

namespace rnla {

namespace tc {

constexpr int BM = 128;           // sketch rows per CTA tile (TMEM lanes)
constexpr int BN = 96;            // data columns per CTA tile
constexpr int BK = 64;            // K per pipeline stage (one 128-byte bf16 row)
constexpr int WIN = 32;           // stages per exact window (2048 K values)
constexpr int STAGES = 2;
constexpr int WORKERS = 16;                          // generator + epilogue warps
constexpr int THREADS = 64 + 32 * WORKERS;           // + loader warp + MMA warp
constexpr int S_BYTES = BM * BK * 2;                 // 16 KB sketch tile
constexpr int ROW_BYTES = BK * 2;                    // 128
constexpr int YD_BYTES = BN * ROW_BYTES;             // one digit tile, 12 KB
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
    d |= (uint64_t)1 << 16;                              // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024u >> 4) << 32;                   // stride byte offset
    d |= (uint64_t)1 << 46;                              // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;                              // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M = 128, N = BN.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

struct Params {
    RngKey key;
    int64_t M, N, K;          // C is M x N, reduction length K
    int64_t M4;               // M rounded up to 4 (sketch stream row stride)
    int tiles_m, tiles_n, Ks, kc_count, stages_per_kc;
    const uint16_t* ydig;     // digit planes [jt][stage][p][BN rows][64] bf16 (SW128 images)
    const int* colexp;        // E_j per column (padded to tiles_n*BN)
    double* partial;          // [kc][tile][BN][BM] FP64 (row fastest)
    unsigned int* status;
};

// 8x the 4 quantised sketch entries of block g (rows 4q..4q+3 of stream
// column k): the integers t in [-63, 63]; the 1/8 goes into the final scale.
// The four quantised entries t (integers, |t| <= 63) of block g.
__device__ __forceinline__ void sketch_block(const RngKey& key, uint64_t g, const uint32_t* tab, float v[4]) {
    uint32_t w[4];
    block_words(key, g, w);
#pragma unroll
    for (int t = 0; t < 4; ++t) v[t] = (float)qgauss_t(w[t], tab);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    // both values are integers with |t| <= 63: exact in bf16 (truncation is exact)
    return (__float_as_uint(lo) >> 16) | (__float_as_uint(hi) & 0xFFFF0000u);
}

// DSMEM helpers: the shared::cluster address of `p` in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa_u32(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// local shared -> peer shared bulk copy, completing on the peer's mbarrier
__device__ __forceinline__ void bulk_s2peer(uint32_t dst_cluster, uint32_t src_cta, uint32_t bytes,
                                            uint32_t bar_cluster) {
    asm volatile(
        "cp.async.bulk.shared::cluster.shared::cta.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst_cluster),
        "r"(src_cta), "r"(bytes), "r"(bar_cluster)
        : "memory");
}
__device__ __forceinline__ void mma_commit_mc(uint64_t* bar, uint16_t mask) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"(mask)
        : "memory");
}

// C = CTAs per cluster along the column tiles of Y.  They apply the same
// sketch tile, so each generates 1/C of its rows and copies that piece into
// every peer's stage buffer (cp.async.bulk shared::cta -> shared::cluster);
// MMA completion is multicast to every peer's `empty` barrier, so no CTA
// overwrites a stage a peer is still reading.
template <int P, int C>
__global__ void __launch_bounds__(THREADS, 1) sketch_tc_kernel(const Params prm) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    __shared__ uint32_t qtab[128];                                // quantised-Gaussian alias table
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sS = smem;                                           // STAGES x 16 KB
    uint8_t* sY = smem + STAGES * S_BYTES;                        // STAGES x P x 12 KB
    uint64_t* bars = (uint64_t*)(sY + STAGES * P * YD_BYTES);
    uint64_t* fullY = bars;                                       // digit tile landed (tx)
    uint64_t* fullS = bars + STAGES;                              // whole sketch tile present (arrive + tx)
    uint64_t* empty = bars + 2 * STAGES;                          // every cluster MMA done with the stage
    uint64_t* genDone = bars + 3 * STAGES;                        // local worker warps wrote their rows
    uint64_t* accFull = bars + 4 * STAGES;
    uint64_t* accEmpty = accFull + 1;
    uint64_t* drain = accEmpty + 1;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    volatile int* err = (volatile int*)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // blockIdx.x = jr + C * (it + tiles_m * (kc + kc_count * jg)), jt = jg * C + jr
    const uint32_t jr = (C > 1) ? cluster_rank() : 0u;
    const int rest0 = blockIdx.x / C;
    const int it = rest0 % prm.tiles_m;
    const int rest = rest0 / prm.tiles_m;
    const int kc = rest % prm.kc_count;
    const int jg = rest / prm.kc_count;
    const int jt = jg * C + (int)jr;
    const int s_begin = kc * prm.stages_per_kc;
    const int s_end = min(prm.Ks, s_begin + prm.stages_per_kc);
    const int nst = s_end - s_begin;
    // this CTA's share of the 32 four-row groups of the sketch tile
    const int g_lo = (32 * (int)jr) / C, g_hi = (32 * ((int)jr + 1)) / C;
    const uint32_t own_bytes = (uint32_t)(g_hi - g_lo) * 4u * ROW_BYTES;

    if (threadIdx.x < 128) qtab[threadIdx.x] = k_qgauss_table[threadIdx.x];
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&fullY[s], 1);
            mbar_init(&fullS[s], 1);
            mbar_init(&empty[s], C);
            mbar_init(&genDone[s], WORKERS);
        }
        mbar_init(accFull, 1);
        mbar_init(accEmpty, WORKERS);
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
    if (C > 1) cluster_sync_all();          // peers' barriers exist before any remote operation
    tc_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ---------------- digit-tile loader ----------------
        if (lane == 0) {
            int issued = 0;
            for (int i = 0; i < nst; ++i) {
                const int slot = i % STAGES;
                if (i >= STAGES && !mbar_wait(&empty[slot], ((i / STAGES) - 1) & 1, err)) break;
                mbar_expect_tx(&fullY[slot], (uint32_t)(P * YD_BYTES));
                const uint8_t* src = (const uint8_t*)prm.ydig +
                                     ((size_t)jt * prm.Ks + (s_begin + i)) * (size_t)(P * YD_BYTES);
#pragma unroll
                for (int p = 0; p < P; ++p)
                    bulk_g2s(sY + (slot * P + p) * YD_BYTES, src + p * YD_BYTES, YD_BYTES, &fullY[slot]);
                ++issued;
            }
            for (int i = (issued > STAGES ? issued - STAGES : 0); i < issued; ++i) {
                const int slot = i % STAGES;
                if (!mbar_try(&fullY[slot], (i / STAGES) & 1)) {
                    const unsigned long long t0 = globaltimer_ns();
                    while (!mbar_try(&fullY[slot], (i / STAGES) & 1))
                        if (globaltimer_ns() - t0 > WAIT_NS) break;
                }
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(BM, BN);
            int win_count = 0;
            for (int i = 0; i < nst; ++i) {
                const int slot = i % STAGES;
                const int in_win = i % WIN;
                if (in_win == 0 && win_count > 0) {
                    if (!mbar_wait(accEmpty, (win_count - 1) & 1, err)) break;
                    tc_after();
                }
                if (!mbar_wait(&fullY[slot], (i / STAGES) & 1, err)) break;
                if (!mbar_wait(&fullS[slot], (i / STAGES) & 1, err)) break;
                tc_after();
                const uint32_t a0 = smem_u32(sS + slot * S_BYTES);
#pragma unroll
                for (int p = 0; p < P; ++p) {
                    const uint32_t b0 = smem_u32(sY + (slot * P + p) * YD_BYTES);
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk)
                        mma_bf16(tmem + p * BN, sw128_desc(a0 + kk * 32), sw128_desc(b0 + kk * 32), idesc,
                                 (in_win > 0 || kk > 0) ? 1u : 0u);
                }
                if (C > 1) mma_commit_mc(&empty[slot], (uint16_t)((1u << C) - 1u));
                else mma_commit(&empty[slot]);
                if (in_win == WIN - 1 || i == nst - 1) {
                    mma_commit(accFull);
                    ++win_count;
                }
            }
            mma_commit(drain);
            const unsigned long long t0 = globaltimer_ns();
            while (!mbar_try(drain, 0))
                if (globaltimer_ns() - t0 > WAIT_NS) { *err = 1; break; }
        }
    } else {
        // ---------------- workers: this CTA's rows of each sketch tile, TMEM drain per window ----
        const int wk = warp - 2;
        const int wt = threadIdx.x - 64;
        const int64_t i_base = (int64_t)it * BM;
        const uint64_t gstride = (uint64_t)(prm.M4 >> 2);
        const int q = warp & 3;
        const int h = wk >> 2;
        constexpr int CW = BN / 4;
        const int row = 32 * q + lane;
        const int tile = it + prm.tiles_m * jt;
        double* out = prm.partial + ((size_t)kc * prm.tiles_m * prm.tiles_n + tile) * (size_t)(BM * BN);
        const int units = (g_hi - g_lo) * 32;          // (4 rows, 2 consecutive k) per unit
        int win = 0;
        bool ok = true;
        for (int i = 0; i < nst && ok; ++i) {
            const int slot = i % STAGES;
            if (i >= STAGES) {
                bool w_ok = true;
                if (lane == 0) w_ok = mbar_wait(&empty[slot], ((i / STAGES) - 1) & 1, err);
                w_ok = __shfl_sync(0xffffffffu, w_ok, 0);
                if (!w_ok) { ok = false; break; }
            }
            const int64_t k0 = (int64_t)(s_begin + i) * BK;
            uint8_t* dst = sS + slot * S_BYTES;
#pragma unroll 1
            for (int u = wt; u < units; u += 32 * WORKERS) {
                const int kp = u & 31, ig = g_lo + (u >> 5);
                const int64_t row0 = i_base + 4 * ig;
                const int64_t k = k0 + 2 * kp;
                float v0[4], v1[4];
                if (row0 < prm.M && k < prm.K) sketch_block(prm.key, (uint64_t)(row0 >> 2) + (uint64_t)k * gstride, qtab, v0);
                else v0[0] = v0[1] = v0[2] = v0[3] = 0.f;
                if (row0 < prm.M && k + 1 < prm.K)
                    sketch_block(prm.key, (uint64_t)(row0 >> 2) + (uint64_t)(k + 1) * gstride, qtab, v1);
                else v1[0] = v1[1] = v1[2] = v1[3] = 0.f;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int r = 4 * ig + t;
                    const bool rv = row0 + t < prm.M;
                    const int kl = 2 * kp;                      // 0..62 within the stage
                    uint32_t* qd = (uint32_t*)(dst + r * ROW_BYTES + ((((kl >> 3) ^ (r & 7))) << 4) + ((kl & 7) << 1));
                    *qd = pack_bf16(rv ? v0[t] : 0.f, rv ? v1[t] : 0.f);
                }
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&genDone[slot]);
            if (wk == 0 && lane == 0) {
                // all local rows written: push them to the peers, then announce them locally
                if (!mbar_wait(&genDone[slot], (i / STAGES) & 1, err)) { ok = false; }
                else {
                    if (C > 1) {
                        const uint32_t src = smem_u32(dst) + (uint32_t)(4 * g_lo * ROW_BYTES);
                        for (uint32_t pr = 0; pr < (uint32_t)C; ++pr) {
                            if (pr == jr) continue;
                            bulk_s2peer(mapa_u32(src, pr), src, own_bytes, mapa_u32(smem_u32(&fullS[slot]), pr));
                        }
                        mbar_expect_tx(&fullS[slot], (uint32_t)S_BYTES - own_bytes);
                    } else {
                        mbar_arrive(&fullS[slot]);
                    }
                }
            }
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            if (!ok) break;
            if ((i % WIN) == WIN - 1 || i == nst - 1) {
                if (!mbar_wait(accFull, win & 1, err)) { ok = false; break; }
                tc_after();
#pragma unroll 1
                for (int c8 = 0; c8 < CW; c8 += 8) {
                    long long v[8];
#pragma unroll
                    for (int c = 0; c < 8; ++c) v[c] = 0;
#pragma unroll
                    for (int p = 0; p < P; ++p) {
                        uint32_t r[8];
                        tmem_ld8(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(p * BN + h * CW + c8), r);
                        tmem_ld_wait();
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            const long long d = (long long)__float2int_rn(__uint_as_float(r[c]));
                            v[c] += d * (1LL << (7 * (P - 1 - p)));
                        }
                    }
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const int col = h * CW + c8 + c;
                        const double val = ldexp((double)v[c], prm.colexp[jt * BN + col] - 7 * P - 3);
                        double* o = out + (size_t)col * BM + row;
                        *o = (win == 0) ? val : *o + val;
                    }
                }
                tc_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(accEmpty);
                ++win;
            }
        }
    }
    tc_before();
    __syncthreads();
    if (C > 1) cluster_sync_all();          // no peer still copies into or arrives on this CTA
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

template <typename T>
__global__ void colexp_kernel(const T* __restrict__ Y, int64_t K, int64_t N, int64_t ldy,
                              const double* __restrict__ extra, int* __restrict__ E) {
    const int64_t j = blockIdx.x;
    int best = -100000;
    for (int64_t k = threadIdx.x; k < K; k += blockDim.x) {
        uint64_t M;
        int e2;
        bool neg;
        load_elem(Y, ldy, N, extra, k, j, M, e2, neg);
        if (M) best = max(best, e2 + 64 - __clzll((long long)M));
    }
    __shared__ int red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x < 32) {
        best = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : -100000;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
        if (threadIdx.x == 0) E[j] = (best == -100000) ? -1074 : best;
    }
}

__device__ __forceinline__ uint16_t digit_bf16(uint32_t d, bool neg) {
    // d <= 128: the float of d has at most 8 significant bits, so its top 16 bits are the bf16
    const float f = (float)d;
    return (uint16_t)((__float_as_uint(f) >> 16) | (neg && d ? 0x8000u : 0u));
}

// One thread per (column j, 8 consecutive k): reads 8 values, writes P 16-byte
// chunks into the SW128 images [jt][stage][p][BN][64].  Ntot = N (+1 with extra).
template <typename T, int P>
__global__ void slice_kernel(const T* __restrict__ Y, int64_t K, int64_t N, int64_t ldy,
                             const double* __restrict__ extra, int64_t Ntot, const int* __restrict__ E,
                             int Ks, int tiles_n, uint16_t* __restrict__ out) {
    const int64_t chunks_per_col = (int64_t)Ks * 8;
    const int64_t total = chunks_per_col * (int64_t)tiles_n * BN;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < total;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = u / chunks_per_col;
        const int64_t cc = u % chunks_per_col;
        const int s = (int)(cc >> 3), c8 = (int)(cc & 7);
        const int jt = (int)(j / BN), jl = (int)(j % BN);
        const int Ej = (j < Ntot) ? E[j] : 0;
        uint16_t dg[P][8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int64_t k = (int64_t)s * BK + c8 * 8 + t;
            uint64_t M = 0;
            int e2 = 0;
            bool neg = false;
            if (j < Ntot && k < K) load_elem(Y, ldy, N, extra, k, j, M, e2, neg);
            uint64_t Tq = 0;
            if (M) {
                const int sh = Ej - 7 * P - e2;
                if (sh <= 0) Tq = M << (-sh);
                else if (sh < 64) Tq = (M + (1ull << (sh - 1))) >> sh;
            }
#pragma unroll
            for (int p = 0; p < P; ++p) {
                const uint32_t d = (p == 0) ? (uint32_t)(Tq >> (7 * (P - 1)))
                                            : (uint32_t)((Tq >> (7 * (P - 1 - p))) & 127u);
                dg[p][t] = digit_bf16(d, neg);
            }
        }
        const size_t blk = ((size_t)jt * Ks + s) * P;
#pragma unroll
        for (int p = 0; p < P; ++p) {
            uint4 v;
            v.x = dg[p][0] | ((uint32_t)dg[p][1] << 16);
            v.y = dg[p][2] | ((uint32_t)dg[p][3] << 16);
            v.z = dg[p][4] | ((uint32_t)dg[p][5] << 16);
            v.w = dg[p][6] | ((uint32_t)dg[p][7] << 16);
            uint8_t* base = (uint8_t*)out + (blk + p) * (size_t)YD_BYTES;
            *(uint4*)(base + jl * ROW_BYTES + ((c8 ^ (jl & 7)) << 4)) = v;
        }
    }
}

// C[i, j] = sum over kc of partial[kc][tile][col][row]
__global__ void splitk_sum_kernel(const double* __restrict__ part, int kc_count, int tiles_m, int tiles_n,
                                  int64_t M, int64_t N, double* __restrict__ C, int64_t ldc) {
    const int64_t total = M * N;
    const size_t tile_elems = (size_t)BM * BN;
    const size_t kc_stride = (size_t)tiles_m * tiles_n * tile_elems;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % M, j = e / M;
        const int it = (int)(i / BM), jt = (int)(j / BN);
        const size_t off = (size_t)(it + (int64_t)tiles_m * jt) * tile_elems + (size_t)(j % BN) * BM + (i % BM);
        double s = 0.0;
        for (int k = 0; k < kc_count; ++k) s += part[k * kc_stride + off];
        C[i + j * ldc] = s;
    }
}

template <int P>
static size_t smem_bytes() {
    return 1024 + (size_t)STAGES * S_BYTES + (size_t)STAGES * P * YD_BYTES + 512;
}

// cluster sizes that are instantiated; a column-tile count between them is
// padded with all-zero tiles
static int pick_cluster(int tiles_n) {
    static const int sizes[] = {1, 2, 4, 6, 8};
    if (tiles_n <= 8) {
        for (int c : sizes) if (c >= tiles_n) return c;
    }
    const int groups = (tiles_n + 7) / 8;
    const int want = (tiles_n + groups - 1) / groups;
    for (int c : sizes) if (c >= want) return c;
    return 8;
}

template <int P, int C>
static void launch_sketch(Ctx& ctx, const Params& prm, int64_t grid, size_t smem) {
    auto kfn = sketch_tc_kernel<P, C>;
    RNLA_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RNLA_CUDA(cudaLaunchKernelEx(&cfg, kfn, prm));
    RNLA_LAUNCH_CHECK();
}

template <int P, int C>
static bool cluster_fits(size_t smem) {
    auto kfn = sketch_tc_kernel<P, C>;
    if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (C == 1) return true;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, kfn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return nclusters > 0;
}

template <int P>
static void run(Ctx& ctx, const RngKey& key, const void* Y, bool y_f32, int64_t K, int64_t N0, int64_t ldy,
                const double* extra, int64_t M, double* C, int64_t ldc) {
    const int64_t N = N0 + (extra ? 1 : 0);      // the extra column is appended as column N0
    const int tiles_m = div_up(M, BM), tiles_n_real = div_up(N, BN);
    const size_t smem = smem_bytes<P>();
    int CL = (P >= 4) ? pick_cluster(tiles_n_real) : 1;
    bool fits = true;
    switch (CL) {
        case 2: fits = cluster_fits<P, 2>(smem); break;
        case 4: fits = cluster_fits<P, 4>(smem); break;
        case 6: fits = cluster_fits<P, 6>(smem); break;
        case 8: fits = cluster_fits<P, 8>(smem); break;
        default: break;
    }
    if (!fits) CL = 1;
    const int tiles_n = ((tiles_n_real + CL - 1) / CL) * CL;
    const int Ks = div_up(K, BK);
    const int wins = div_up(Ks, WIN);
    // choose the K split: minimise waves x windows-per-CTA plus partial traffic
    const int sm = ctx.sm_count;
    const int64_t tiles = (int64_t)tiles_m * tiles_n;
    int best_kc = 1;
    double best_cost = 1e300;
    for (int kcn = 1; kcn <= wins; ++kcn) {
        const int wpk = div_up(wins, kcn);
        const int kc_eff = div_up(wins, wpk);
        const int64_t ctas = tiles * kc_eff;
        const int64_t waves = (ctas + sm - 1) / sm;
        const double cost = (double)waves * wpk + 0.02 * (double)kc_eff * tiles / sm;
        if (cost < best_cost - 1e-9) { best_cost = cost; best_kc = kc_eff; }
    }
    const int spk = div_up(Ks, best_kc);
    const int kc_count = div_up(Ks, spk);

    DevBuf<int> E((size_t)tiles_n * BN, ctx.stream);
    RNLA_CUDA(cudaMemsetAsync(E.get(), 0, sizeof(int) * tiles_n * BN, ctx.stream));
    DevBuf<uint16_t> dig((size_t)tiles_n * Ks * P * (YD_BYTES / 2), ctx.stream);
    DevBuf<double> part((size_t)kc_count * tiles * BM * BN, ctx.stream);
    if (y_f32) colexp_kernel<float><<<(unsigned)N, 256, 0, ctx.stream>>>((const float*)Y, K, N0, ldy, extra, E);
    else colexp_kernel<double><<<(unsigned)N, 256, 0, ctx.stream>>>((const double*)Y, K, N0, ldy, extra, E);
    RNLA_LAUNCH_CHECK();
    {
        const int64_t units = (int64_t)Ks * 8 * tiles_n * BN;
        int g = div_up(units, 256);
        if (g > 32 * sm) g = 32 * sm;
        if (y_f32)
            slice_kernel<float, P><<<g, 256, 0, ctx.stream>>>((const float*)Y, K, N0, ldy, extra, N, E, Ks, tiles_n, dig);
        else
            slice_kernel<double, P><<<g, 256, 0, ctx.stream>>>((const double*)Y, K, N0, ldy, extra, N, E, Ks, tiles_n, dig);
        RNLA_LAUNCH_CHECK();
    }
    Params prm;
    prm.key = key;
    prm.M = M; prm.N = N; prm.K = K; prm.M4 = (M + 3) & ~3LL;
    prm.tiles_m = tiles_m; prm.tiles_n = tiles_n; prm.Ks = Ks;
    prm.kc_count = kc_count; prm.stages_per_kc = spk;
    prm.ydig = dig; prm.colexp = E; prm.partial = part; prm.status = ctx.status;
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    const int64_t grid = tiles * kc_count;
    switch (CL) {
        case 2: launch_sketch<P, 2>(ctx, prm, grid, smem); break;
        case 4: launch_sketch<P, 4>(ctx, prm, grid, smem); break;
        case 6: launch_sketch<P, 6>(ctx, prm, grid, smem); break;
        case 8: launch_sketch<P, 8>(ctx, prm, grid, smem); break;
        default: launch_sketch<P, 1>(ctx, prm, grid, smem); break;
    }
    int g = div_up(M * N, 256);
    if (g > 8 * sm) g = 8 * sm;
    splitk_sum_kernel<<<g, 256, 0, ctx.stream>>>(part, kc_count, tiles_m, tiles_n, M, N, C, ldc);
    RNLA_LAUNCH_CHECK();
    ctx.check_status("tensor-core sketch");
}

}  // namespace tc

bool tc_available(Ctx& ctx) {
    int major = 0, minor = 0;
    RNLA_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, ctx.device));
    RNLA_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, ctx.device));
    return major == 10 && minor == 3;
}

void tc_sketch_apply(Ctx& ctx, const RngKey& key, const void* X, bool x_f32, int64_t K, int64_t N,
                     int64_t ldx, const double* extra, int64_t M, int digits, double* C, int64_t ldc) {
    if (K <= 0 || (N <= 0 && !extra) || M <= 0) return;
    if (digits <= 0) digits = x_f32 ? 4 : 5;
    switch (digits) {
        case 1: tc::run<1>(ctx, key, X, x_f32, K, N, ldx, extra, M, C, ldc); break;
        case 2: tc::run<2>(ctx, key, X, x_f32, K, N, ldx, extra, M, C, ldc); break;
        case 3: tc::run<3>(ctx, key, X, x_f32, K, N, ldx, extra, M, C, ldc); break;
        case 4: tc::run<4>(ctx, key, X, x_f32, K, N, ldx, extra, M, C, ldc); break;
        case 5: tc::run<5>(ctx, key, X, x_f32, K, N, ldx, extra, M, C, ldc); break;
        default: fail(RNLA_ERR_INVALID_PARAMETERS, "digits must be 1..5");
    }
}

void tc_gemm_tn(Ctx&, const double*, int64_t, int64_t, int64_t, const double*, int64_t, int64_t, int,
                int, double*, int64_t) {
    fail(RNLA_ERR_UNSUPPORTED, "two-sided digit-sliced GEMM is not built; use RNLA_PREC_FP64");
}

}  // namespace rnla
