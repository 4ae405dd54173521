// Split-bf16 tensor-core GEMM for the tensor-core path of rand_svd: the
// range-finder products A Omega, A^T Q, A Z and Q^T A (lora_helpers.rs:17-44,
// 58-105 in the RandNLA form) and the Gram / triangular products of the
// CholeskyQR2 orthonormalisations between them.
//
//   C (M x N, FP64) = X^T Y,   X (K x M) and Y (K x N) given as bf16 planes:
//   X = X_0 + X_1 + X_2 + ..., X_0 the bf16 rounding of X, X_p the bf16
//   rounding of what X_0 .. X_{p-1} leave (each remainder is formed exactly),
//   likewise Y.  Level L keeps the plane pairs p + q < L:
//     L = 1: X_0 Y_0                             (plain bf16 operands)
//     L = 2: X_0 Y_0 + X_0 Y_1 + X_1 Y_0        (~16 significant bits each)
//     L = 3: the six pairs with p + q < 3       (~24 bits: FP32 data exact)
//   The products accumulate in FP32 in TMEM over a whole K chunk; split-K
//   chunks are summed in FP64 in a fixed order, so results are reproducible.
//
// Operand images.  bfx_planes() writes a matrix as tiles [row tile][K stage]
// [plane] of TR rows x 64 K bf16 in the K-major SWIZZLE_128B layout of the
// tcgen05 shared-memory descriptors (row r at byte 128 r, 16-byte chunk c at
// position c ^ (r & 7)), from either storage order: element (r, k) of the
// operand is src[r sr + k sk], so the columns of a column-major matrix
// (sr = ld, sk = 1) and its rows (sr = 1, sk = ld) are both operands.  One
// cp.async.bulk moves the L planes of a tile.
//
// Kernel (persistent, one CTA per SM, 192 threads): warp 0 streams the X and
// Y planes of each K stage into a 3-stage mbarrier ring; warp 1 issues, per
// 16-wide K step and per X plane p, ONE tcgen05.mma of M = 128 and N =
// (L - p) BN against the first L - p Y planes (contiguous in shared memory),
// each pair accumulating in its own TMEM column block; warps 2-5 drain TMEM
// at the end of each work unit, summing the pair blocks in FP64, and store
// the unit's FP64 tile.  Work units are (M tile, N tile, K chunk) with the N
// tile fastest, so the CTAs that share an X tile run side by side and X is
// read from HBM about once.  Every mbarrier wait is bounded (2 s).
#include "rnla_internal.h"
#include "rnla_async.cuh"
#include "rnla_tc.cuh"
#include "rnla_ff.cuh"
#include <cuda_bf16.h>
#include <algorithm>

namespace rnla {
namespace bfx {

using namespace tc;

constexpr int BM = 128;
constexpr int BK = 64;
constexpr int THREADS = 192;
constexpr int DRAIN_WARPS = 4;
constexpr int XT_BYTES = BM * BK * 2;        // one X plane tile, 16 KB
constexpr unsigned long long WAIT_NS = 2000000000ull;

template <int L>
struct Shape;
template <>
struct Shape<1> {
    static constexpr int BN = 256;            // one bf16 product per K step, N = 256
    static constexpr int STAGES = 4;
};
template <>
struct Shape<2> {
    static constexpr int BN = 96;             // N per pair block; N of one MMA: 192 or 96
    static constexpr int STAGES = 3;
};
template <>
struct Shape<3> {
    static constexpr int BN = 64;             // N of one MMA: 192, 128 or 64
    static constexpr int STAGES = 3;
};

struct Params {
    int64_t M, N;
    int tiles_m, tiles_n, Ks, kc_count, stages_per_kc, units;
    int px, py;                  // planes stored per tile in the X / Y images
    const uint8_t* xp;           // [tiles_m][Ks][px] tiles of BM x 64
    const uint8_t* yp;           // [tiles_n][Ks][py] tiles of BN x 64
    double* partial;             // [kc][tile][BN][BM]
    unsigned int* status;
};

struct Unit {
    int it, jt, kc, s_begin, nst;
};
__device__ __forceinline__ Unit unit_of(const Params& p, int u) {
    Unit w;
    w.jt = u % p.tiles_n;
    const int rest = u / p.tiles_n;
    w.it = rest % p.tiles_m;
    w.kc = rest / p.tiles_m;
    w.s_begin = w.kc * p.stages_per_kc;
    w.nst = min(p.Ks, w.s_begin + p.stages_per_kc) - w.s_begin;
    return w;
}

template <int L>
__host__ __device__ constexpr int region_off(int p) {
    int o = 0;
    for (int q = 0; q < p; ++q) o += (L - q) * Shape<L>::BN;
    return o;
}

template <int L>
__global__ void __launch_bounds__(THREADS, 1) bfx_gemm_kernel(const Params prm) {
    constexpr int BN = Shape<L>::BN;
    constexpr int STAGES = Shape<L>::STAGES;
    constexpr int YT_BYTES = BN * BK * 2;
    constexpr int XS_BYTES = L * XT_BYTES;
    constexpr int YS_BYTES = L * YT_BYTES;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* sX = smem;                                       // STAGES x L x 16 KB
    uint8_t* sY = smem + STAGES * XS_BYTES;                   // STAGES x L x BN x 128 B
    uint64_t* bars = (uint64_t*)(sY + STAGES * YS_BYTES);
    uint64_t* full = bars;
    uint64_t* empty = bars + STAGES;
    uint64_t* accFull = bars + 2 * STAGES;
    uint64_t* accEmpty = accFull + 1;
    uint64_t* drain = accEmpty + 1;
    uint32_t* tmem_slot = (uint32_t*)(drain + 1);
    volatile int* err = (volatile int*)(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accFull, 1);
        mbar_init(accEmpty, DRAIN_WARPS);
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
        // ---------------- loader ----------------
        if (lane == 0) {
            int g = 0;
            bool ok = true;
            for (int u = blockIdx.x; u < prm.units && ok; u += gridDim.x) {
                const Unit w = unit_of(prm, u);
                const uint8_t* xs = prm.xp + ((size_t)w.it * prm.Ks + w.s_begin) * prm.px * XT_BYTES;
                const uint8_t* ys = prm.yp + ((size_t)w.jt * prm.Ks + w.s_begin) * prm.py * (size_t)YT_BYTES;
                for (int i = 0; i < w.nst; ++i) {
                    const int slot = g % STAGES;
                    if (g >= STAGES && !mbar_wait(&empty[slot], (uint32_t)((g / STAGES) - 1) & 1u, err)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&full[slot], (uint32_t)(XS_BYTES + YS_BYTES));
                    bulk_g2s(sX + slot * XS_BYTES, xs + (size_t)i * prm.px * XT_BYTES, XS_BYTES, &full[slot]);
                    bulk_g2s(sY + slot * YS_BYTES, ys + (size_t)i * prm.py * YT_BYTES, YS_BYTES, &full[slot]);
                    ++g;
                }
            }
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
            int slot = 0;
            uint32_t fph = 0;
            int nu = 0;                  // units started
            bool ok = true;
            for (int u = blockIdx.x; u < prm.units && ok; u += gridDim.x, ++nu) {
                const Unit w = unit_of(prm, u);
                if (nu > 0) {
                    // the single accumulator set is free once the previous unit is drained
                    if (!mbar_wait(accEmpty, (uint32_t)(nu - 1) & 1u, err)) { ok = false; break; }
                    tc_after();
                }
                for (int i = 0; i < w.nst; ++i) {
                    if (!mbar_wait(&full[slot], fph, err)) { ok = false; break; }
                    tc_after();
                    const uint32_t x0 = smem_u32(sX + slot * XS_BYTES);
                    const uint32_t y0 = smem_u32(sY + slot * YS_BYTES);
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
#pragma unroll
                        for (int p = 0; p < L; ++p)
                            mma_bf16(tmem + (uint32_t)region_off<L>(p), sw128_desc(x0 + p * XT_BYTES + kk * 32),
                                     sw128_desc(y0 + kk * 32), idesc_bf16(BM, (L - p) * BN),
                                     (i > 0 || kk > 0) ? 1u : 0u);
                    }
                    mma_commit(&empty[slot]);
                    if (++slot == STAGES) { slot = 0; fph ^= 1u; }
                }
                if (!ok) break;
                mma_commit(accFull);
            }
            mma_commit(drain);
            const unsigned long long t0 = globaltimer_ns();
            while (!mbar_try(drain, 0))
                if (globaltimer_ns() - t0 > WAIT_NS) { *err = 1; break; }
        }
    } else {
        // ---------------- drain: TMEM lane quarter (warp & 3) ----------------
        const int q = warp & 3;
        const int row = 32 * q + lane;
        int nu = 0;
        for (int u = blockIdx.x; u < prm.units; u += gridDim.x, ++nu) {
            const Unit w = unit_of(prm, u);
            if (!mbar_wait(accFull, (uint32_t)nu & 1u, err)) break;
            tc_after();
            const uint32_t base = tmem + ((uint32_t)(32 * q) << 16);
            const int tile = w.it + prm.tiles_m * w.jt;
            double* out = prm.partial + ((size_t)w.kc * prm.tiles_m * prm.tiles_n + tile) * (size_t)(BM * BN);
#pragma unroll 1
            for (int c16 = 0; c16 < BN; c16 += 16) {
                double v[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) v[c] = 0.0;
#pragma unroll
                for (int p = 0; p < L; ++p) {
#pragma unroll
                    for (int qq = 0; qq < L - p; ++qq) {
                        uint32_t r[16];
                        tmem_ld16(base + (uint32_t)(region_off<L>(p) + qq * BN + c16), r);
                        tmem_ld_wait();
#pragma unroll
                        for (int c = 0; c < 16; ++c) v[c] += (double)__uint_as_float(r[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < 16; ++c) out[(size_t)(c16 + c) * BM + row] = v[c];
            }
            tc_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(accEmpty);
        }
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    if (threadIdx.x == 0 && *err) atomicCAS(prm.status, 0u, (unsigned int)KSTATUS_MBAR_TIMEOUT);
}

// ---------------------------------------------------------------------------
// Operand images
// ---------------------------------------------------------------------------
// Plane split of one value: p-th plane = bf16 rounding of what the earlier
// planes leave, in FP32 (each remainder v - bf16(v) is exact in FP32).  FP64
// data is first rounded to 24 bits with integer operations (ff_split), which
// the three planes of the widest level hold exactly.
__device__ __forceinline__ uint16_t split_step(float& rem) {
    const __nv_bfloat16 h = __float2bfloat16_rn(rem);
    rem -= __bfloat162float(h);
    return __bfloat16_as_ushort(h);
}
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(double v) { return ff_split(v).x; }

// Block = one (row tile, K stage): TR x 64 elements staged through shared
// memory as FP32 (coalesced reads along whichever index is contiguous, eight
// loads in flight per thread), then each thread writes one 16-byte chunk (8 K
// values) of one row for every plane.  TR x 64 is a multiple of 8 x 256.
template <typename T>
__global__ void __launch_bounds__(256) planes_kernel(const T* __restrict__ src, int64_t R, int64_t K, int64_t sr,
                                                     int64_t sk, int TR, int Ks, int PL, uint8_t* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char st_raw[];
    float* st = reinterpret_cast<float*>(st_raw);         // TR x (64 + 1)
    const int rt = blockIdx.x / Ks, s = blockIdx.x % Ks;
    const int64_t r0 = (int64_t)rt * TR, k0 = (int64_t)s * BK;
    const int n = TR * BK;
    const bool kfast = (sk == 1);
    for (int e0 = threadIdx.x; e0 < n; e0 += 8 * blockDim.x) {
        T v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int e = e0 + q * blockDim.x;
            const int r = kfast ? e / BK : e % TR;
            const int k = kfast ? e % BK : e / TR;
            const int64_t rg = r0 + r, kg = k0 + k;
            v[q] = (e < n && rg < R && kg < K) ? src[rg * sr + kg * sk] : (T)0;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int e = e0 + q * blockDim.x;
            const int r = kfast ? e / BK : e % TR;
            const int k = kfast ? e % BK : e / TR;
            if (e < n) st[r * (BK + 1) + k] = to_f32(v[q]);
        }
    }
    __syncthreads();
    const size_t tile_bytes = (size_t)TR * BK * 2;
    uint8_t* base = out + ((size_t)rt * Ks + s) * PL * tile_bytes;
    for (int t = threadIdx.x; t < TR * 8; t += blockDim.x) {
        const int r = t >> 3, c8 = t & 7;
        float rem[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) rem[j] = st[r * (BK + 1) + c8 * 8 + j];
        for (int p = 0; p < PL; ++p) {
            uint16_t h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) h[j] = split_step(rem[j]);
            uint4 v;
            v.x = h[0] | ((uint32_t)h[1] << 16);
            v.y = h[2] | ((uint32_t)h[3] << 16);
            v.z = h[4] | ((uint32_t)h[5] << 16);
            v.w = h[6] | ((uint32_t)h[7] << 16);
            *(uint4*)(base + p * tile_bytes + (size_t)r * 128 + ((c8 ^ (r & 7)) << 4)) = v;
        }
    }
}

// C[i, j] (or C[j, i] when trans) = sum over kc of partial[kc][tile][j % BN][i % BM].
__global__ void bfx_sum_kernel(const double* __restrict__ part, int kc_count, int tiles_m, int tiles_n, int BN,
                               int64_t M, int64_t N, int trans, double* __restrict__ C, int64_t ldc) {
    const size_t tile_elems = (size_t)BM * BN;
    const size_t kc_stride = (size_t)tiles_m * tiles_n * tile_elems;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < M * N; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % M, j = e / M;
        const size_t off = (size_t)((i / BM) + (int64_t)tiles_m * (j / BN)) * tile_elems + (size_t)(j % BN) * BM + (i % BM);
        double s = 0.0;
        for (int k = 0; k < kc_count; ++k) s += part[k * kc_stride + off];
        if (trans) C[j + i * ldc] = s;
        else C[i + j * ldc] = s;
    }
}

}  // namespace bfx

int bfx_tile_rows(int level, bool x_side) {
    if (x_side) return bfx::BM;
    return level == 1 ? bfx::Shape<1>::BN : level == 2 ? bfx::Shape<2>::BN : bfx::Shape<3>::BN;
}

void bfx_planes(Ctx& ctx, BfxPlanes& P, const void* src, bool f32, int64_t R, int64_t K, int64_t sr, int64_t sk,
                int TR, int planes) {
    using namespace bfx;
    if (R <= 0 || K <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "bfx planes: empty operand");
    if (planes < 1 || planes > 3) fail(RNLA_ERR_INVALID_PARAMETERS, "bfx planes: 1..3 planes");
    P.R = R;
    P.K = K;
    P.TR = TR;
    P.planes = planes;
    P.tiles = div_up(R, TR);
    P.Ks = div_up(K, BK);
    P.buf.alloc((size_t)P.tiles * P.Ks * planes * TR * BK * 2, ctx.stream);
    const size_t smem = (size_t)TR * (BK + 1) * sizeof(float);
    const unsigned blocks = (unsigned)((int64_t)P.tiles * P.Ks);
    if (f32) {
        auto k = planes_kernel<float>;
        set_smem_limit((const void*)k, smem);
        k<<<blocks, 256, smem, ctx.stream>>>(static_cast<const float*>(src), R, K, sr, sk, TR, P.Ks, planes, P.buf);
    } else {
        auto k = planes_kernel<double>;
        set_smem_limit((const void*)k, smem);
        k<<<blocks, 256, smem, ctx.stream>>>(static_cast<const double*>(src), R, K, sr, sk, TR, P.Ks, planes, P.buf);
    }
    RNLA_LAUNCH_CHECK();
}

template <int L>
static void run(Ctx& ctx, const BfxPlanes& X, const BfxPlanes& Y, double* C, int64_t ldc, bool trans) {
    using namespace bfx;
    constexpr int BN = Shape<L>::BN;
    constexpr int STAGES = Shape<L>::STAGES;
    const int sm = ctx.sm_count;
    const int64_t M = X.R, N = Y.R;
    const int tiles_m = X.tiles, tiles_n = Y.tiles, Ks = X.Ks;
    const int64_t tiles = (int64_t)tiles_m * tiles_n;
    // K split: minimise rounds x stages per unit (+ a per-unit drain cost of
    // about 8 stages), with rounds = ceil(units / SMs)
    int best = 1;
    double best_cost = 1e300;
    for (int kcn = 1; kcn <= 64 && kcn <= Ks; ++kcn) {
        const int spk = div_up(Ks, kcn);
        const int kc = div_up(Ks, spk);
        const int64_t units = tiles * kc;
        const int64_t rounds = (units + sm - 1) / sm;
        const double cost = (double)rounds * (spk + 8) + 0.001 * units;
        if (cost < best_cost - 1e-9) { best_cost = cost; best = kc; }
    }
    const int spk = div_up(Ks, best);
    const int kc_count = div_up(Ks, spk);
    const int64_t units = tiles * kc_count;
    DevBuf<double> part((size_t)kc_count * tiles * BM * BN, ctx.stream);
    Params prm;
    prm.M = M; prm.N = N;
    prm.tiles_m = tiles_m; prm.tiles_n = tiles_n; prm.Ks = Ks;
    prm.kc_count = kc_count; prm.stages_per_kc = spk; prm.units = (int)units;
    prm.px = X.planes; prm.py = Y.planes;
    prm.xp = X.buf; prm.yp = Y.buf; prm.partial = part; prm.status = ctx.status;
    const size_t smem = 1024 + (size_t)STAGES * (L * XT_BYTES + L * BN * BK * 2) + 256;
    auto kfn = bfx_gemm_kernel<L>;
    set_smem_limit((const void*)kfn, smem);
    ctx.clear_status();
    kfn<<<(unsigned)std::min<int64_t>(units, sm), THREADS, smem, ctx.stream>>>(prm);
    RNLA_LAUNCH_CHECK();
    int g = div_up(M * N, 256);
    if (g > 8 * sm) g = 8 * sm;
    bfx_sum_kernel<<<g, 256, 0, ctx.stream>>>(part, kc_count, tiles_m, tiles_n, BN, M, N, trans ? 1 : 0, C, ldc);
    RNLA_LAUNCH_CHECK();
    ctx.check_status("split-bf16 GEMM");
}

void bfx_gemm(Ctx& ctx, int level, const BfxPlanes& X, const BfxPlanes& Y, double* C, int64_t ldc, bool trans) {
    if (X.K != Y.K) fail(RNLA_ERR_INVALID_DIMENSIONS, "bfx gemm: operands disagree on K");
    if (X.TR != bfx::BM || Y.TR != bfx_tile_rows(level, false))
        fail(RNLA_ERR_INVALID_PARAMETERS, "bfx gemm: operand images have the wrong tile height");
    if (X.planes < level || Y.planes < level) fail(RNLA_ERR_INVALID_PARAMETERS, "bfx gemm: too few planes");
    if (level == 1) run<1>(ctx, X, Y, C, ldc, trans);
    else if (level == 2) run<2>(ctx, X, Y, C, ldc, trans);
    else if (level == 3) run<3>(ctx, X, Y, C, ldc, trans);
    else fail(RNLA_ERR_INVALID_PARAMETERS, "bfx gemm: level must be 1, 2 or 3");
}

}  // namespace rnla
