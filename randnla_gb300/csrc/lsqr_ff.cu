// Float-float LSQR for the BF16X precision: solvers.rs:115-278 run on the
// preconditioned operator A M, M = R^-1 of the sketch
// (sketch_and_precondition.rs:56), in one persistent cooperative launch.
//
// Layout.  The data matrix is re-laid out once per solve as a ROW-MAJOR
// float-float copy AF: the row stride ldf is n rounded up to even, and each
// 16-byte chunk holds a column pair as (hi_2p, hi_2p+1, lo_2p, lo_2p+1), so
// one load yields two packed f32x2 operands.  A tile of R rows is one
// contiguous block that a single cp.async.bulk moves into shared memory,
// completing on an mbarrier.  Each CTA streams its tiles (tile t = cta + k G)
// through a 3-stage ring that runs continuously across passes -- A never
// changes -- so the first tiles of the next pass are in flight while the
// grid is between passes.
//
// One pass over a tile (256 threads = 8 warps, R = 8 RW rows):
//   phase 1  warp w forms t_r = (A y)_r for rows r = w + 8 s (s < RW): each
//            lane reads 16-byte chunks of the row, y sits in registers,
//            products are exact (FMA error term) and summed with TwoSum on
//            packed pairs, then a warp butterfly; lane s forms
//            u_r = c1 t_r + c2 u_r + c3 b_r and accumulates ||u||^2;
//   phase 2  thread t owns the column pairs t + 256 q and accumulates A^T u
//            over the tile's rows.
// Both phases read 512 contiguous bytes per warp instruction (no bank
// conflicts).  Per-CTA partials are summed in a fixed order, so the run is
// reproducible.
//
// Arithmetic.  Every vector operation is float-float on the FP32 pipe.  FP64
// is used only by warp 0 of each CTA for the scalar recurrences: on GB300 a
// dependent FP64 operation takes ~64 cycles and a divide or square root
// several hundred, so the recurrences are arranged as a few lane-parallel
// rsqrt steps (different lanes of one warp instruction evaluate independent
// reciprocal square roots) plus multiplies; divisions become products with
// those reciprocals.  Results agree with the FP64 LSQR to float-float
// accuracy, and the iteration count can differ by one at a tolerance
// boundary.
//
// Waits are bounded: the grid barrier and the tile mbarriers give up after
// 2 s, record a status, let the CTA's own bulk copies land and return.
#include "rnla_internal.h"
#include "rnla_ff.cuh"
#include "rnla_async.cuh"

namespace rnla {
namespace lsff {

constexpr int T = 256;          // threads per CTA
constexpr int W = T / 32;       // warps per CTA
constexpr int ST = 3;           // tile ring depth
constexpr int64_t MAX_N = 1024;

struct Args {
    const float2* AF;           // row-major float-float copy of A, m x ldf
    int64_t m, n, ldf, hp;      // hp = ldf / 2 column pairs
    int R;                      // rows per tile (multiple of 8)
    int64_t ntiles;
    const float2* MF;           // M, column-major n x n (null: identity)
    const float2* MtF;          // M^T, column-major (row i of M contiguous)
    const float2* bF;           // b (m)
    const float2* x0F;          // x0 (n) or null
    float2 *uF, *yF, *gF, *vF, *wF, *xF, *vunF, *varF, *partF, *spF;
    float4* colsq;              // per column: vun_j^2 and w_j^2 (float-float each)
    double* x;                  // result z (n)
    double* var;                // nullable
    double* arn;                // nullable: arnorm before each iteration
    double* out;                // istop, itn, r1norm, r2norm, anorm, acond, xnorm, arnorm
    double damp, atol, btol, conlim, abs_tol;
    int64_t iter_lim;
    int calc_var;
    GridBarrier bar;
};

// Values warp 0 hands to the other warps.
struct Bcast {
    float2 ib, beta, ia, t1, t2, c2, irho;
    int beta_pos;
    int istop;
};

struct Ring {
    uint64_t* full;             // ST mbarriers
    float4* tiles;              // ST stages of R x hp float4
    int64_t cnt;                // sequence number of the next tile to consume
    int64_t issued;             // sequence number of the next tile to issue (thread 0)
    int64_t ntl;                // tiles of this CTA per pass
};

__device__ __forceinline__ void ring_issue(const Args& a, Ring& rg) {
    if (rg.ntl == 0) return;
    while (rg.issued < rg.cnt + ST) {
        const int64_t t = (int64_t)blockIdx.x + (rg.issued % rg.ntl) * (int64_t)gridDim.x;
        const int64_t r0 = t * a.R;
        const int64_t rows = min((int64_t)a.R, a.m - r0);
        const uint32_t bytes = (uint32_t)(rows * a.ldf * 8);
        const int st = (int)(rg.issued % ST);
        mbar_expect_tx(&rg.full[st], bytes);
        bulk_g2s(rg.tiles + (size_t)st * a.R * a.hp, a.AF + r0 * a.ldf, bytes, &rg.full[st]);
        ++rg.issued;
    }
}

// Thread 0: wait (bounded) until every copy still in flight has landed, so
// the CTA can exit with no bulk copy writing into its shared memory.
__device__ void ring_drain(Ring& rg) {
    if (threadIdx.x != 0) return;
    volatile int quiet = 0;
    for (int64_t s = rg.cnt; s < rg.issued; ++s)
        mbar_wait(&rg.full[s % ST], (uint32_t)((s / ST) & 1), &quiet);
}

__device__ __forceinline__ void set_status(const Args& a, unsigned int code) {
    atomicCAS(a.bar.status, 0u, code);
}

// One pass over the CTA's tiles:
//   dst_i = c1 (A y)_i + c2 old_i + c3 bvec_i     (A y skipped when !dot)
// accumulating sum dst_i^2 (spF slot 0), sum bvec_i^2 (slot 3, want_b2) and,
// when acc_at, the CTA's partial of A^T dst into partF.
// Tile rows: warp w handles rows w + 8 s (s < RW); a 16-byte chunk of a row
// is one column pair stored (hi_2p, hi_2p+1, lo_2p, lo_2p+1), i.e. two packed
// f32x2 operands, so every float-float multiply-add below serves two columns.
template <int KP, int RW>
__device__ bool ff_pass(const Args& a, Ring& rg, ulonglong2* usm, float2 c1, float2 c2, float2 c3, bool dot,
                        const float2* oldv, const float2* bvec, float2* dst, bool want_b2, bool acc_at,
                        volatile int* err) {
    constexpr int R = W * RW;
    __shared__ float2 wred[W][2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int hp = (int)a.hp;
    f32x2 yh[KP], nyh[KP], yl[KP];
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        const int p = lane + 32 * k;
        float2 y0 = make_float2(0.f, 0.f), y1 = make_float2(0.f, 0.f);
        if (dot && p < hp) { y0 = a.yF[2 * p]; y1 = a.yF[2 * p + 1]; }
        yh[k] = pk2(y0.x, y1.x);
        nyh[k] = pk2(-y0.x, -y1.x);
        yl[k] = pk2(y0.y, y1.y);
    }
    f32x2 ah[2][2], al[2][2];            // phase 2: [pair q][row-parity chain]
#pragma unroll
    for (int q = 0; q < 2; ++q) { ah[q][0] = ah[q][1] = al[q][0] = al[q][1] = 0ull; }
    float sqh = 0.f, sql = 0.f, b2h = 0.f, b2l = 0.f;

#pragma unroll 1
    for (int64_t k = 0; k < rg.ntl; ++k) {
        const int64_t s = rg.cnt;
        const int st = (int)(s % ST);
        const bool ok = mbar_wait(&rg.full[st], (uint32_t)((s / ST) & 1), err);
        const int64_t t = (int64_t)blockIdx.x + k * (int64_t)gridDim.x;
        const int64_t r0 = t * R;
        const int rows = (int)min((int64_t)R, a.m - r0);
        const ulonglong2* tile = reinterpret_cast<const ulonglong2*>(rg.tiles) + (size_t)st * R * hp;
        if (ok) {
            // lane w prefetches the old value and b of row warp + 8 w
            float2 uo = make_float2(0.f, 0.f), bb = make_float2(0.f, 0.f);
            if (lane < RW && warp + W * lane < rows) {
                const int64_t i = r0 + warp + W * lane;
                if (oldv) uo = oldv[i];
                if (bvec) bb = bvec[i];
            }
            float tvh[RW], tvl[RW];
#pragma unroll
            for (int w = 0; w < RW; ++w) { tvh[w] = 0.f; tvl[w] = 0.f; }
            if (dot) {
                f32x2 sh[RW][2], sl[RW][2];
#pragma unroll
                for (int w = 0; w < RW; ++w) { sh[w][0] = sh[w][1] = sl[w][0] = sl[w][1] = 0ull; }
#pragma unroll
                for (int kk = 0; kk < KP; ++kk) {
                    const int p = lane + 32 * kk;
                    if (p < hp) {
#pragma unroll
                        for (int w = 0; w < RW; ++w) {
                            const ulonglong2 v = tile[(size_t)(warp + W * w) * hp + p];
                            ff2_madd(v.x, v.y, yh[kk], nyh[kk], yl[kk], sh[w][kk & 1], sl[w][kk & 1]);
                        }
                    }
                }
#pragma unroll
                for (int w = 0; w < RW; ++w) {
                    ff2_acc(sh[w][0], sl[w][0], sh[w][1], sl[w][1]);
                    const float2 H = upk2(sh[w][0]), L = upk2(sl[w][0]);
                    float h = H.x, l = L.x;
                    ff_acc(h, l, H.y, L.y);
                    tvh[w] = h;
                    tvl[w] = l;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                    for (int w = 0; w < RW; ++w) {
                        const float oh = __shfl_xor_sync(0xffffffffu, tvh[w], o);
                        const float ol = __shfl_xor_sync(0xffffffffu, tvl[w], o);
                        ff_acc(tvh[w], tvl[w], oh, ol);
                    }
            }
            // lane w forms row warp + 8 w (its own butterfly result: all lanes hold the sum)
            if (lane < RW && warp + W * lane < rows) {
                float th = tvh[0], tl = tvl[0];
#pragma unroll
                for (int w = 1; w < RW; ++w)
                    if (lane == w) { th = tvh[w]; tl = tvl[w]; }
                const int r = warp + W * lane;
                const int64_t i = r0 + r;
                const float2 tv = ff_norm(th, tl);
                const float2 nv = ff_add(ff_add(ff_mul(c1, tv), ff_mul(c2, uo)), ff_mul(c3, bb));
                dst[i] = nv;
                usm[r] = make_ulonglong2(pk2(nv.x, nv.x), pk2(nv.y, nv.y));
                ff_madd(nv.x, nv.y, nv.x, nv.y, sqh, sql);
                if (want_b2) ff_madd(bb.x, bb.y, bb.x, bb.y, b2h, b2l);
            }
        }
        __syncthreads();
        if (*err) return false;
        if (acc_at) {
            int r = 0;
            for (; r + 1 < rows; r += 2) {
                const ulonglong2 u0 = usm[r], u1 = usm[r + 1];
                const f32x2 nu0 = neg2(u0.x), nu1 = neg2(u1.x);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int p = tid + q * T;
                    if (p < hp) {
                        const ulonglong2 v0 = tile[(size_t)r * hp + p];
                        const ulonglong2 v1 = tile[(size_t)(r + 1) * hp + p];
                        ff2_madd(v0.x, v0.y, u0.x, nu0, u0.y, ah[q][0], al[q][0]);
                        ff2_madd(v1.x, v1.y, u1.x, nu1, u1.y, ah[q][1], al[q][1]);
                    }
                }
            }
            if (r < rows) {
                const ulonglong2 u0 = usm[r];
                const f32x2 nu0 = neg2(u0.x);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int p = tid + q * T;
                    if (p < hp) {
                        const ulonglong2 v0 = tile[(size_t)r * hp + p];
                        ff2_madd(v0.x, v0.y, u0.x, nu0, u0.y, ah[q][0], al[q][0]);
                    }
                }
            }
        }
        __syncthreads();
        ++rg.cnt;
        if (tid == 0) ring_issue(a, rg);
    }
    if (acc_at) {
        float4* P4 = reinterpret_cast<float4*>(a.partF) + (size_t)blockIdx.x * hp;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int p = tid + q * T;
            if (p < hp) {
                ff2_acc(ah[q][0], al[q][0], ah[q][1], al[q][1]);
                const float2 H = upk2(ah[q][0]), L = upk2(al[q][0]);
                const float2 c0 = ff_norm(H.x, L.x), c1v = ff_norm(H.y, L.y);
                P4[p] = make_float4(c0.x, c0.y, c1v.x, c1v.y);
            }
        }
    }
    {
        const float2 sq = ff_warp_sum(sqh, sql);
        const float2 b2 = ff_warp_sum(b2h, b2l);
        if (lane == 0) { wred[warp][0] = sq; wred[warp][1] = b2; }
    }
    __syncthreads();
    if (tid == 0) {
        float h = 0.f, l = 0.f, h2 = 0.f, l2 = 0.f;
        for (int w = 0; w < W; ++w) {
            ff_acc(h, l, wred[w][0].x, wred[w][0].y);
            ff_acc(h2, l2, wred[w][1].x, wred[w][1].y);
        }
        a.spF[blockIdx.x * 4 + 0] = ff_norm(h, l);
        a.spF[blockIdx.x * 4 + 3] = ff_norm(h2, l2);
    }
    return true;
}

// Sum over CTAs of scalar slot `slot` (warp-level, identical in every CTA).
__device__ __forceinline__ float2 sum_slot(const Args& a, int slot, int lane) {
    float h = 0.f, l = 0.f;
    for (unsigned c = lane; c < gridDim.x; c += 32) {
        const float2 v = a.spF[c * 4 + slot];
        ff_acc(h, l, v.x, v.y);
    }
    return ff_warp_sum(h, l);
}

// g_j = sum over CTAs of partF[c][j]; one warp per column, warps 1..W-1.
__device__ void reduce_columns(const Args& a, int warp, int lane) {
    const int64_t nw = (int64_t)gridDim.x * (W - 1);
    for (int64_t j = (int64_t)blockIdx.x * (W - 1) + (warp - 1); j < a.n; j += nw) {
        float h = 0.f, l = 0.f;
        for (int64_t c = lane; c < gridDim.x; c += 32) {
            const float2 v = a.partF[c * a.ldf + j];
            ff_acc(h, l, v.x, v.y);
        }
        const float2 s = ff_warp_sum(h, l);
        if (lane == 0) a.gF[j] = s;
    }
}

// vun_j = (M^T g)_j ib - [sub] beta v_j, and the squares of vun_j and w_j;
// one warp per column, all warps.
__device__ void update_vun(const Args& a, const Bcast& bc, bool sub, int warp, int lane) {
    const int64_t n = a.n;
    const int64_t nw = (int64_t)gridDim.x * W;
    for (int64_t j = (int64_t)blockIdx.x * W + warp; j < n; j += nw) {
        float2 z;
        if (a.MF) {
            float h = 0.f, l = 0.f;
            const float2* col = a.MF + j * n;
            for (int64_t i = lane; i <= j; i += 32) {
                const float2 mv = col[i], gv = a.gF[i];
                ff_madd(mv.x, mv.y, gv.x, gv.y, h, l);
            }
            z = ff_warp_sum(h, l);
        } else {
            z = a.gF[j];
        }
        if (lane == 0) {
            float2 vv = ff_mul(z, bc.ib);
            if (sub) vv = ff_add(vv, ff_neg(ff_mul(bc.beta, a.vF[j])));
            a.vunF[j] = vv;
            const float2 wj = a.wF[j];
            float q1h = 0.f, q1l = 0.f, q2h = 0.f, q2l = 0.f;
            ff_madd(vv.x, vv.y, vv.x, vv.y, q1h, q1l);
            ff_madd(wj.x, wj.y, wj.x, wj.y, q2h, q2l);
            const float2 q1 = ff_norm(q1h, q1l), q2 = ff_norm(q2h, q2l);
            a.colsq[j] = make_float4(q1.x, q1.y, q2.x, q2.y);
        }
    }
}

// (sum_j vun_j^2, sum_j w_j^2), warp-level, identical in every CTA.
__device__ __forceinline__ void sum_colsq(const Args& a, int lane, float2& s1, float2& s2) {
    float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;
    for (int64_t j = lane; j < a.n; j += 32) {
        const float4 v = a.colsq[j];
        ff_acc(h1, l1, v.x, v.y);
        ff_acc(h2, l2, v.z, v.w);
    }
    s1 = ff_warp_sum(h1, l1);
    s2 = ff_warp_sum(h2, l2);
}

// Raw rows of M src (src float-float, n): warps 1..W-1, one warp per row;
// the raw value goes to dst[i] and is rescaled by the same lane later.
__device__ void trmv_rows_raw(const Args& a, const float2* src, float2* dst, int warp, int lane) {
    const int64_t n = a.n;
    const int64_t nw = (int64_t)gridDim.x * (W - 1);
    for (int64_t i = (int64_t)blockIdx.x * (W - 1) + (warp - 1); i < n; i += nw) {
        float2 s;
        if (a.MtF) {
            float h = 0.f, l = 0.f;
            const float2* row = a.MtF + i * n;
            for (int64_t j = i + lane; j < n; j += 32) {
                const float2 mv = row[j], xv = src[j];
                ff_madd(mv.x, mv.y, xv.x, xv.y, h, l);
            }
            s = ff_warp_sum(h, l);
        } else {
            s = src[i];
        }
        if (lane == 0) dst[i] = s;
    }
}

__device__ void scale_rows(const Args& a, float2* dst, float2 sc, int warp, int lane) {
    const int64_t nw = (int64_t)gridDim.x * (W - 1);
    if (lane != 0) return;
    for (int64_t i = (int64_t)blockIdx.x * (W - 1) + (warp - 1); i < a.n; i += nw) dst[i] = ff_mul(dst[i], sc);
}

__device__ __forceinline__ double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

// Lane-parallel reciprocal square roots: lane k returns rsqrt of its own
// argument (0 for a non-positive one); the caller shuffles the results out.
__device__ __forceinline__ double lane_rsqrt(double arg) { return arg > 0.0 ? rsqrt(arg) : 0.0; }

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

template <int KP, int RW>
__global__ void __launch_bounds__(T, 1) lsqr_ff_kernel(Args a) {
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ __align__(8) uint64_t full[ST];
    __shared__ Bcast bc;
    __shared__ int err_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t n = a.n;
    const int64_t G = gridDim.x;
    const double eps = 2.220446049250313e-16;
    const double dampsq = a.damp * a.damp;

    Ring rg;
    rg.full = full;
    rg.tiles = reinterpret_cast<float4*>(dsm);
    rg.cnt = 0;
    rg.issued = 0;
    rg.ntl = (blockIdx.x < a.ntiles) ? (a.ntiles - blockIdx.x + G - 1) / G : 0;
    ulonglong2* usm = reinterpret_cast<ulonglong2*>(dsm + (size_t)ST * a.R * a.ldf * 8);
    volatile int* err = &err_s;
    if (tid == 0) {
        err_s = 0;
        for (int s = 0; s < ST; ++s) mbar_init(&full[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        ring_issue(a, rg);
    }
    __syncthreads();

#define LSFF_SYNC()                    \
    do {                               \
        if (!grid_sync(a.bar)) {       \
            ring_drain(rg);            \
            return;                    \
        }                              \
    } while (0)
#define LSFF_PASS(...)                                             \
    do {                                                           \
        if (!ff_pass<KP, RW>(a, rg, usm, __VA_ARGS__, err)) {      \
            set_status(a, KSTATUS_BARRIER_TIMEOUT);                \
            ring_drain(rg);                                        \
            return;                                                \
        }                                                          \
    } while (0)

    const int64_t gt = (int64_t)blockIdx.x * T + tid;
    const int64_t gthreads = G * T;
    const float2 zero2 = make_float2(0.f, 0.f), one2 = make_float2(1.f, 0.f), mone2 = make_float2(-1.f, 0.f);

    // ---- initialisation (solvers.rs:141-182) ----
    for (int64_t j = gt; j < n; j += gthreads) {
        a.xF[j] = a.x0F ? a.x0F[j] : zero2;
        a.wF[j] = zero2;
        a.vF[j] = zero2;
        if (a.calc_var) a.varF[j] = zero2;
    }
    if (a.x0F) {
        if (warp > 0) trmv_rows_raw(a, a.x0F, a.yF, warp, lane);
        LSFF_SYNC();
    }
    // u = b - A M x0 (or b); beta^2, ||b||^2, A^T u partials
    LSFF_PASS(a.x0F ? mone2 : zero2, zero2, one2, a.x0F != nullptr, nullptr, a.bF, a.uF, true, true);
    LSFF_SYNC();

    // warp 0 keeps the scalar state (all lanes identical)
    double alfa = 0, beta = 0, bnorm = 0, ibn = 0, us = 0;
    if (warp == 0) {
        const float2 S = sum_slot(a, 0, lane);
        const float2 B2 = sum_slot(a, 3, lane);
        const double Sd = ff_to_double(S), B2d = ff_to_double(B2);
        const double r = lane_rsqrt(lane == 0 ? Sd : B2d);
        const double ib = shfl_d(r, 0);
        ibn = shfl_d(r, 1);
        beta = Sd * ib;
        bnorm = B2d * ibn;
        us = ib;
        if (lane == 0) {
            bc.ib = ff_split(ib);
            bc.beta = ff_split(beta);
        }
    } else {
        reduce_columns(a, warp, lane);
    }
    LSFF_SYNC();
    update_vun(a, bc, false, warp, lane);
    LSFF_SYNC();
    if (warp == 0) {
        float2 A2, W2;
        sum_colsq(a, lane, A2, W2);
        const double A2d = ff_to_double(A2);
        const double ia = lane_rsqrt(A2d);
        alfa = A2d * ia;
        if (lane == 0) bc.ia = ff_split(ia);
    } else {
        trmv_rows_raw(a, a.vunF, a.yF, warp, lane);
    }
    __syncthreads();
    if (warp > 0) {
        scale_rows(a, a.yF, bc.ia, warp, lane);
        for (int64_t j = (int64_t)blockIdx.x * (T - 32) + (tid - 32); j < n; j += G * (T - 32)) {
            const float2 vv = ff_mul(a.vunF[j], bc.ia);
            a.vF[j] = vv;
            a.wF[j] = vv;
        }
    }
    // all lanes of warp 0 hold the scalars; publish what the exit test needs
    if (warp == 0 && lane == 0) bc.istop = (alfa * beta == 0.0) ? -1 : 0;
    LSFF_SYNC();
    if (bc.istop == -1) {
        if (gt == 0) {
            const double bb = (double)bc.beta.x + (double)bc.beta.y;
            a.out[0] = 0; a.out[1] = 0; a.out[2] = bb; a.out[3] = bb;
            a.out[4] = 0; a.out[5] = 0; a.out[6] = 0; a.out[7] = 0;
            if (a.arn) a.arn[0] = 0.0;
        }
        for (int64_t j = gt; j < n; j += gthreads) {
            a.x[j] = ff_to_double(a.xF[j]);
            if (a.calc_var && a.var) a.var[j] = 0.0;
        }
        ring_drain(rg);
        return;
    }

    double rhobar = alfa, phibar = beta, rnorm = beta, r1norm = beta, r2norm = beta;
    double anorm = 0.0, acond = 0.0, ddnorm = 0.0, res2 = 0.0, xnorm = 0.0, xxnorm = 0.0, z = 0.0;
    double cs2 = -1.0, sn2 = 0.0;
    double arnorm = alfa * beta;
    double rho = 0, irho = 0, c = 0, s = 0, phi = 0, tau = 0, psi = 0;
    int beta_pos = 1;
    const double ctol = a.conlim > 0.0 ? 1.0 / a.conlim : 0.0;
    int64_t itn = 0;
    int istop = 0;
    if (warp == 0 && lane == 0) bc.c2 = ff_split(-alfa * us);
    __syncthreads();

    while (itn < a.iter_lim) {
        if (gt == 0 && a.arn) a.arn[itn] = arnorm;
        ++itn;
        // u = A M v - alfa u (u stored unnormalised); A^T u partials (solvers.rs:194-195)
        {
            const float2 c2 = bc.c2;
            LSFF_PASS(one2, c2, zero2, true, a.uF, nullptr, a.uF, false, true);
        }
        LSFF_SYNC();
        if (warp == 0) {
            // beta, the first plane rotation and phi, tau, t1 need only beta (solvers.rs:196-216)
            const float2 S = sum_slot(a, 0, lane);
            const double Sd = ff_to_double(S);
            beta_pos = Sd > 0.0;
            const double rb2 = rhobar * rhobar + dampsq;
            const double an2 = anorm * anorm + alfa * alfa + Sd + dampsq;
            const double arg = lane == 0 ? Sd : lane == 1 ? rb2 + Sd : lane == 2 ? rb2 : an2;
            const double r = lane_rsqrt(arg);
            const double ib = shfl_d(r, 0);
            irho = shfl_d(r, 1);
            const double irb1 = shfl_d(r, 2);
            const double ian = shfl_d(r, 3);
            beta = Sd * ib;
            if (beta_pos) {
                us = ib;
                anorm = an2 * ian;
            }
            double rhobar1, cs1, sn1;
            if (dampsq == 0.0) {
                rhobar1 = fabs(rhobar);
                cs1 = sgn(rhobar);
                sn1 = 0.0;
            } else {
                rhobar1 = rb2 * irb1;
                cs1 = rhobar * irb1;
                sn1 = a.damp * irb1;
            }
            psi = sn1 * phibar;
            phibar *= cs1;
            rho = (rb2 + Sd) * irho;
            c = rhobar1 * irho;
            s = beta * irho;
            phi = c * phibar;
            phibar = s * phibar;
            tau = s * phi;
            if (lane == 0) {
                bc.ib = ff_split(ib);
                bc.beta = ff_split(beta);
                bc.beta_pos = beta_pos;
                bc.t1 = ff_split(phi * irho);
                bc.irho = ff_split(irho);
            }
        } else {
            reduce_columns(a, warp, lane);
        }
        LSFF_SYNC();
        // v = M^T A^T u / beta - beta v  (solvers.rs:197-204)
        if (bc.beta_pos) update_vun(a, bc, true, warp, lane);
        else {
            // keep v; ||w||^2 is still needed
            for (int64_t j = gt; j < n; j += gthreads) {
                const float2 wj = a.wF[j];
                float q2h = 0.f, q2l = 0.f;
                ff_madd(wj.x, wj.y, wj.x, wj.y, q2h, q2l);
                const float2 q2 = ff_norm(q2h, q2l);
                a.colsq[j] = make_float4(0.f, 0.f, q2.x, q2.y);
            }
        }
        LSFF_SYNC();
        const bool bp = bc.beta_pos != 0;
        double wsq = 0.0;
        if (warp == 0) {
            float2 A2, W2;
            sum_colsq(a, lane, A2, W2);
            wsq = ff_to_double(W2);
            if (bp) {
                const double A2d = ff_to_double(A2);
                const double ia = lane_rsqrt(A2d);
                alfa = A2d * ia;
                if (lane == 0) bc.ia = ff_split(ia);
            }
            const double theta = s * alfa;
            rhobar = -c * alfa;
            if (lane == 0) {
                bc.t2 = ff_split(-theta * irho);
                bc.c2 = ff_split(-alfa * us);
            }
        } else if (bp) {
            trmv_rows_raw(a, a.vunF, a.yF, warp, lane);
        }
        __syncthreads();
        if (warp > 0) {
            // x += t1 w ; w = v + t2 w ; var += (w / rho)^2 ; y = M v  (solvers.rs:222-232)
            if (bp) scale_rows(a, a.yF, bc.ia, warp, lane);
            const float2 t1 = bc.t1, t2 = bc.t2, ia = bc.ia, ir = bc.irho;
            for (int64_t j = (int64_t)blockIdx.x * (T - 32) + (tid - 32); j < n; j += G * (T - 32)) {
                const float2 vv = bp ? ff_mul(a.vunF[j], ia) : a.vF[j];
                const float2 wj = a.wF[j];
                a.vF[j] = vv;
                a.xF[j] = ff_fma(t1, wj, a.xF[j]);
                a.wF[j] = ff_fma(t2, wj, vv);
                if (a.calc_var) {
                    const float2 dk = ff_mul(wj, ir);
                    a.varF[j] = ff_fma(dk, dk, a.varF[j]);
                }
            }
        } else {
            // norm estimates and stopping tests (solvers.rs:235-272)
            const double theta = s * alfa;
            ddnorm += wsq * irho * irho;
            const double delta = sn2 * rho;
            const double gambar = -cs2 * rho;
            const double rhs = phi - delta * z;
            res2 += psi * psi;
            const double rn2 = phibar * phibar + res2;
            const double g2 = gambar * gambar + theta * theta;
            const double arg1 = lane == 0 ? g2 : lane == 1 ? gambar * gambar : lane == 2 ? ddnorm : rn2;
            const double r1 = lane_rsqrt(arg1);
            const double igamma = shfl_d(r1, 0);
            const double igb = shfl_d(r1, 1);
            const double idd = shfl_d(r1, 2);
            const double irn = shfl_d(r1, 3);
            const double zbar = rhs * igb * sgn(gambar);
            cs2 = gambar * igamma;
            sn2 = theta * igamma;
            z = rhs * igamma;
            const double xn2 = xxnorm + zbar * zbar;
            xxnorm += z * z;
            acond = anorm * (ddnorm * idd);
            rnorm = rn2 * irn;
            arnorm = alfa * fabs(tau);
            const double r1sq = rnorm * rnorm - dampsq * xxnorm;
            const double arg2 = lane == 0 ? xn2 : fabs(r1sq);
            const double r2 = lane_rsqrt(arg2);
            xnorm = xn2 * shfl_d(r2, 0);
            r1norm = fabs(r1sq) * shfl_d(r2, 1);
            r2norm = rnorm;
            const double test1 = rnorm * ibn;
            const double axb = anorm * xnorm * ibn;
            const double arg3 = lane == 0 ? anorm * rnorm + eps : lane == 1 ? acond + eps : 1.0 + axb;
            const double r3 = lane_rsqrt(arg3);
            const double q0 = shfl_d(r3, 0), q1 = shfl_d(r3, 1), q2 = shfl_d(r3, 2);
            const double test2 = arnorm * (q0 * q0);
            const double test3 = q1 * q1;
            const double tt1 = test1 * (q2 * q2);
            const double rtol = a.atol + a.btol * axb;
            istop = 0;
            if (itn >= a.iter_lim) istop = 7;
            if (1.0 + test3 <= 1.0) istop = 6;
            if (1.0 + test2 <= 1.0) istop = 5;
            if (1.0 + tt1 <= 1.0) istop = 4;
            if (test3 <= ctol) istop = 3;
            if (test2 <= a.atol) istop = 2;
            if (test1 <= rtol) istop = 1;
            if (a.abs_tol > 0.0 && arnorm < a.abs_tol && (istop == 0 || istop == 7)) istop = 2;
            if (lane == 0) bc.istop = istop;
        }
        LSFF_SYNC();
        if (bc.istop != 0) break;
    }
    for (int64_t j = gt; j < n; j += gthreads) {
        a.x[j] = ff_to_double(a.xF[j]);
        if (a.calc_var && a.var) a.var[j] = ff_to_double(a.varF[j]);
    }
    if (gt == 0) {
        a.out[0] = istop; a.out[1] = (double)itn; a.out[2] = r1norm; a.out[3] = r2norm;
        a.out[4] = anorm; a.out[5] = acond; a.out[6] = xnorm; a.out[7] = arnorm;
    }
    ring_drain(rg);
#undef LSFF_SYNC
#undef LSFF_PASS
}

// Row-major float-float copy in column-pair order: row i is hp = ldf / 2
// chunks of 16 bytes, chunk p = (hi_2p, hi_2p+1, lo_2p, lo_2p+1); zero for
// columns in [n, ldf).  32 x 32 tiles through shared memory.
__global__ void rowmajor_split_kernel(const double* __restrict__ A, int64_t m, int64_t n, int64_t lda,
                                      float* __restrict__ AF, int64_t ldf) {
    __shared__ float2 tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int64_t i = i0 + threadIdx.x, j = j0 + k;
        float2 v = make_float2(0.f, 0.f);
        if (i < m && j < n) v = ff_split(A[i + j * lda]);
        tile[k][threadIdx.x] = v;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int64_t i = i0 + k, j = j0 + threadIdx.x;
        if (i < m && j < ldf) {
            const float2 v = tile[threadIdx.x][k];
            float* row = AF + i * 2 * ldf + 4 * (j >> 1) + (j & 1);
            row[0] = v.x;
            row[2] = v.y;
        }
    }
}

__global__ void vec_split_kernel(const double* __restrict__ v, int64_t n, float2* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = ff_split(v[i]);
}

// MF = split(M) (column-major, upper part), MtF = its transpose.
__global__ void msplit_kernel(const double* __restrict__ M, int64_t n, int64_t ldm, float2* __restrict__ MF,
                              float2* __restrict__ MtF) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        const float2 v = (i <= j) ? ff_split(M[i + j * ldm]) : make_float2(0.f, 0.f);
        MF[i + j * n] = v;
        MtF[j + i * n] = v;
    }
}

template <int KP, int RW>
static const void* kernel_kp() { return (const void*)lsqr_ff_kernel<KP, RW>; }

// (kernel, rows per warp) for hp column pairs: the y registers cover hp, and
// a tile of 8 RW rows stays within 64 KB.
static const void* pick_kernel(int64_t hp, int& RW) {
    if (hp <= 32) { RW = 4; return kernel_kp<1, 4>(); }
    if (hp <= 64) { RW = 4; return kernel_kp<2, 4>(); }
    if (hp <= 128) { RW = 2; return kernel_kp<4, 2>(); }
    if (hp <= 256) { RW = 2; return kernel_kp<8, 2>(); }
    RW = 1;
    return kernel_kp<16, 1>();
}

}  // namespace lsff

bool lsqr_ff_supported(int64_t n) { return n >= 1 && n <= lsff::MAX_N; }

LsqrResult lsqr_ff_solve(Ctx& ctx, const double* A, int64_t m, int64_t n, int64_t lda, const double* M,
                         const double* b, const double* x0, const LsqrParams& prm, double* x, double* var,
                         double* arnorms_dev) {
    using namespace lsff;
    if (!lsqr_ff_supported(n)) fail(RNLA_ERR_UNSUPPORTED, "lsqr (float-float): n must be in [1, 1024]");
    cudaStream_t st = ctx.stream;
    const int64_t ldf = (n + 1) & ~1LL;
    const int64_t hp = ldf / 2;
    int RW = 1;
    const void* k = pick_kernel(hp, RW);
    const int R = W * RW;
    const size_t smem = (size_t)ST * R * ldf * 8 + (size_t)R * 16;
    if (smem > 48 * 1024)
        RNLA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, T, smem));
    if (nb < 1) fail(RNLA_ERR_UNSUPPORTED, "lsqr (float-float): kernel does not fit on an SM");
    if (nb > 2) nb = 2;
    const int G = nb * ctx.sm_count;

    DevBuf<float2> AF, MF, MtF, bF, x0F, uF, yF, gF, vF, wF, xF, vunF, varF, partF, spF;
    DevBuf<float4> colsq;
    DevBuf<double> out;
    DevBuf<unsigned int> bar;
    AF.alloc((size_t)m * ldf, st);
    bF.alloc(m, st);
    uF.alloc(m, st);
    yF.alloc(ldf, st);
    gF.alloc(n, st); vF.alloc(n, st); wF.alloc(n, st); xF.alloc(n, st); vunF.alloc(n, st); varF.alloc(n, st);
    partF.alloc((size_t)G * ldf, st);
    spF.alloc((size_t)G * 4, st);
    colsq.alloc(n, st);
    out.alloc(8, st);
    bar.alloc(2, st);
    RNLA_CUDA(cudaMemsetAsync(bar.get(), 0, 2 * sizeof(unsigned int), st));
    RNLA_CUDA(cudaMemsetAsync(out.get(), 0, 8 * sizeof(double), st));
    RNLA_CUDA(cudaMemsetAsync(yF.get(), 0, ldf * sizeof(float2), st));
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), st));
    {
        dim3 grid((unsigned)div_up(m, 32), (unsigned)div_up(ldf, 32));
        rowmajor_split_kernel<<<grid, dim3(32, 8), 0, st>>>(A, m, n, lda, reinterpret_cast<float*>(AF.get()), ldf);
        RNLA_LAUNCH_CHECK();
        int g = (int)div_up(m, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        vec_split_kernel<<<g, 256, 0, st>>>(b, m, bF);
        RNLA_LAUNCH_CHECK();
    }
    Args a{};
    if (M) {
        MF.alloc((size_t)n * n, st);
        MtF.alloc((size_t)n * n, st);
        int g = (int)div_up(n * n, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        msplit_kernel<<<g, 256, 0, st>>>(M, n, n, MF, MtF);
        RNLA_LAUNCH_CHECK();
        a.MF = MF.get();
        a.MtF = MtF.get();
    }
    if (x0) {
        x0F.alloc(n, st);
        vec_split_kernel<<<(unsigned)div_up(n, 256), 256, 0, st>>>(x0, n, x0F);
        RNLA_LAUNCH_CHECK();
        a.x0F = x0F.get();
    }
    a.AF = AF.get(); a.m = m; a.n = n; a.ldf = ldf; a.hp = hp; a.R = R; a.ntiles = div_up(m, R);
    a.bF = bF.get();
    a.uF = uF.get(); a.yF = yF.get(); a.gF = gF.get(); a.vF = vF.get(); a.wF = wF.get(); a.xF = xF.get();
    a.vunF = vunF.get(); a.varF = varF.get(); a.partF = partF.get(); a.spF = spF.get(); a.colsq = colsq.get();
    a.x = x; a.var = var; a.arn = arnorms_dev; a.out = out.get();
    a.damp = prm.damp; a.atol = prm.atol; a.btol = prm.btol; a.conlim = prm.conlim;
    a.abs_tol = prm.abs_arnorm_tol;
    a.iter_lim = prm.iter_lim < 0 ? 2 * n : prm.iter_lim;
    a.calc_var = (prm.calc_var && var) ? 1 : 0;
    a.bar.count = bar.get(); a.bar.gen = bar.get() + 1; a.bar.status = ctx.status;
    void* params[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3(G), dim3(T), params, smem, st));
    count_launch();
    double h[8];
    RNLA_CUDA(cudaMemcpyAsync(h, out.get(), sizeof h, cudaMemcpyDeviceToHost, st));
    ctx.check_status("lsqr");
    LsqrResult r;
    r.istop = (int64_t)h[0]; r.itn = (int64_t)h[1];
    r.r1norm = h[2]; r.r2norm = h[3]; r.anorm = h[4]; r.acond = h[5]; r.xnorm = h[6]; r.arnorm = h[7];
    return r;
}

}  // namespace rnla
