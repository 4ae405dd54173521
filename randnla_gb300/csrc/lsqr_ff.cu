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
// through a ring of ST stages (up to 192 KB) that runs continuously across
// passes -- A never changes -- so the first tiles of the next pass are in
// flight while the grid is between passes.
//
// One pass (512 threads, two warp roles working on consecutive tiles):
//   row warps 0-7     tile k: warp w forms t_r = (A y)_r for rows
//                     r = w + 8 s (s < RW): 16-byte chunks of the row, y in
//                     registers, exact FMA products summed with TwoSum on
//                     packed pairs, a warp reduce-scatter over the RW rows;
//                     one lane per row forms
//                     u_r = c1 t_r + c2 u_r + c3 b_r, accumulates ||u||^2 and
//                     hands u to the column warps (double-buffered, named
//                     barriers: bar.arrive "u ready", bar.sync "u consumed");
//   column warps 8-15 tile k - 1: thread t owns the column pairs t + 256 q
//                     and accumulates A^T u over the tile's rows, then frees
//                     the ring stage and issues the next bulk copy.
// Both roles read 512 contiguous bytes per warp instruction (no bank
// conflicts).  Per-CTA partials are summed in a fixed order, so the run is
// reproducible.
//
// Arithmetic.  Every vector operation is float-float on the FP32 pipe.  FP64
// is used only by warp 0 of each CTA for the scalar recurrences (state kept
// in shared memory): on GB300 a dependent FP64 operation takes ~64 cycles and
// a divide or square root several hundred, so the recurrences are arranged as
// a few lane-parallel rsqrt steps (different lanes of one warp instruction
// evaluate independent reciprocal square roots) plus multiplies; divisions
// become products with those reciprocals.  Results agree with the FP64 LSQR
// to float-float accuracy, and the iteration count can differ by one at a
// tolerance boundary.
//
// Waits are bounded: the grid barrier and the tile mbarriers give up after
// 2 s and record a status; the named-barrier hand-offs still run to the end
// of the pass (no role leaves early), then the CTA lets its own bulk copies
// land and returns.
#include "rnla_internal.h"
#include "rnla_ff.cuh"
#include "rnla_async.cuh"

namespace rnla {
namespace lsff {

constexpr int T = 512;          // threads per CTA (split roles)
constexpr int W = T / 32;       // warps per CTA
constexpr int WA = 8;           // row warps (0..7); warps 8..15 are column warps
constexpr int TB = T - 32 * WA; // column threads
constexpr int TF = 256;         // threads per CTA (fused roles)
constexpr int WF = TF / 32;
constexpr int MAX_ST = 6;       // ring stages
constexpr size_t RING_BYTES = 192 * 1024;
constexpr int64_t MAX_N = 1024;
// named barriers (0 is __syncthreads)
constexpr int NB_URDY = 1;      // + (k & 1): u of tile k written
constexpr int NB_UFREE = 3;     // + (k & 1): u of tile k consumed

struct Args {
    const float2* AF;           // row-major copy of A, m rows of rowq 16-byte chunks
    int64_t m, n, ldf, hp;      // hp = ldf / 2 column pairs
    int64_t rowq;               // 16-byte chunks per row: hp (float-float rows) or ldf / 4 (FP32 rows)
    int nparts;                 // rows of partF: one per CTA, or one per warp (FP32-row passes)
    int R;                      // rows per tile (multiple of 8)
    int ST;                     // ring stages
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

// Scalar state of the recurrences (warp 0).
struct Scal {
    double alfa, beta, bnorm, ibn, us;
    double rhobar, phibar, rnorm, r1norm, r2norm, anorm, acond, ddnorm, res2, xnorm, xxnorm, z, cs2, sn2, arnorm;
    double rho, irho, c, s, phi, tau, psi;
    int istop;
};

// Tile ring.  Every thread tracks the stage and mbarrier phase of the next
// tile to consume; the issuing thread also tracks the next stage to fill, the
// next tile (index into this CTA's tile list) and the copies in flight.  All
// counters advance by increment and wrap: no integer division in the loop.
struct Ring {
    uint64_t* full;             // ST mbarriers
    float4* tiles;              // ST stages of R x hp float4
    int64_t ntl;                // tiles of this CTA per pass
    int cst;                    // stage of the next tile to consume
    uint32_t cph;               // its phase parity
    int ist;                    // issuer: next stage to fill
    int64_t ik;                 // issuer: next tile index (0..ntl-1)
    int inflight;               // issuer: issued and not yet consumed
    // fused roles: per-stage release counters and the number of copies
    // issued so far (shared memory); tiles consumed so far (every thread)
    unsigned int* rel;
    unsigned long long* issued;
    unsigned long long consumed;
};

constexpr int ISSUER = 32 * WA;  // first column thread issues the bulk copies

__device__ __forceinline__ void nb_sync(int id) { asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(T) : "memory"); }
__device__ __forceinline__ void nb_arrive(int id) { asm volatile("bar.arrive %0, %1;" ::"r"(id), "n"(T) : "memory"); }

__device__ __forceinline__ void ring_issue(const Args& a, Ring& rg) {
    if (rg.ntl == 0) return;
    while (rg.inflight < a.ST) {
        const int64_t t = (int64_t)blockIdx.x + rg.ik * (int64_t)gridDim.x;
        const int64_t r0 = t * a.R;
        const int64_t rows = min((int64_t)a.R, a.m - r0);
        const uint32_t bytes = (uint32_t)(rows * a.rowq * 16);
        mbar_expect_tx(&rg.full[rg.ist], bytes);
        bulk_g2s(rg.tiles + (size_t)rg.ist * a.R * a.rowq, reinterpret_cast<const float4*>(a.AF) + r0 * a.rowq,
                 bytes, &rg.full[rg.ist]);
        rg.ist = (rg.ist + 1 == a.ST) ? 0 : rg.ist + 1;
        rg.ik = (rg.ik + 1 == rg.ntl) ? 0 : rg.ik + 1;
        ++rg.inflight;
    }
}

__device__ __forceinline__ void ring_advance(const Args& a, Ring& rg) {
    if (++rg.cst == a.ST) { rg.cst = 0; rg.cph ^= 1u; }
    ++rg.consumed;
}

// One bulk copy of this CTA's tile `ik` into stage `st`.
__device__ __forceinline__ void ring_copy(const Args& a, const Ring& rg, int st, int64_t ik) {
    const int64_t t = (int64_t)blockIdx.x + ik * (int64_t)gridDim.x;
    const int64_t r0 = t * a.R;
    const int64_t rows = min((int64_t)a.R, a.m - r0);
    const uint32_t bytes = (uint32_t)(rows * a.rowq * 16);
    mbar_expect_tx(&rg.full[st], bytes);
    bulk_g2s(rg.tiles + (size_t)st * a.R * a.rowq, reinterpret_cast<const float4*>(a.AF) + r0 * a.rowq, bytes,
             &rg.full[st]);
}

// Fused roles: the stage a warp has just read into registers is released
// by lane 0; the last of the WF warps refills it with the tile ST places
// further along this CTA's (cyclic) tile list.  Every thread tracks that
// tile index in rg.ik.  Stages are released in order because every warp
// reads the tiles in order.
__device__ __forceinline__ void ring_release(const Args& a, Ring& rg, int st, int lane, volatile int* err,
                                             int nwarps = WF) {
    __syncwarp();
    if (lane == 0) {
        __threadfence_block();
        if (atomicAdd(&rg.rel[st], 1u) == (unsigned)(nwarps - 1)) {
            rg.rel[st] = 0;
            if (*err == 0) {
                __threadfence_block();
                fence_proxy_async();
                ring_copy(a, rg, st, rg.ik);
                atomicAdd(rg.issued, 1ull);
            }
        }
    }
    rg.ik = (rg.ik + 1 == rg.ntl) ? 0 : rg.ik + 1;
}

// Fused roles, thread 0: wait (bounded) for every copy still in flight.
__device__ void ring_drain_fused(const Args& a, Ring& rg) {
    if (threadIdx.x != 0) return;
    volatile int quiet = 0;
    int st = rg.cst;
    uint32_t ph = rg.cph;
    const unsigned long long out = *rg.issued - rg.consumed;
    for (unsigned long long c = 0; c < out; ++c) {
        mbar_wait(&rg.full[st], ph, &quiet);
        if (++st == a.ST) { st = 0; ph ^= 1u; }
    }
}

// Issuing thread: wait (bounded) until every copy still in flight has
// landed, so the CTA can exit with no bulk copy writing into its shared
// memory.
__device__ void ring_drain(const Args& a, Ring& rg) {
    if (threadIdx.x != ISSUER) return;
    volatile int quiet = 0;
    int st = rg.cst;
    uint32_t ph = rg.cph;
    for (int c = 0; c < rg.inflight; ++c) {
        mbar_wait(&rg.full[st], ph, &quiet);
        if (++st == a.ST) { st = 0; ph ^= 1u; }
    }
}

__device__ __forceinline__ void set_status(const Args& a, unsigned int code) {
    atomicCAS(a.bar.status, 0u, code);
}

// One pass over the CTA's tiles:
//   dst_i = c1 (A y)_i + c2 old_i + c3 bvec_i     (A y skipped when !dot)
// accumulating sum dst_i^2 (spF slot 0), sum bvec_i^2 (slot 3, want_b2) and,
// when acc_at, the CTA's partial of A^T dst into partF.  Returns false if a
// tile wait failed (after completing the hand-off protocol).
template <int KP, int RW>
__device__ bool ff_pass(const Args& a, Ring& rg, ulonglong2* usm, float2 c1, float2 c2, float2 c3, bool dot,
                        const float2* oldv, const float2* bvec, float2* dst, bool want_b2, bool acc_at,
                        volatile int* err) {
    constexpr int R = WA * RW;
    __shared__ float2 wred[WA][2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int hp = (int)a.hp;
    const int64_t ntl = rg.ntl;
    if (warp < WA) {
        // ---------------- row warps ----------------
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
        float sqh = 0.f, sql = 0.f, b2h = 0.f, b2l = 0.f;
        // After the reduce-scatter below, lane l holds the sum of row slot
        // l >> SHL; the first lane of each group (owner) forms that row's u.
        // Its old value and b are loaded two tiles ahead (the loads sit
        // behind the streaming).
        constexpr int SHL = (RW == 1) ? 5 : (RW == 2) ? 4 : (RW == 4) ? 3 : 2;
        const bool owner = (lane & ((1 << SHL) - 1)) == 0;
        const int rw = lane >> SHL;                      // row slot of an owner lane
        auto row_of = [&](int64_t kk) { return ((int64_t)blockIdx.x + kk * (int64_t)gridDim.x) * R + warp + WA * rw; };
        auto fetch = [&](int64_t kk, float2& u, float2& bv) {
            u = make_float2(0.f, 0.f);
            bv = make_float2(0.f, 0.f);
            if (owner && kk < ntl) {
                const int64_t i = row_of(kk);
                if (i < a.m) {
                    if (oldv) u = oldv[i];
                    if (bvec) bv = bvec[i];
                }
            }
        };
        float2 qu0, qb0, qu1, qb1;
        fetch(0, qu0, qb0);
        fetch(1, qu1, qb1);
#pragma unroll 1
        for (int64_t k = 0; k < ntl; ++k) {
            const float2 uo = qu0, bb = qb0;
            qu0 = qu1;
            qb0 = qb1;
            fetch(k + 2, qu1, qb1);
            const int st = rg.cst;
            const bool ok = mbar_wait(&rg.full[st], rg.cph, err);
            ring_advance(a, rg);
            const int64_t t = (int64_t)blockIdx.x + k * (int64_t)gridDim.x;
            const int64_t r0 = t * R;
            const int rows = (int)min((int64_t)R, a.m - r0);
            const ulonglong2* tile = reinterpret_cast<const ulonglong2*>(rg.tiles) + (size_t)st * R * hp;
            const bool mine = owner && warp + WA * rw < rows;
            float tvh[RW], tvl[RW];
#pragma unroll
            for (int w = 0; w < RW; ++w) { tvh[w] = 0.f; tvl[w] = 0.f; }
            if (dot && ok) {
                f32x2 sh[RW][2], sl[RW][2];
#pragma unroll
                for (int w = 0; w < RW; ++w) { sh[w][0] = sh[w][1] = sl[w][0] = sl[w][1] = 0ull; }
#pragma unroll
                for (int kk = 0; kk < KP; ++kk) {
                    const int p = lane + 32 * kk;
                    if (p < hp) {
#pragma unroll
                        for (int w = 0; w < RW; ++w) {
                            const ulonglong2 v = tile[(size_t)(warp + WA * w) * hp + p];
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
                // reduce-scatter: each exchange level halves the rows a lane
                // keeps (lanes with the level's bit set keep the upper half)
                int off = 16;
#pragma unroll
                for (int half = RW / 2; half >= 1; half /= 2) {
                    const bool up = (lane & off) != 0;
#pragma unroll
                    for (int k2 = 0; k2 < half; ++k2) {
                        const float sh_ = up ? tvh[k2] : tvh[k2 + half], sl_ = up ? tvl[k2] : tvl[k2 + half];
                        float kh = up ? tvh[k2 + half] : tvh[k2], kl = up ? tvl[k2 + half] : tvl[k2];
                        const float rh = __shfl_xor_sync(0xffffffffu, sh_, off);
                        const float rl = __shfl_xor_sync(0xffffffffu, sl_, off);
                        ff_acc(kh, kl, rh, rl);
                        tvh[k2] = kh;
                        tvl[k2] = kl;
                    }
                    off >>= 1;
                }
                for (; off >= 1; off >>= 1) {
                    const float oh = __shfl_xor_sync(0xffffffffu, tvh[0], off);
                    const float ol = __shfl_xor_sync(0xffffffffu, tvl[0], off);
                    ff_acc(tvh[0], tvl[0], oh, ol);
                }
            }
            float2 nv = make_float2(0.f, 0.f);
            int r = 0;
            if (mine) {
                const float th = tvh[0], tl = tvl[0];
                r = warp + WA * rw;
                const float2 tv = ff_norm(th, tl);
                nv = ff_add(ff_add(ff_mul(c1, tv), ff_mul(c2, uo)), ff_mul(c3, bb));
            }
            if (k >= 2) nb_sync(NB_UFREE + (int)(k & 1));        // column warps are done with this u buffer
            if (mine && ok) {
                dst[r0 + r] = nv;
                usm[(k & 1) * R + r] = make_ulonglong2(pk2(nv.x, nv.x), pk2(nv.y, nv.y));
                ff_madd(nv.x, nv.y, nv.x, nv.y, sqh, sql);
                if (want_b2) ff_madd(bb.x, bb.y, bb.x, bb.y, b2h, b2l);
            }
            nb_arrive(NB_URDY + (int)(k & 1));
        }
        for (int64_t k = (ntl >= 2 ? ntl - 2 : 0); k < ntl; ++k) nb_sync(NB_UFREE + (int)(k & 1));
        const float2 sq = ff_warp_sum(sqh, sql);
        const float2 b2 = ff_warp_sum(b2h, b2l);
        if (lane == 0) { wred[warp][0] = sq; wred[warp][1] = b2; }
    } else {
        // ---------------- column warps ----------------
        const int tb = tid - 32 * WA;
        constexpr int CH = (KP >= 16) ? 2 : 4;   // independent accumulation chains (rows mod CH)
        constexpr int QP = (KP >= 16) ? 2 : 1;   // column pairs per thread
        f32x2 ah[QP][CH], al[QP][CH];
#pragma unroll
        for (int q = 0; q < QP; ++q)
#pragma unroll
            for (int c = 0; c < CH; ++c) { ah[q][c] = 0ull; al[q][c] = 0ull; }
#pragma unroll 1
        for (int64_t k = 0; k < ntl; ++k) {
            const int st = rg.cst;
            const bool ok = mbar_wait(&rg.full[st], rg.cph, err);
            ring_advance(a, rg);
            const int64_t t = (int64_t)blockIdx.x + k * (int64_t)gridDim.x;
            const int rows = (int)min((int64_t)R, a.m - t * R);
            const ulonglong2* tile = reinterpret_cast<const ulonglong2*>(rg.tiles) + (size_t)st * R * hp;
            const ulonglong2* ub = usm + (k & 1) * R;
            nb_sync(NB_URDY + (int)(k & 1));
            if (acc_at && ok) {
                int r = 0;
                for (; r + CH <= rows; r += CH) {
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        const ulonglong2 u = ub[r + c];
                        const f32x2 nu = neg2(u.x);
#pragma unroll
                        for (int q = 0; q < QP; ++q) {
                            const int p = tb + q * TB;
                            if (p < hp) {
                                const ulonglong2 v = tile[(size_t)(r + c) * hp + p];
                                ff2_madd(v.x, v.y, u.x, nu, u.y, ah[q][c], al[q][c]);
                            }
                        }
                    }
                }
                for (; r < rows; ++r) {
                    const ulonglong2 u = ub[r];
                    const f32x2 nu = neg2(u.x);
#pragma unroll
                    for (int q = 0; q < QP; ++q) {
                        const int p = tb + q * TB;
                        if (p < hp) {
                            const ulonglong2 v = tile[(size_t)r * hp + p];
                            ff2_madd(v.x, v.y, u.x, nu, u.y, ah[q][0], al[q][0]);
                        }
                    }
                }
            }
            nb_arrive(NB_UFREE + (int)(k & 1));
            if (tid == ISSUER) {
                --rg.inflight;
                ring_issue(a, rg);
            }
        }
        if (acc_at) {
            float4* P4 = reinterpret_cast<float4*>(a.partF) + (size_t)blockIdx.x * hp;
#pragma unroll
            for (int q = 0; q < QP; ++q) {
                const int p = tb + q * TB;
                if (p < hp) {
#pragma unroll
                    for (int c = 1; c < CH; ++c) ff2_acc(ah[q][0], al[q][0], ah[q][c], al[q][c]);
                    const float2 H = upk2(ah[q][0]), L = upk2(al[q][0]);
                    const float2 c0 = ff_norm(H.x, L.x), c1v = ff_norm(H.y, L.y);
                    P4[p] = make_float4(c0.x, c0.y, c1v.x, c1v.y);
                }
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        float h = 0.f, l = 0.f, h2 = 0.f, l2 = 0.f;
        for (int w = 0; w < WA; ++w) {
            ff_acc(h, l, wred[w][0].x, wred[w][0].y);
            ff_acc(h2, l2, wred[w][1].x, wred[w][1].y);
        }
        a.spF[blockIdx.x * 4 + 0] = ff_norm(h, l);
        a.spF[blockIdx.x * 4 + 3] = ff_norm(h2, l2);
    }
    return *err == 0;
}

// The same pass with fused roles (TF threads): each warp takes RW rows of
// every tile, loads their chunks into registers and releases the stage at
// once, forms the RW row dots (packed float-float, warp reduce-scatter), the
// owner lane of each row forms u_r, and after a broadcast every lane adds
// u_r times its chunks to its own A^T u accumulators (KP column pairs).  The
// WF per-warp accumulators are summed in warp order at the end of the pass
// through `scratch` (WF x hp float4).
template <int KP, int RW>
__device__ bool ff_pass_fused(const Args& a, Ring& rg, float4* scratch, float2 c1, float2 c2, float2 c3,
                              bool dot, const float2* oldv, const float2* bvec, float2* dst, bool want_b2,
                              bool acc_at, volatile int* err) {
    constexpr int R = WF * RW;
    __shared__ float2 wred[WF][2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int hp = (int)a.hp;
    const int64_t ntl = rg.ntl;
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
    f32x2 ah[KP], al[KP];
#pragma unroll
    for (int k = 0; k < KP; ++k) { ah[k] = 0ull; al[k] = 0ull; }
    float sqh = 0.f, sql = 0.f, b2h = 0.f, b2l = 0.f;
    // after the reduce-scatter lane l holds the dot of row slot l >> SHL; the
    // first lane of each group (owner) forms that row's u
    constexpr int SHL = (RW == 1) ? 5 : (RW == 2) ? 4 : (RW == 4) ? 3 : 2;
    const bool owner = (lane & ((1 << SHL) - 1)) == 0;
    const int rw = lane >> SHL;
    auto row_of = [&](int64_t kk) { return ((int64_t)blockIdx.x + kk * (int64_t)gridDim.x) * R + warp + WF * rw; };
    auto fetch = [&](int64_t kk, float2& u, float2& bv) {
        u = make_float2(0.f, 0.f);
        bv = make_float2(0.f, 0.f);
        if (owner && kk < ntl) {
            const int64_t i = row_of(kk);
            if (i < a.m) {
                if (oldv) u = oldv[i];
                if (bvec) bv = bvec[i];
            }
        }
    };
    float2 qu0, qb0, qu1, qb1;
    fetch(0, qu0, qb0);
    fetch(1, qu1, qb1);
#pragma unroll 1
    for (int64_t k = 0; k < ntl; ++k) {
        const float2 uo = qu0, bb = qb0;
        qu0 = qu1;
        qb0 = qb1;
        fetch(k + 2, qu1, qb1);
        const int st = rg.cst;
        const bool ok = mbar_wait(&rg.full[st], rg.cph, err);
        ring_advance(a, rg);
        const int64_t r0 = ((int64_t)blockIdx.x + k * (int64_t)gridDim.x) * R;
        const int rows = (int)min((int64_t)R, a.m - r0);
        const ulonglong2* tile = reinterpret_cast<const ulonglong2*>(rg.tiles) + (size_t)st * R * hp;
        ulonglong2 v[RW][KP];
#pragma unroll
        for (int w = 0; w < RW; ++w) {
            const int r = warp + WF * w;
            const bool rv = ok && r < rows;
#pragma unroll
            for (int kk = 0; kk < KP; ++kk) {
                const int p = lane + 32 * kk;
                v[w][kk] = (rv && p < hp) ? tile[(size_t)r * hp + p] : make_ulonglong2(0ull, 0ull);
            }
        }
        ring_release(a, rg, st, lane, err);
        float tvh[RW], tvl[RW];
#pragma unroll
        for (int w = 0; w < RW; ++w) { tvh[w] = 0.f; tvl[w] = 0.f; }
        if (dot) {
            f32x2 sh[RW][2], sl[RW][2];
#pragma unroll
            for (int w = 0; w < RW; ++w) { sh[w][0] = sh[w][1] = sl[w][0] = sl[w][1] = 0ull; }
#pragma unroll
            for (int kk = 0; kk < KP; ++kk) {
#pragma unroll
                for (int w = 0; w < RW; ++w)
                    ff2_madd(v[w][kk].x, v[w][kk].y, yh[kk], nyh[kk], yl[kk], sh[w][kk & 1], sl[w][kk & 1]);
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
            int off = 16;
#pragma unroll
            for (int half = RW / 2; half >= 1; half /= 2) {
                const bool up = (lane & off) != 0;
#pragma unroll
                for (int k2 = 0; k2 < half; ++k2) {
                    const float sh_ = up ? tvh[k2] : tvh[k2 + half], sl_ = up ? tvl[k2] : tvl[k2 + half];
                    float kh = up ? tvh[k2 + half] : tvh[k2], kl = up ? tvl[k2 + half] : tvl[k2];
                    const float rh = __shfl_xor_sync(0xffffffffu, sh_, off);
                    const float rl = __shfl_xor_sync(0xffffffffu, sl_, off);
                    ff_acc(kh, kl, rh, rl);
                    tvh[k2] = kh;
                    tvl[k2] = kl;
                }
                off >>= 1;
            }
            for (; off >= 1; off >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, tvh[0], off);
                const float ol = __shfl_xor_sync(0xffffffffu, tvl[0], off);
                ff_acc(tvh[0], tvl[0], oh, ol);
            }
        }
        float2 nv = make_float2(0.f, 0.f);
        if (owner) {
            const float2 tv = ff_norm(tvh[0], tvl[0]);
            nv = ff_add(ff_add(ff_mul(c1, tv), ff_mul(c2, uo)), ff_mul(c3, bb));
            const int r = warp + WF * rw;
            if (ok && r < rows) {
                dst[r0 + r] = nv;
                ff_madd(nv.x, nv.y, nv.x, nv.y, sqh, sql);
                if (want_b2) ff_madd(bb.x, bb.y, bb.x, bb.y, b2h, b2l);
            }
        }
        if (acc_at) {
            f32x2 uh[RW], nuh[RW], ul[RW];
#pragma unroll
            for (int w = 0; w < RW; ++w) {
                const float x = __shfl_sync(0xffffffffu, nv.x, w << SHL);
                const float y = __shfl_sync(0xffffffffu, nv.y, w << SHL);
                uh[w] = pk2(x, x);
                nuh[w] = pk2(-x, -x);
                ul[w] = pk2(y, y);
            }
#pragma unroll
            for (int kk = 0; kk < KP; ++kk) {
#pragma unroll
                for (int w = 0; w < RW; ++w) ff2_madd(v[w][kk].x, v[w][kk].y, uh[w], nuh[w], ul[w], ah[kk], al[kk]);
            }
        }
    }
    const float2 sq = ff_warp_sum(sqh, sql);
    const float2 b2 = ff_warp_sum(b2h, b2l);
    if (lane == 0) { wred[warp][0] = sq; wred[warp][1] = b2; }
    if (acc_at) {
#pragma unroll
        for (int kk = 0; kk < KP; ++kk) {
            const int p = lane + 32 * kk;
            if (p < hp) {
                const float2 H = upk2(ah[kk]), L = upk2(al[kk]);
                scratch[(size_t)warp * hp + p] = make_float4(H.x, L.x, H.y, L.y);
            }
        }
    }
    __syncthreads();
    if (acc_at) {
        float4* P4 = reinterpret_cast<float4*>(a.partF) + (size_t)blockIdx.x * hp;
        for (int p = tid; p < hp; p += TF) {
            float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
#pragma unroll
            for (int w = 0; w < WF; ++w) {
                const float4 q = scratch[(size_t)w * hp + p];
                ff_acc(h0, l0, q.x, q.y);
                ff_acc(h1, l1, q.z, q.w);
            }
            const float2 c0 = ff_norm(h0, l0), c1v = ff_norm(h1, l1);
            P4[p] = make_float4(c0.x, c0.y, c1v.x, c1v.y);
        }
    }
    if (tid == 0) {
        float h = 0.f, l = 0.f, h2 = 0.f, l2 = 0.f;
        for (int w = 0; w < WF; ++w) {
            ff_acc(h, l, wred[w][0].x, wred[w][0].y);
            ff_acc(h2, l2, wred[w][1].x, wred[w][1].y);
        }
        a.spF[blockIdx.x * 4 + 0] = ff_norm(h, l);
        a.spF[blockIdx.x * 4 + 3] = ff_norm(h2, l2);
    }
    __syncthreads();
    return *err == 0;
}

// The fused pass over FP32 rows (A stored in FP32: rows of ldf floats, ldf =
// n rounded up to a multiple of 4, 4 bytes per element instead of 8).  Chunk
// c of a row holds columns 4c .. 4c+3; lane l of every warp takes chunks
// c = l + 32 kk (KC per lane), i.e. the column pairs 2c and 2c+1, so y and the
// A^T u accumulators are 2 KC packed pairs per lane.  The data are exact in
// FP32, so each product is a * (y_hi + y_lo) with the FMA error term of
// a * y_hi (one multiply-add fewer than a float-float element).  Everything
// else -- ring, row ownership, u, the per-warp column sums -- is as in
// ff_pass_fused.
template <int KC, int RW>
__device__ bool ff_pass_fused_f32(const Args& a, Ring& rg, float4* scratch, float2 c1, float2 c2, float2 c3,
                                  bool dot, const float2* oldv, const float2* bvec, float2* dst, bool want_b2,
                                  bool acc_at, volatile int* err) {
    constexpr int R = WF * RW;
    constexpr int KP = 2 * KC;
    __shared__ float2 wred[WF][2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int hp = (int)a.hp;
    const int hq = (int)a.rowq;
    const int64_t ntl = rg.ntl;
    f32x2 yh[KP], yl[KP];
#pragma unroll
    for (int kk = 0; kk < KC; ++kk) {
        const int c = lane + 32 * kk;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float2 y0 = make_float2(0.f, 0.f), y1 = make_float2(0.f, 0.f);
            if (dot && c < hq) { y0 = a.yF[4 * c + 2 * h]; y1 = a.yF[4 * c + 2 * h + 1]; }
            yh[2 * kk + h] = pk2(y0.x, y1.x);
            yl[2 * kk + h] = pk2(y0.y, y1.y);
        }
    }
    f32x2 ah[KP], al[KP];
#pragma unroll
    for (int k = 0; k < KP; ++k) { ah[k] = 0ull; al[k] = 0ull; }
    float sqh = 0.f, sql = 0.f, b2h = 0.f, b2l = 0.f;
    constexpr int SHL = (RW == 1) ? 5 : (RW == 2) ? 4 : (RW == 4) ? 3 : 2;
    const bool owner = (lane & ((1 << SHL) - 1)) == 0;
    const int rw = lane >> SHL;
    auto row_of = [&](int64_t kk) { return ((int64_t)blockIdx.x + kk * (int64_t)gridDim.x) * R + warp + WF * rw; };
    auto fetch = [&](int64_t kk, float2& u, float2& bv) {
        u = make_float2(0.f, 0.f);
        bv = make_float2(0.f, 0.f);
        if (owner && kk < ntl) {
            const int64_t i = row_of(kk);
            if (i < a.m) {
                if (oldv) u = oldv[i];
                if (bvec) bv = bvec[i];
            }
        }
    };
    float2 qu0, qb0, qu1, qb1;
    fetch(0, qu0, qb0);
    fetch(1, qu1, qb1);
#pragma unroll 1
    for (int64_t k = 0; k < ntl; ++k) {
        const float2 uo = qu0, bb = qb0;
        qu0 = qu1;
        qb0 = qb1;
        fetch(k + 2, qu1, qb1);
        const int st = rg.cst;
        const bool ok = mbar_wait(&rg.full[st], rg.cph, err);
        ring_advance(a, rg);
        const int64_t r0 = ((int64_t)blockIdx.x + k * (int64_t)gridDim.x) * R;
        const int rows = (int)min((int64_t)R, a.m - r0);
        const ulonglong2* tile = reinterpret_cast<const ulonglong2*>(rg.tiles) + (size_t)st * R * hq;
        ulonglong2 v[RW][KC];
#pragma unroll
        for (int w = 0; w < RW; ++w) {
            const int r = warp + WF * w;
            const bool rv = ok && r < rows;
#pragma unroll
            for (int kk = 0; kk < KC; ++kk) {
                const int c = lane + 32 * kk;
                v[w][kk] = (rv && c < hq) ? tile[(size_t)r * hq + c] : make_ulonglong2(0ull, 0ull);
            }
        }
        ring_release(a, rg, st, lane, err);
        float tvh[RW], tvl[RW];
#pragma unroll
        for (int w = 0; w < RW; ++w) { tvh[w] = 0.f; tvl[w] = 0.f; }
        if (dot) {
            f32x2 sh[RW][2], sl[RW][2];
#pragma unroll
            for (int w = 0; w < RW; ++w) { sh[w][0] = sh[w][1] = sl[w][0] = sl[w][1] = 0ull; }
#pragma unroll
            for (int kk = 0; kk < KC; ++kk) {
#pragma unroll
                for (int w = 0; w < RW; ++w) {
                    ff2_madd_xp(v[w][kk].x, yh[2 * kk], yl[2 * kk], sh[w][0], sl[w][0]);
                    ff2_madd_xp(v[w][kk].y, yh[2 * kk + 1], yl[2 * kk + 1], sh[w][1], sl[w][1]);
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
            int off = 16;
#pragma unroll
            for (int half = RW / 2; half >= 1; half /= 2) {
                const bool up = (lane & off) != 0;
#pragma unroll
                for (int k2 = 0; k2 < half; ++k2) {
                    const float sh_ = up ? tvh[k2] : tvh[k2 + half], sl_ = up ? tvl[k2] : tvl[k2 + half];
                    float kh = up ? tvh[k2 + half] : tvh[k2], kl = up ? tvl[k2 + half] : tvl[k2];
                    const float rh = __shfl_xor_sync(0xffffffffu, sh_, off);
                    const float rl = __shfl_xor_sync(0xffffffffu, sl_, off);
                    ff_acc(kh, kl, rh, rl);
                    tvh[k2] = kh;
                    tvl[k2] = kl;
                }
                off >>= 1;
            }
            for (; off >= 1; off >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, tvh[0], off);
                const float ol = __shfl_xor_sync(0xffffffffu, tvl[0], off);
                ff_acc(tvh[0], tvl[0], oh, ol);
            }
        }
        float2 nv = make_float2(0.f, 0.f);
        if (owner) {
            const float2 tv = ff_norm(tvh[0], tvl[0]);
            nv = ff_add(ff_add(ff_mul(c1, tv), ff_mul(c2, uo)), ff_mul(c3, bb));
            const int r = warp + WF * rw;
            if (ok && r < rows) {
                dst[r0 + r] = nv;
                ff_madd(nv.x, nv.y, nv.x, nv.y, sqh, sql);
                if (want_b2) ff_madd(bb.x, bb.y, bb.x, bb.y, b2h, b2l);
            }
        }
        if (acc_at) {
            f32x2 uh[RW], ul[RW];
#pragma unroll
            for (int w = 0; w < RW; ++w) {
                const float x = __shfl_sync(0xffffffffu, nv.x, w << SHL);
                const float y = __shfl_sync(0xffffffffu, nv.y, w << SHL);
                uh[w] = pk2(x, x);
                ul[w] = pk2(y, y);
            }
#pragma unroll
            for (int kk = 0; kk < KC; ++kk) {
#pragma unroll
                for (int w = 0; w < RW; ++w) {
                    ff2_madd_xp(v[w][kk].x, uh[w], ul[w], ah[2 * kk], al[2 * kk]);
                    ff2_madd_xp(v[w][kk].y, uh[w], ul[w], ah[2 * kk + 1], al[2 * kk + 1]);
                }
            }
        }
    }
    const float2 sq = ff_warp_sum(sqh, sql);
    const float2 b2 = ff_warp_sum(b2h, b2l);
    if (lane == 0) { wred[warp][0] = sq; wred[warp][1] = b2; }
    if (acc_at) {
        // each warp's column sums go straight to its own row of partF (no
        // shared-memory scratch: the ring gets that space)
        float4* P4 = reinterpret_cast<float4*>(a.partF) + ((size_t)blockIdx.x * WF + warp) * hp;
#pragma unroll
        for (int kk = 0; kk < KC; ++kk) {
            const int c = lane + 32 * kk;
            if (c < hq) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float2 H = upk2(ah[2 * kk + h]), L = upk2(al[2 * kk + h]);
                    const float2 c0 = ff_norm(H.x, L.x), c1v = ff_norm(H.y, L.y);
                    P4[2 * c + h] = make_float4(c0.x, c0.y, c1v.x, c1v.y);
                }
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        float h = 0.f, l = 0.f, h2 = 0.f, l2 = 0.f;
        for (int w = 0; w < WF; ++w) {
            ff_acc(h, l, wred[w][0].x, wred[w][0].y);
            ff_acc(h2, l2, wred[w][1].x, wred[w][1].y);
        }
        a.spF[blockIdx.x * 4 + 0] = ff_norm(h, l);
        a.spF[blockIdx.x * 4 + 3] = ff_norm(h2, l2);
    }
    __syncthreads();
    return *err == 0;
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

// g_j = sum over the nparts rows of partF[c][j] (one per CTA, or per warp);
// one warp per column, warps 1..nwc-1.
__device__ void reduce_columns(const Args& a, int warp, int lane, int nwc) {
    const int64_t nw = (int64_t)gridDim.x * (nwc - 1);
    for (int64_t j = (int64_t)blockIdx.x * (nwc - 1) + (warp - 1); j < a.n; j += nw) {
        float h = 0.f, l = 0.f;
        for (int64_t c = lane; c < a.nparts; c += 32) {
            const float2 v = a.partF[c * a.ldf + j];
            ff_acc(h, l, v.x, v.y);
        }
        const float2 s = ff_warp_sum(h, l);
        if (lane == 0) a.gF[j] = s;
    }
}

// vun_j = (M^T g)_j ib - [sub] beta v_j, and the squares of vun_j and w_j;
// one warp per column, all warps.
__device__ void update_vun(const Args& a, const Bcast& bc, bool sub, int warp, int lane, int nwc) {
    const int64_t n = a.n;
    const int64_t nw = (int64_t)gridDim.x * nwc;
    for (int64_t j = (int64_t)blockIdx.x * nwc + warp; j < n; j += nw) {
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

// Raw rows of M src (src float-float, n): warps 1..nwc-1, one warp per row;
// the raw value goes to dst[i] and is rescaled by the same lane later.
__device__ void trmv_rows_raw(const Args& a, const float2* src, float2* dst, int warp, int lane, int nwc) {
    const int64_t n = a.n;
    const int64_t nw = (int64_t)gridDim.x * (nwc - 1);
    for (int64_t i = (int64_t)blockIdx.x * (nwc - 1) + (warp - 1); i < n; i += nw) {
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

__device__ void scale_rows(const Args& a, float2* dst, float2 sc, int warp, int lane, int nwc) {
    const int64_t nw = (int64_t)gridDim.x * (nwc - 1);
    if (lane != 0) return;
    for (int64_t i = (int64_t)blockIdx.x * (nwc - 1) + (warp - 1); i < a.n; i += nw) dst[i] = ff_mul(dst[i], sc);
}

__device__ __forceinline__ double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

// Lane-parallel reciprocal square roots: lane k returns rsqrt of its own
// argument (0 for a non-positive one); the caller shuffles the results out.
__device__ __forceinline__ double lane_rsqrt(double arg) { return arg > 0.0 ? rsqrt(arg) : 0.0; }

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// FUSED selects the pass: fused roles on TF threads, or split row/column
// roles on T threads.
// F32: 0 = float-float rows, 1 = FP32 rows (ff_pass_fused_f32)
template <int KP, int RW, bool FUSED, int F32 = 0>
__global__ void __launch_bounds__(FUSED ? TF : T, 1) lsqr_ff_kernel(Args a) {
    constexpr int NT = FUSED ? TF : T;
    constexpr int NWC = NT / 32;
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ __align__(8) uint64_t full[MAX_ST];
    __shared__ unsigned int rel[MAX_ST];
    __shared__ unsigned long long issued;
    __shared__ Bcast bc;
    __shared__ Scal sc;
    __shared__ int err_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t n = a.n;
    const int64_t G = gridDim.x;
    const double eps = 2.220446049250313e-16;
    const double dampsq = a.damp * a.damp;
    const int XW = NT - 32;                // threads of warps 1.. (elementwise work)

    Ring rg;
    rg.full = full;
    rg.tiles = reinterpret_cast<float4*>(dsm);
    rg.ntl = (blockIdx.x < a.ntiles) ? (a.ntiles - blockIdx.x + G - 1) / G : 0;
    rg.cst = 0;
    rg.cph = 0;
    rg.ist = 0;
    rg.ik = 0;
    rg.inflight = 0;
    rg.rel = rel;
    rg.issued = &issued;
    rg.consumed = 0;
    // split roles: the u hand-off buffers; fused roles: the column scratch
    unsigned char* extra = dsm + (size_t)a.ST * a.R * a.rowq * 16;
    ulonglong2* usm = reinterpret_cast<ulonglong2*>(extra);
    float4* scratch = reinterpret_cast<float4*>(extra);
    volatile int* err = &err_s;
    if (tid == 0) {
        err_s = 0;
        issued = 0;
        for (int s = 0; s < a.ST; ++s) {
            mbar_init(&full[s], 1);
            rel[s] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (FUSED) {
        if (rg.ntl > 0) {
            if (tid == 0) {
                int64_t ik = 0;
                for (int s = 0; s < a.ST; ++s) {
                    ring_copy(a, rg, s, ik);
                    ik = (ik + 1 == rg.ntl) ? 0 : ik + 1;
                }
                issued = (unsigned long long)a.ST;
            }
            rg.ik = a.ST % rg.ntl;
        }
    } else if (tid == ISSUER) {
        ring_issue(a, rg);
    }

#define LSFF_DRAIN()                                   \
    do {                                               \
        if (FUSED) {                                   \
            __syncthreads();                           \
            ring_drain_fused(a, rg);                   \
        } else {                                       \
            ring_drain(a, rg);                         \
        }                                              \
    } while (0)
#define LSFF_SYNC()                    \
    do {                               \
        if (!grid_sync(a.bar)) {       \
            LSFF_DRAIN();              \
            return;                    \
        }                              \
    } while (0)
#define LSFF_PASS(...)                                                                 \
    do {                                                                               \
        bool pass_ok;                                                                  \
        if constexpr (F32 != 0) pass_ok = ff_pass_fused_f32<KP / 2, RW>(a, rg, scratch, __VA_ARGS__, err); \
        else if constexpr (FUSED) pass_ok = ff_pass_fused<KP, RW>(a, rg, scratch, __VA_ARGS__, err); \
        else pass_ok = ff_pass<KP, RW>(a, rg, usm, __VA_ARGS__, err);                  \
        if (!pass_ok) {                                                                \
            set_status(a, KSTATUS_BARRIER_TIMEOUT);                                    \
            LSFF_DRAIN();                                                              \
            return;                                                                    \
        }                                                                              \
    } while (0)

    const int64_t gt = (int64_t)blockIdx.x * NT + tid;
    const int64_t gthreads = G * NT;
    const float2 zero2 = make_float2(0.f, 0.f), one2 = make_float2(1.f, 0.f), mone2 = make_float2(-1.f, 0.f);

    // ---- initialisation (solvers.rs:141-182) ----
    for (int64_t j = gt; j < n; j += gthreads) {
        a.xF[j] = a.x0F ? a.x0F[j] : zero2;
        a.wF[j] = zero2;
        a.vF[j] = zero2;
        if (a.calc_var) a.varF[j] = zero2;
    }
    if (a.x0F) {
        if (warp > 0) trmv_rows_raw(a, a.x0F, a.yF, warp, lane, NWC);
        LSFF_SYNC();
    }
    // u = b - A M x0 (or b); beta^2, ||b||^2, A^T u partials
    LSFF_PASS(a.x0F ? mone2 : zero2, zero2, one2, a.x0F != nullptr, nullptr, a.bF, a.uF, true, true);
    LSFF_SYNC();
    if (warp == 0) {
        const float2 S = sum_slot(a, 0, lane);
        const float2 B2 = sum_slot(a, 3, lane);
        const double Sd = ff_to_double(S), B2d = ff_to_double(B2);
        const double r = lane_rsqrt(lane == 0 ? Sd : B2d);
        const double ib = shfl_d(r, 0);
        const double ibn = shfl_d(r, 1);
        if (lane == 0) {
            sc.beta = Sd * ib;
            sc.bnorm = B2d * ibn;
            sc.ibn = ibn;
            sc.us = ib;
            bc.ib = ff_split(ib);
            bc.beta = ff_split(sc.beta);
        }
    } else {
        reduce_columns(a, warp, lane, NWC);
    }
    LSFF_SYNC();
    update_vun(a, bc, false, warp, lane, NWC);
    LSFF_SYNC();
    if (warp == 0) {
        float2 A2, W2;
        sum_colsq(a, lane, A2, W2);
        const double A2d = ff_to_double(A2);
        const double ia = lane_rsqrt(A2d);
        if (lane == 0) {
            sc.alfa = A2d * ia;
            bc.ia = ff_split(ia);
        }
    } else {
        trmv_rows_raw(a, a.vunF, a.yF, warp, lane, NWC);
    }
    __syncthreads();
    if (warp > 0) {
        scale_rows(a, a.yF, bc.ia, warp, lane, NWC);
        for (int64_t j = (int64_t)blockIdx.x * XW + (tid - 32); j < n; j += G * XW) {
            const float2 vv = ff_mul(a.vunF[j], bc.ia);
            a.vF[j] = vv;
            a.wF[j] = vv;
        }
    } else if (lane == 0) {
        bc.istop = (sc.alfa * sc.beta == 0.0) ? -1 : 0;
        sc.rhobar = sc.alfa; sc.phibar = sc.beta; sc.rnorm = sc.beta; sc.r1norm = sc.beta; sc.r2norm = sc.beta;
        sc.anorm = 0; sc.acond = 0; sc.ddnorm = 0; sc.res2 = 0; sc.xnorm = 0; sc.xxnorm = 0; sc.z = 0;
        sc.cs2 = -1.0; sc.sn2 = 0.0;
        sc.arnorm = sc.alfa * sc.beta;
        sc.istop = 0;
        bc.c2 = ff_split(-sc.alfa * sc.us);
    }
    LSFF_SYNC();
    if (bc.istop == -1) {
        if (gt == 0) {
            a.out[0] = 0; a.out[1] = 0; a.out[2] = sc.beta; a.out[3] = sc.beta;
            a.out[4] = 0; a.out[5] = 0; a.out[6] = 0; a.out[7] = 0;
            if (a.arn) a.arn[0] = 0.0;
        }
        for (int64_t j = gt; j < n; j += gthreads) {
            a.x[j] = ff_to_double(a.xF[j]);
            if (a.calc_var && a.var) a.var[j] = 0.0;
        }
        LSFF_DRAIN();
        return;
    }
    const double ctol = a.conlim > 0.0 ? 1.0 / a.conlim : 0.0;
    int64_t itn = 0;

    while (itn < a.iter_lim) {
        if (gt == 0 && a.arn) a.arn[itn] = sc.arnorm;
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
            const int beta_pos = Sd > 0.0;
            const double rhobar = sc.rhobar, alfa = sc.alfa, anorm0 = sc.anorm;
            const double rb2 = rhobar * rhobar + dampsq;
            const double an2 = anorm0 * anorm0 + alfa * alfa + Sd + dampsq;
            const double arg = lane == 0 ? Sd : lane == 1 ? rb2 + Sd : lane == 2 ? rb2 : an2;
            const double r = lane_rsqrt(arg);
            const double ib = shfl_d(r, 0);
            const double irho = shfl_d(r, 1);
            const double irb1 = shfl_d(r, 2);
            const double ian = shfl_d(r, 3);
            const double beta = Sd * ib;
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
            const double psi = sn1 * sc.phibar;
            double phibar = sc.phibar * cs1;
            const double rho = (rb2 + Sd) * irho;
            const double c = rhobar1 * irho;
            const double s = beta * irho;
            const double phi = c * phibar;
            phibar = s * phibar;
            const double tau = s * phi;
            if (lane == 0) {
                sc.beta = beta;
                if (beta_pos) {
                    sc.us = ib;
                    sc.anorm = an2 * ian;
                }
                sc.psi = psi; sc.phibar = phibar; sc.rho = rho; sc.irho = irho; sc.c = c; sc.s = s;
                sc.phi = phi; sc.tau = tau;
                bc.ib = ff_split(ib);
                bc.beta = ff_split(beta);
                bc.beta_pos = beta_pos;
                bc.t1 = ff_split(phi * irho);
                bc.irho = ff_split(irho);
            }
        } else {
            reduce_columns(a, warp, lane, NWC);
        }
        LSFF_SYNC();
        // v = M^T A^T u / beta - beta v  (solvers.rs:197-204)
        if (bc.beta_pos) update_vun(a, bc, true, warp, lane, NWC);
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
            double alfa = sc.alfa;
            if (bp) {
                const double A2d = ff_to_double(A2);
                const double ia = lane_rsqrt(A2d);
                alfa = A2d * ia;
                if (lane == 0) bc.ia = ff_split(ia);
            }
            const double theta = sc.s * alfa;
            if (lane == 0) {
                sc.alfa = alfa;
                sc.rhobar = -sc.c * alfa;
                bc.t2 = ff_split(-theta * sc.irho);
                bc.c2 = ff_split(-alfa * sc.us);
            }
        } else if (bp) {
            trmv_rows_raw(a, a.vunF, a.yF, warp, lane, NWC);
        }
        __syncthreads();
        if (warp > 0) {
            // x += t1 w ; w = v + t2 w ; var += (w / rho)^2 ; y = M v  (solvers.rs:222-232)
            if (bp) scale_rows(a, a.yF, bc.ia, warp, lane, NWC);
            const float2 t1 = bc.t1, t2 = bc.t2, ia = bc.ia, ir = bc.irho;
            for (int64_t j = (int64_t)blockIdx.x * XW + (tid - 32); j < n; j += G * XW) {
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
            const double alfa = sc.alfa, rho = sc.rho, irho = sc.irho, phi = sc.phi, psi = sc.psi;
            const double phibar = sc.phibar, anorm = sc.anorm, bnorm_inv = sc.ibn;
            const double theta = sc.s * alfa;
            const double ddnorm = sc.ddnorm + wsq * irho * irho;
            const double delta = sc.sn2 * rho;
            const double gambar = -sc.cs2 * rho;
            const double rhs = phi - delta * sc.z;
            const double res2 = sc.res2 + psi * psi;
            const double rn2 = phibar * phibar + res2;
            const double g2 = gambar * gambar + theta * theta;
            const double arg1 = lane == 0 ? g2 : lane == 1 ? gambar * gambar : lane == 2 ? ddnorm : rn2;
            const double r1 = lane_rsqrt(arg1);
            const double igamma = shfl_d(r1, 0);
            const double igb = shfl_d(r1, 1);
            const double idd = shfl_d(r1, 2);
            const double irn = shfl_d(r1, 3);
            const double zbar = rhs * igb * sgn(gambar);
            const double cs2 = gambar * igamma;
            const double sn2 = theta * igamma;
            const double z = rhs * igamma;
            const double xn2 = sc.xxnorm + zbar * zbar;
            const double xxnorm = sc.xxnorm + z * z;
            const double acond = anorm * (ddnorm * idd);
            const double rnorm = rn2 * irn;
            const double arnorm = alfa * fabs(sc.tau);
            const double r1sq = rnorm * rnorm - dampsq * xxnorm;
            const double arg2 = lane == 0 ? xn2 : fabs(r1sq);
            const double r2 = lane_rsqrt(arg2);
            const double xnorm = xn2 * shfl_d(r2, 0);
            const double r1norm = fabs(r1sq) * shfl_d(r2, 1);
            const double test1 = rnorm * bnorm_inv;
            const double axb = anorm * xnorm * bnorm_inv;
            const double arg3 = lane == 0 ? anorm * rnorm + eps : lane == 1 ? acond + eps : 1.0 + axb;
            const double r3 = lane_rsqrt(arg3);
            const double q0 = shfl_d(r3, 0), q1 = shfl_d(r3, 1), q2 = shfl_d(r3, 2);
            const double test2 = arnorm * (q0 * q0);
            const double test3 = q1 * q1;
            const double tt1 = test1 * (q2 * q2);
            const double rtol = a.atol + a.btol * axb;
            int istop = 0;
            if (itn >= a.iter_lim) istop = 7;
            if (1.0 + test3 <= 1.0) istop = 6;
            if (1.0 + test2 <= 1.0) istop = 5;
            if (1.0 + tt1 <= 1.0) istop = 4;
            if (test3 <= ctol) istop = 3;
            if (test2 <= a.atol) istop = 2;
            if (test1 <= rtol) istop = 1;
            if (a.abs_tol > 0.0 && arnorm < a.abs_tol && (istop == 0 || istop == 7)) istop = 2;
            if (lane == 0) {
                sc.ddnorm = ddnorm; sc.res2 = res2; sc.cs2 = cs2; sc.sn2 = sn2; sc.z = z; sc.xxnorm = xxnorm;
                sc.acond = acond; sc.rnorm = rnorm; sc.arnorm = arnorm; sc.xnorm = xnorm; sc.r1norm = r1norm;
                sc.r2norm = rnorm; sc.istop = istop;
                bc.istop = istop;
            }
        }
        LSFF_SYNC();
        if (bc.istop != 0) break;
    }
    for (int64_t j = gt; j < n; j += gthreads) {
        a.x[j] = ff_to_double(a.xF[j]);
        if (a.calc_var && a.var) a.var[j] = ff_to_double(a.varF[j]);
    }
    if (gt == 0) {
        a.out[0] = sc.istop; a.out[1] = (double)itn; a.out[2] = sc.r1norm; a.out[3] = sc.r2norm;
        a.out[4] = sc.anorm; a.out[5] = sc.acond; a.out[6] = sc.xnorm; a.out[7] = sc.arnorm;
    }
    LSFF_DRAIN();
#undef LSFF_DRAIN
#undef LSFF_SYNC
#undef LSFF_PASS
}

// Row-major float-float copy in column-pair order: row i is hp = ldf / 2
// chunks of 16 bytes, chunk p = (hi_2p, hi_2p+1, lo_2p, lo_2p+1); zero for
// columns in [n, ldf).  FP32 data has lo = 0.  32 x 32 tiles through shared
// memory.
__device__ __forceinline__ float2 ff_of(double v) { return ff_split(v); }
__device__ __forceinline__ float2 ff_of(float v) { return make_float2(v, 0.f); }

template <typename TA>
__global__ void rowmajor_split_kernel(const TA* __restrict__ A, int64_t m, int64_t n, int64_t lda,
                                      float* __restrict__ AF, int64_t ldf) {
    __shared__ float2 tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, j0 = (int64_t)blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += 8) {
        const int64_t i = i0 + threadIdx.x, j = j0 + k;
        float2 v = make_float2(0.f, 0.f);
        if (i < m && j < n) v = ff_of(A[i + j * lda]);
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

// Row-major FP32 copy of a column-major FP32 A: row i is ldq floats (n
// rounded up to a multiple of 4, zero beyond n), so a 16-byte chunk holds 4
// consecutive columns.  64 x 64 tiles through shared memory (256-byte column
// segments in, 256-byte row segments out), eight persistent blocks per SM
// walking the tiles.
__global__ void __launch_bounds__(256) rowmajor_f32_kernel(const float* __restrict__ A, int64_t m, int64_t n,
                                                           int64_t lda, float* __restrict__ AQ, int64_t ldq) {
    __shared__ float tile[64][65];
    const int64_t tm = (m + 63) / 64, tn = (ldq + 63) / 64;
    const int tx = threadIdx.x & 63, ty = threadIdx.x >> 6;       // 64 x 4
    for (int64_t t = blockIdx.x; t < tm * tn; t += gridDim.x) {
        const int64_t i0 = (t % tm) * 64, j0 = (t / tm) * 64;
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t i = i0 + tx, j = j0 + ty + 4 * q;
            v[q] = (i < m && j < n) ? A[i + j * lda] : 0.f;
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) tile[ty + 4 * q][tx] = v[q];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t i = i0 + ty + 4 * q, j = j0 + tx;
            if (i < m && j < ldq) AQ[i * ldq + j] = tile[tx][ty + 4 * q];
        }
        __syncthreads();
    }
}

__global__ void vec_split_kernel(const double* __restrict__ v, int64_t n, float2* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = ff_split(v[i]);
}

// M <- hi + lo of its float-float split (upper part, in place).
__global__ void ff_round_kernel(double* __restrict__ M, int64_t n, int64_t ldm) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        if (i <= j) {
            const float2 v = ff_split(M[i + j * ldm]);
            M[i + j * ldm] = (double)v.x + (double)v.y;
        }
    }
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

template <int KP, int RW, bool FUSED, int F32 = 0>
static const void* kernel_kp() { return (const void*)lsqr_ff_kernel<KP, RW, FUSED, F32>; }

// Kernel for hp column pairs: the y registers cover hp (KP chunks of 32
// pairs per lane) and a tile (R rows) is at most 64 KB, so the ring holds 3
// or more tiles.  Up to 256 pairs the fused roles (registers hold y, the A^T u
// accumulators and RW rows of chunks: RW KP <= 16); above, the split roles.
struct KernelPick {
    const void* fn;
    int R;          // rows per tile
    int threads;
    bool fused;
};
static KernelPick pick_kernel(int64_t hp) {
    if (hp <= 32) return {kernel_kp<1, 8, true>(), WF * 8, TF, true};
    if (hp <= 64) return {kernel_kp<2, 8, true>(), WF * 8, TF, true};
    if (hp <= 128) return {kernel_kp<4, 4, true>(), WF * 4, TF, true};
    if (hp <= 256) return {kernel_kp<8, 2, true>(), WF * 2, TF, true};
    return {kernel_kp<16, 1, false>(), WA * 1, T, false};
}
// FP32 rows: hq 16-byte chunks (4 columns each) per row, KC = KP / 2 chunks
// per lane, fused roles throughout (n <= 1024: 8 chunks per lane, two rows
// per warp).
static KernelPick pick_kernel_f32(int64_t hq) {
    if (hq <= 32) return {kernel_kp<2, 8, true, 1>(), WF * 8, TF, true};
    if (hq <= 64) return {kernel_kp<4, 4, true, 1>(), WF * 4, TF, true};
    if (hq <= 128) return {kernel_kp<8, 4, true, 1>(), WF * 4, TF, true};
    return {kernel_kp<16, 2, true, 1>(), WF * 2, TF, true};
}

}  // namespace lsff

bool lsqr_ff_supported(int64_t n) { return n >= 1 && n <= lsff::MAX_N; }

void ff_round_upper(Ctx& ctx, double* M, int64_t n, int64_t ldm) {
    int g = (int)div_up(n * n, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    lsff::ff_round_kernel<<<g, 256, 0, ctx.stream>>>(M, n, ldm);
    RNLA_LAUNCH_CHECK();
}

// Float-float copies of A (row-major, column-pair order) and b, enqueued on
// `st`.
static void build_ff_input(Ctx& ctx, cudaStream_t st, const void* A, bool a_f32, int64_t m, int64_t n,
                           int64_t lda, const double* b, int64_t ldf, float2* AF, float2* bF,
                           bool a_done = false) {
    using namespace lsff;
    dim3 grid((unsigned)div_up(m, 32), (unsigned)div_up(ldf, 32));
    if (a_f32 && !a_done) {
        rowmajor_f32_kernel<<<(unsigned)std::min<int64_t>(div_up(m, 64) * div_up(ldf, 64), 8 * ctx.sm_count), 256, 0,
                              st>>>(static_cast<const float*>(A), m, n, lda, reinterpret_cast<float*>(AF), ldf);
        RNLA_LAUNCH_CHECK();
    } else if (!a_done) {
        rowmajor_split_kernel<double><<<grid, dim3(32, 8), 0, st>>>(static_cast<const double*>(A), m, n, lda,
                                                                    reinterpret_cast<float*>(AF), ldf);
        RNLA_LAUNCH_CHECK();
    }
    int g = (int)div_up(m, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    vec_split_kernel<<<g, 256, 0, st>>>(b, m, bF);
    RNLA_LAUNCH_CHECK();
}

void lsqr_ff_alloc(Ctx& ctx, const void* A, bool a_f32, int64_t m, int64_t n, LsqrFFInput& in) {
    if (!lsqr_ff_supported(n)) fail(RNLA_ERR_UNSUPPORTED, "lsqr (float-float): n must be in [1, 1024]");
    in.A = A; in.m = m; in.n = n;
    in.f32 = a_f32;
    // FP32 data: a row-major FP32 copy (ldf = n rounded up to 4 floats);
    // FP64 data: the float-float copy (ldf = n rounded up to 2 pairs)
    in.ldf = a_f32 ? (n + 3) & ~3LL : (n + 1) & ~1LL;
    in.AF.alloc(a_f32 ? (size_t)m * in.ldf / 2 : (size_t)m * in.ldf, ctx.stream);
    in.bF.alloc(m, ctx.stream);
    in.owner = ctx.stream;
}

void lsqr_ff_build(Ctx& ctx, LsqrFFInput& in, int64_t lda, const double* b, cudaStream_t st,
                   bool a_done) {
    build_ff_input(ctx, st, in.A, in.f32, in.m, in.n, lda, b, in.ldf, in.AF, in.bF, a_done);
    RNLA_CUDA(cudaEventCreateWithFlags(&in.ready, cudaEventDisableTiming));
    RNLA_CUDA(cudaEventRecord(in.ready, st));
}

void lsqr_ff_prepare(Ctx& ctx, const void* A, bool a_f32, int64_t m, int64_t n, int64_t lda, const double* b,
                     LsqrFFInput& in) {
    lsqr_ff_alloc(ctx, A, a_f32, m, n, in);
    const cudaStream_t st = ctx.side ? ctx.side : side_stream(ctx.device);
    stream_wait(st, ctx.stream);                   // buffers allocated, A and b written
    lsqr_ff_build(ctx, in, lda, b, st);
}

LsqrResult lsqr_ff_solve(Ctx& ctx, const void* A, bool a_f32, int64_t m, int64_t n, int64_t lda, const double* M,
                         const double* b, const double* x0, const LsqrParams& prm, double* x, double* var,
                         double* arnorms_dev, const LsqrFFInput* pre, LsqrPending* pend) {
    using namespace lsff;
    if (!lsqr_ff_supported(n)) fail(RNLA_ERR_UNSUPPORTED, "lsqr (float-float): n must be in [1, 1024]");
    if (pre && (pre->A != A || pre->m != m || pre->n != n || pre->f32 != a_f32)) pre = nullptr;
    cudaStream_t st = ctx.stream;
    const int64_t ldf = a_f32 ? (n + 3) & ~3LL : (n + 1) & ~1LL;
    const int64_t hp = ldf / 2;
    const int64_t rowq = a_f32 ? ldf / 4 : hp;
    const KernelPick kp = a_f32 ? pick_kernel_f32(rowq) : pick_kernel(hp);
    const void* k = kp.fn;
    const int R = kp.R;
    const size_t stage = (size_t)R * rowq * 16;
    // fused: per-warp column scratch (none for FP32 rows, whose warps write
    // partF directly); split: the two u hand-off buffers
    const size_t extra = a_f32 ? 0 : kp.fused ? (size_t)WF * hp * 16 : (size_t)2 * R * 16;
    int STn = (int)(RING_BYTES / stage);
    STn = STn > MAX_ST ? MAX_ST : STn;
    const size_t smem_cap = 224 * 1024;            // dynamic shared memory per CTA (static use is < 2 KB)
    if ((size_t)STn * stage + extra > smem_cap) STn = extra < smem_cap ? (int)((smem_cap - extra) / stage) : 0;
    if (STn < 3) fail(RNLA_ERR_UNSUPPORTED, "lsqr (float-float): tile ring does not fit");
    const size_t smem = (size_t)STn * stage + extra;
    set_smem_limit((const void*)k, smem);
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kp.threads, smem));
    if (nb < 1) fail(RNLA_ERR_UNSUPPORTED, "lsqr (float-float): kernel does not fit on an SM");
    const int G = ctx.sm_count;

    DevBuf<float2> AFo, MF, MtF, bFo, x0F, uF, yF, gF, vF, wF, xF, vunF, varF, partF, spF;
    DevBuf<float4> colsq;
    DevBuf<double> out;
    DevBuf<unsigned int> bar;
    const float2* AF;
    const float2* bF;
    if (pre) {
        RNLA_CUDA(cudaStreamWaitEvent(st, pre->ready, 0));
        AF = pre->AF.get();
        bF = pre->bF.get();
    } else {
        AFo.alloc(a_f32 ? (size_t)m * ldf / 2 : (size_t)m * ldf, st);
        bFo.alloc(m, st);
        build_ff_input(ctx, st, A, a_f32, m, n, lda, b, ldf, AFo, bFo);
        AF = AFo.get();
        bF = bFo.get();
    }
    uF.alloc(m, st);
    yF.alloc(ldf, st);
    gF.alloc(n, st); vF.alloc(n, st); wF.alloc(n, st); xF.alloc(n, st); vunF.alloc(n, st); varF.alloc(n, st);
    const int nparts = a_f32 ? G * WF : G;
    partF.alloc((size_t)nparts * ldf, st);
    spF.alloc((size_t)G * 4, st);
    colsq.alloc(n, st);
    out.alloc(8, st);
    bar.alloc(2, st);
    RNLA_CUDA(cudaMemsetAsync(bar.get(), 0, 2 * sizeof(unsigned int), st));
    RNLA_CUDA(cudaMemsetAsync(out.get(), 0, 8 * sizeof(double), st));
    RNLA_CUDA(cudaMemsetAsync(yF.get(), 0, ldf * sizeof(float2), st));
    ctx.clear_status();
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
    a.AF = AF; a.m = m; a.n = n; a.ldf = ldf; a.hp = hp; a.rowq = rowq; a.nparts = nparts; a.R = R; a.ST = STn;
    a.ntiles = div_up(m, R);
    a.bF = bF;
    a.uF = uF.get(); a.yF = yF.get(); a.gF = gF.get(); a.vF = vF.get(); a.wF = wF.get(); a.xF = xF.get();
    a.vunF = vunF.get(); a.varF = varF.get(); a.partF = partF.get(); a.spF = spF.get(); a.colsq = colsq.get();
    a.x = x; a.var = var; a.arn = arnorms_dev; a.out = out.get();
    a.damp = prm.damp; a.atol = prm.atol; a.btol = prm.btol; a.conlim = prm.conlim;
    a.abs_tol = prm.abs_arnorm_tol;
    a.iter_lim = prm.iter_lim < 0 ? 2 * n : prm.iter_lim;
    a.calc_var = (prm.calc_var && var) ? 1 : 0;
    a.bar.count = bar.get(); a.bar.gen = bar.get() + 1; a.bar.status = ctx.status;
    void* params[] = {&a};
    cudaEvent_t ev[2];
    RNLA_CUDA(cudaEventCreate(&ev[0]));
    RNLA_CUDA(cudaEventCreate(&ev[1]));
    RNLA_CUDA(cudaEventRecord(ev[0], st));
    RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3(G), dim3(kp.threads), params, smem, st));
    count_launch();
    RNLA_CUDA(cudaEventRecord(ev[1], st));
    if (pend && ctx.deferred) {
        // no host synchronisation: the scalars go to pinned memory and are
        // read after the caller's final synchronisation
        static thread_local double* pinned = nullptr;
        if (!pinned) RNLA_CUDA(cudaMallocHost(&pinned, 8 * sizeof(double)));
        pend->host = pinned;
        pend->ev[0] = ev[0];
        pend->ev[1] = ev[1];
        pend->armed = true;
        RNLA_CUDA(cudaMemcpyAsync(pinned, out.get(), 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
        return LsqrResult{};
    }
    double h[8];
    RNLA_CUDA(cudaMemcpyAsync(h, out.get(), sizeof h, cudaMemcpyDeviceToHost, st));
    RNLA_CUDA(cudaStreamSynchronize(st));
    ctx.check_status("lsqr");
    float kms = 0.f;
    RNLA_CUDA(cudaEventElapsedTime(&kms, ev[0], ev[1]));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    LsqrResult r;
    r.ms_kernel = kms;
    r.istop = (int64_t)h[0]; r.itn = (int64_t)h[1];
    r.r1norm = h[2]; r.r2norm = h[3]; r.anorm = h[4]; r.acond = h[5]; r.xnorm = h[6]; r.arnorm = h[7];
    return r;
}

void LsqrPending::resolve(LsqrResult& r) const {
    if (!armed) return;
    const double* h = host;
    r.istop = (int64_t)h[0]; r.itn = (int64_t)h[1];
    r.r1norm = h[2]; r.r2norm = h[3]; r.anorm = h[4]; r.acond = h[5]; r.xnorm = h[6]; r.arnorm = h[7];
    float kms = 0.f;
    if (cudaEventElapsedTime(&kms, ev[0], ev[1]) == cudaSuccess) r.ms_kernel = kms;
}

}  // namespace rnla
