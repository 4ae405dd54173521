// Persistent cooperative kernels for the inner least-squares solvers:
//   * LSQR (solvers.rs:115-278), one launch for the whole iteration;
//   * CGLS (cg.rs:18-61), same structure.
// Both run on the operator A M, where M = R^-1 (upper triangular) is the
// sketch preconditioner applied inside the kernel (the reference forms
// A R^-1 explicitly, sketch_and_precondition.rs:56) or the identity.
//
// One LSQR iteration reads A once: a CTA stages a tile of R rows x n columns
// in shared memory, forms (A y)_i for its rows, the new u_i (a row-local
// update), and accumulates A^T u over the same staged tile.  Reductions go
// through per-CTA partials summed in a fixed order, so every CTA computes
// the same scalars and the run is reproducible.  Grid barriers are bounded
// (rnla_common.cuh) and end the kernel with a status code on timeout.
#include "rnla_internal.h"
#include "rnla_ff.cuh"
#include <cooperative_groups.h>
#include <type_traits>

namespace rnla {

constexpr int IT_THREADS = 256;
constexpr int IT_MAXACC = 16;          // n <= 256 * 16 = 4096 for the fused kernels

struct IterArgs {
    const void* A;
    int64_t m, n, lda;
    const double* M;    // upper-triangular preconditioner, column-major n x n (nullable)
    const double* Mt;   // its transpose, column-major (row i of M contiguous)
    const double* b;
    const double* x0;   // nullable
    double *u, *v, *vun, *w, *x, *y, *g, *part, *sp, *var, *arn, *ap;
    double damp, atol, btol, conlim, abs_tol;
    int64_t iter_lim;
    int calc_var;
    double* out;
    GridBarrier bar;
    int R;              // rows per staged tile of the general pass (power of two, <= 64)
    int64_t red_off;    // offset (doubles) of the block-reduction scratch in shared memory
};

template <typename TA>
__device__ __forceinline__ double ld_a(const TA* A, int64_t idx) { return (double)A[idx]; }

// y_i = sum_{j>=i} M_ij x_j (row i of M = column i of Mt); identity when M is null.
// One CTA per row (rows round-robin over the grid), fixed-order block sums.
__device__ void trmv_rows(const IterArgs& a, const double* __restrict__ xin, double scale,
                          double* __restrict__ yout) {
    __shared__ double red_r[32];
    const int64_t n = a.n;
    if (!a.Mt) {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (int64_t)gridDim.x * blockDim.x)
            yout[i] = xin[i] * scale;
        return;
    }
    for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
        const double* row = a.Mt + i * n;
        double s = 0.0;
        for (int64_t j = i + threadIdx.x; j < n; j += blockDim.x) s = fma(row[j], xin[j], s);
        s = block_sum(s, red_r);
        if (threadIdx.x == 0) yout[i] = s * scale;
    }
}

// z_j = sum_{i<=j} M_ij g_i (column j of M); identity when M is null.  One
// CTA per column; f(z_j, j, lane) is called by thread 0 of that CTA with lane 0.
template <typename F>
__device__ void trmv_cols(const IterArgs& a, const double* __restrict__ gin, F f) {
    __shared__ double red_c[32];
    const int64_t n = a.n;
    if (!a.M) {
        for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
             j += (int64_t)gridDim.x * blockDim.x)
            f(gin[j], j, 0);
        return;
    }
    for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
        const double* col = a.M + j * n;
        double s = 0.0;
        for (int64_t i = threadIdx.x; i <= j; i += blockDim.x) s = fma(col[i], gin[i], s);
        s = block_sum(s, red_c);
        if (threadIdx.x == 0) f(s, j, 0);
    }
}

// Sum of per-CTA partial slot `slot`: warp 0 of every CTA runs the same
// fixed-order reduction (lanes strided over CTAs, then a butterfly), so all
// CTAs get identical bits; one warp keeps GB300's slow FP64 pipe lightly used.
__device__ __forceinline__ double sum_partials(const double* sp, int slot) {
    __shared__ double v_sp;
    __syncthreads();
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (unsigned c = threadIdx.x; c < gridDim.x; c += 32) s += sp[c * 4 + slot];
        s = warp_sum(s);
        if (threadIdx.x == 0) v_sp = s;
    }
    __syncthreads();
    const double r = v_sp;
    __syncthreads();
    return r;
}

// Block sum of a per-thread value, written by thread 0 to sp[cta*4 + slot].
__device__ __forceinline__ void write_partial(double v, double* sp, int slot, double* red) {
    v = block_sum(v, red);
    if (threadIdx.x == 0) sp[blockIdx.x * 4 + slot] = v;
}

// g_j = sum over CTAs of part[c][j]: one CTA per column, threads over the
// CTAs' partials, fixed-order block sum.
__device__ void reduce_columns(const IterArgs& a) {
    __shared__ double red_g[32];
    const int64_t n = a.n;
    for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
        double s = 0.0;
        for (unsigned c = threadIdx.x; c < gridDim.x; c += blockDim.x) s += a.part[(int64_t)c * n + j];
        s = block_sum(s, red_g);
        if (threadIdx.x == 0) a.g[j] = s;
    }
}

// Fused pass over A: for every row i,
//   t_i   = (A y)_i                         (skipped when c1 == 0)
//   new_i = c1 t_i + c2 old_i + c3 b_i      (old = a.u or a.ap, selected by mode)
// stores new_i, accumulates sum new_i^2 (slot 0) and sum b_i^2 (slot 3 if
// want_b2), and accumulates A^T new into part[cta][:].
template <typename TA, int NACC>
__device__ void row_pass(const IterArgs& a, double* __restrict__ smem, double c1, double c2,
                         double c3, double* __restrict__ vec, bool want_b2, bool accumulate_at) {
    const TA* A = static_cast<const TA*>(a.A);
    const int64_t m = a.m, n = a.n, lda = a.lda;
    const int R = a.R;
    const int ldt = R + 1;
    double* tile = smem;                          // n * (R+1)
    double* ys = tile + (size_t)n * ldt;          // n
    double* us = ys + n;                          // R
    double* red = us + 64;                        // 256 + 32
    const int tid = threadIdx.x;
    for (int64_t j = tid; j < n; j += IT_THREADS) ys[j] = a.y[j];
    double acc[NACC];
#pragma unroll
    for (int q = 0; q < NACC; ++q) acc[q] = 0.0;
    double sq = 0.0, b2 = 0.0;
    const int64_t ntiles = (m + R - 1) / R;
    const int NG = IT_THREADS / R;
    const int r_me = tid % R, grp = tid / R;
    __syncthreads();
    for (int64_t tile_i = blockIdx.x; tile_i < ntiles; tile_i += gridDim.x) {
        const int64_t i0 = tile_i * R;
        const int rows = (int)min((int64_t)R, m - i0);
        const int64_t tot = (int64_t)R * n;
        for (int64_t e = tid; e < tot; e += IT_THREADS) {
            const int r = (int)(e % R);
            const int64_t j = e / R;
            tile[j * ldt + r] = (r < rows) ? ld_a(A, i0 + r + j * lda) : 0.0;
        }
        __syncthreads();
        double t = 0.0;
        if (c1 != 0.0)
            for (int64_t j = grp; j < n; j += NG) t = fma(tile[j * ldt + r_me], ys[j], t);
        red[grp * R + r_me] = t;
        __syncthreads();
        if (tid < R) {
            double s = 0.0;
            for (int q = 0; q < NG; ++q) s += red[q * R + tid];
            double nv = 0.0;
            if (tid < rows) {
                const int64_t i = i0 + tid;
                const double bi = (c3 != 0.0 || want_b2) ? a.b[i] : 0.0;
                const double old = (c2 != 0.0) ? vec[i] : 0.0;
                nv = c1 * s + c2 * old + c3 * bi;
                vec[i] = nv;
                sq = fma(nv, nv, sq);
                if (want_b2) b2 = fma(bi, bi, b2);
            }
            us[tid] = nv;
        }
        __syncthreads();
        if (accumulate_at) {
#pragma unroll
            for (int q = 0; q < NACC; ++q) {
                const int64_t j = tid + (int64_t)q * IT_THREADS;
                if (j < n) {
                    const double* tc = tile + j * ldt;
                    double s = acc[q];
                    for (int r = 0; r < R; ++r) s = fma(tc[r], us[r], s);
                    acc[q] = s;
                }
            }
        }
        __syncthreads();
    }
    if (accumulate_at) {
#pragma unroll
        for (int q = 0; q < NACC; ++q) {
            const int64_t j = tid + (int64_t)q * IT_THREADS;
            if (j < n) a.part[(int64_t)blockIdx.x * n + j] = acc[q];
        }
    }
    write_partial(sq, a.sp, 0, red);
    if (want_b2) write_partial(b2, a.sp, 3, red);
}

// ---------------------------------------------------------------------------
// Streaming fused pass (n <= 1024): tiles of R rows x n columns, each column a
// 64-byte segment, staged through a 3-deep cp.async ring.  16-byte chunk c of
// column j sits at chunk position c ^ ((j >> 1) & 3): the A y phase reads 4
// whole columns per warp instruction and the A^T u phase reads one column per
// lane with 16-byte loads, both without bank conflicts.
//   FF = false: FP64 arithmetic (the plain FP64 path; storage double or float)
//   FF = true : float-float arithmetic on the FP32 pipe (storage float2 =
//               (hi, lo) split of FP64 data, or float); products are formed
//               exactly (fma error term) and summed with TwoSum.
// ---------------------------------------------------------------------------
constexpr int SEG = 64;
constexpr int STG = 3;
constexpr int STREAM_MAX_N = 1024;

template <typename ST> struct StT;
template <> struct StT<double> { static constexpr int B = 8; };
template <> struct StT<float> { static constexpr int B = 4; };
template <> struct StT<float2> { static constexpr int B = 8; };

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, int src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void split_ff(double v, float& h, float& l) {
    h = __double2float_rn(v);
    l = __double2float_rn(v - (double)h);
}

template <typename ST>
__device__ __forceinline__ void elem_hl(const uint8_t* seg, int rr, int j, float& h, float& l, double& d) {
    constexpr int B = StT<ST>::B;
    constexpr int rpc = 16 / B;
    const int off = ((((rr / rpc) ^ ((j >> 1) & 3))) << 4) + (rr % rpc) * B;
    if constexpr (sizeof(ST) == 8 && B == 8 && !std::is_same<ST, double>::value) {
        const float2 v = *(const float2*)(seg + off);
        h = v.x; l = v.y; d = (double)v.x + (double)v.y;
    } else if constexpr (std::is_same<ST, double>::value) {
        d = *(const double*)(seg + off);
        h = 0.f; l = 0.f;
    } else {
        h = *(const float*)(seg + off);
        l = 0.f;
        d = (double)h;
    }
}

template <typename ST>
__device__ __forceinline__ void issue_tile(const IterArgs& a, uint8_t* buf, int64_t tile, bool aligned16) {
    constexpr int B = StT<ST>::B;
    constexpr int R = SEG / B;
    constexpr int rpc = 16 / B;
    const ST* A = static_cast<const ST*>(a.A);
    const int64_t m = a.m, n = a.n, lda = a.lda;
    const int64_t row0 = tile * R;
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(buf);
    if (aligned16) {
        for (int64_t q = threadIdx.x; q < n * 4; q += blockDim.x) {
            const int64_t j = q >> 2;
            const int c = (int)(q & 3);
            const int64_t r = row0 + c * rpc;
            int64_t valid = m - r;
            valid = valid < 0 ? 0 : (valid > rpc ? rpc : valid);
            const ST* src = valid ? A + r + j * lda : A;
            cp_async16(sbase + (uint32_t)(j * SEG + ((c ^ ((j >> 1) & 3)) << 4)), src, (int)(valid * B));
        }
    } else {
        for (int64_t q = threadIdx.x; q < n * R; q += blockDim.x) {
            const int64_t j = q / R;
            const int rr = (int)(q % R);
            const int64_t r = row0 + rr;
            const bool valid = r < m;
            const ST* src = valid ? A + r + j * lda : A;
            const uint32_t dst = sbase + (uint32_t)(j * SEG + ((((rr / rpc) ^ ((j >> 1) & 3))) << 4) + (rr % rpc) * B);
            if (B == 8) cp_async8(dst, src, valid ? 8 : 0);
            else cp_async4(dst, src, valid ? 4 : 0);
        }
    }
}

template <typename ST, bool FF, int NACC>
__device__ void row_pass_stream(const IterArgs& a, double* __restrict__ smem_d, double c1, double c2,
                                double c3, double* __restrict__ vec, bool want_b2, bool accumulate_at) {
    constexpr int B = StT<ST>::B;
    constexpr int R = SEG / B;
    constexpr int CPI = 32 / R;                     // columns per warp instruction in the A y phase
    const int64_t m = a.m, n = a.n;
    uint8_t* tiles = (uint8_t*)smem_d;              // STG x n x 64 B
    double* ysd = smem_d + (size_t)STG * n * (SEG / 8);   // y: n doubles (FP64) or n float2 (FF)
    float2* ysf = (float2*)ysd;
    double* usd = ysd + n;                          // R doubles or R float2
    float2* usf = (float2*)usd;
    double* rowred = usd + 16;                      // 8 warps x R
    double* red = rowred + 8 * 16;                  // block reductions
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int64_t j = tid; j < n; j += blockDim.x) {
        const double yv = a.y[j];
        if (FF) { float h, l; split_ff(yv, h, l); ysf[j] = make_float2(h, l); }
        else ysd[j] = yv;
    }
    const bool aligned16 = ((a.lda * B) % 16 == 0) && (((uintptr_t)a.A & 15) == 0);
    float acch[NACC], accl[NACC];
    double accd[NACC];
#pragma unroll
    for (int q = 0; q < NACC; ++q) { acch[q] = 0.f; accl[q] = 0.f; accd[q] = 0.0; }
    double sq = 0.0, b2 = 0.0;
    const int64_t ntiles = (m + R - 1) / R;
    const int64_t G = gridDim.x;
    const size_t tile_bytes = (size_t)n * SEG;
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < STG - 1; ++s) {
        const int64_t t = blockIdx.x + (int64_t)s * G;
        if (t < ntiles) issue_tile<ST>(a, tiles + s * tile_bytes, t, aligned16);
        cp_commit();
    }
    const int rr_me = lane % R, co = lane / R;
#pragma unroll 1
    for (int64_t k = 0;; ++k) {
        const int64_t t = blockIdx.x + k * G;
        if (t >= ntiles) break;
        {
            const int64_t t2 = blockIdx.x + (k + STG - 1) * G;
            if (t2 < ntiles) issue_tile<ST>(a, tiles + ((k + STG - 1) % STG) * tile_bytes, t2, aligned16);
            cp_commit();
        }
        cp_wait<STG - 1>();
        __syncthreads();
        const uint8_t* tb = tiles + (k % STG) * tile_bytes;
        const int64_t i0 = t * R;
        const int rows = (int)min((int64_t)R, m - i0);
        // ---- (A y)_i for the R rows of the tile ----
        double part = 0.0;
        if (c1 != 0.0) {
            if (FF) {
                float sh = 0.f, sl = 0.f;
                for (int64_t j = co + (int64_t)CPI * warp; j < n; j += (int64_t)CPI * 8) {
                    float ah, al;
                    double dd;
                    elem_hl<ST>(tb + j * SEG, rr_me, (int)j, ah, al, dd);
                    const float2 y = ysf[j];
                    ff_madd(ah, al, y.x, y.y, sh, sl);
                }
                // combine the lanes of the same row in float-float (FP32 pipe)
#pragma unroll
                for (int o = R; o < 32; o <<= 1) {
                    const float oh = __shfl_xor_sync(0xffffffffu, sh, o);
                    const float ol = __shfl_xor_sync(0xffffffffu, sl, o);
                    float t;
                    two_sum(sh, oh, sh, t);
                    sl = sl + ol + t;
                }
                if (co == 0) ((float2*)rowred)[warp * 16 + rr_me] = make_float2(sh, sl);
            } else {
                for (int64_t j = co + (int64_t)CPI * warp; j < n; j += (int64_t)CPI * 8) {
                    float ah, al;
                    double dd;
                    elem_hl<ST>(tb + j * SEG, rr_me, (int)j, ah, al, dd);
                    part = fma(dd, ysd[j], part);
                }
            }
            if (!FF) {
#pragma unroll
                for (int o = R; o < 32; o <<= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                if (co == 0) rowred[warp * 16 + rr_me] = part;
            }
        }
        __syncthreads();
        if (tid < R) {
            double tsum = 0.0;
            if (c1 != 0.0) {
                if (FF)
                    for (int w = 0; w < 8; ++w) {
                        const float2 v = ((const float2*)rowred)[w * 16 + tid];
                        tsum += (double)v.x + (double)v.y;
                    }
                else
                    for (int w = 0; w < 8; ++w) tsum += rowred[w * 16 + tid];
            }
            double nv = 0.0;
            if (tid < rows) {
                const int64_t i = i0 + tid;
                const double bi = (c3 != 0.0 || want_b2) ? a.b[i] : 0.0;
                const double old = (c2 != 0.0) ? vec[i] : 0.0;
                nv = c1 * tsum + c2 * old + c3 * bi;
                vec[i] = nv;
                sq = fma(nv, nv, sq);
                if (want_b2) b2 = fma(bi, bi, b2);
            }
            if (FF) { float h, l; split_ff(nv, h, l); usf[tid] = make_float2(h, l); }
            else usd[tid] = nv;
        }
        __syncthreads();
        // ---- A^T u over the staged tile ----
        if (accumulate_at) {
#pragma unroll
            for (int q = 0; q < NACC; ++q) {
                const int64_t j = tid + (int64_t)q * blockDim.x;
                if (j < n) {
                    const uint8_t* seg = tb + j * SEG;
#pragma unroll
                    for (int rr = 0; rr < R; ++rr) {
                        float ah, al;
                        double dd;
                        elem_hl<ST>(seg, rr, (int)j, ah, al, dd);
                        if (FF) {
                            const float2 u = usf[rr];
                            ff_madd(ah, al, u.x, u.y, acch[q], accl[q]);
                        } else {
                            accd[q] = fma(dd, usd[rr], accd[q]);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
    cp_wait<0>();
    if (accumulate_at) {
#pragma unroll
        for (int q = 0; q < NACC; ++q) {
            const int64_t j = tid + (int64_t)q * blockDim.x;
            if (j < n) a.part[(int64_t)blockIdx.x * n + j] = FF ? ((double)acch[q] + (double)accl[q]) : accd[q];
        }
    }
    write_partial(sq, a.sp, 0, red);
    if (want_b2) write_partial(b2, a.sp, 3, red);
}

// Float-float pass specialised for (hi, lo) FP32 storage (8-byte elements,
// R = 8 rows per tile).  Same data flow as row_pass_stream, tuned for issue
// rate: in the A y phase a thread's swizzle position is the same for all of
// its columns ((j >> 1) & 3 is fixed by lane and warp), so addressing is a
// pointer increment, and four independent TwoSum chains hide latency; in the
// A^T u phase each 16-byte load brings two rows, u sits in registers, and
// each column keeps two chains.
template <int NACC>
__device__ void row_pass_ff2(const IterArgs& a, double* __restrict__ smem_d, double c1, double c2, double c3,
                             double* __restrict__ vec, bool want_b2, bool accumulate_at) {
    using ST = float2;
    constexpr int R = 8;
    const int64_t m = a.m, n = a.n;
    uint8_t* tiles = (uint8_t*)smem_d;
    double* ysd = smem_d + (size_t)STG * n * (SEG / 8);
    float2* ysf = (float2*)ysd;
    double* usd = ysd + n;
    float2* usf = (float2*)usd;
    double* rowred = usd + 16;
    double* red = rowred + 8 * 16;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int64_t j = tid; j < n; j += blockDim.x) {
        float h, l;
        split_ff(a.y[j], h, l);
        ysf[j] = make_float2(h, l);
    }
    const bool aligned16 = ((a.lda * 8) % 16 == 0) && (((uintptr_t)a.A & 15) == 0);
    float ach[NACC][2], acl[NACC][2];
#pragma unroll
    for (int q = 0; q < NACC; ++q) { ach[q][0] = ach[q][1] = acl[q][0] = acl[q][1] = 0.f; }
    double sq = 0.0, b2 = 0.0;
    const int64_t ntiles = (m + R - 1) / R;
    const int64_t G = gridDim.x;
    const size_t tile_bytes = (size_t)n * SEG;
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < STG - 1; ++s) {
        const int64_t t = blockIdx.x + (int64_t)s * G;
        if (t < ntiles) issue_tile<ST>(a, tiles + s * tile_bytes, t, aligned16);
        cp_commit();
    }
    // A y mapping: row rr of the tile, columns j = co + 4 warp + 32 k
    const int rr = lane & 7, co = lane >> 3;
    const int j0 = co + 4 * warp;
    const int off_y = ((((rr >> 1) ^ ((j0 >> 1) & 3))) << 4) + ((rr & 1) << 3);
#pragma unroll 1
    for (int64_t k = 0;; ++k) {
        const int64_t t = blockIdx.x + k * G;
        if (t >= ntiles) break;
        {
            const int64_t t2 = blockIdx.x + (k + STG - 1) * G;
            if (t2 < ntiles) issue_tile<ST>(a, tiles + ((k + STG - 1) % STG) * tile_bytes, t2, aligned16);
            cp_commit();
        }
        cp_wait<STG - 1>();
        __syncthreads();
        const uint8_t* tb = tiles + (k % STG) * tile_bytes;
        const int64_t i0 = t * R;
        const int rows = (int)min((int64_t)R, m - i0);
        if (c1 != 0.0) {
            float h[4] = {0.f, 0.f, 0.f, 0.f}, l[4] = {0.f, 0.f, 0.f, 0.f};
            const uint8_t* pa = tb + (size_t)j0 * SEG + off_y;
            int64_t j = j0;
            for (; j + 96 < n; j += 128, pa += 128 * SEG) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float2 av = *(const float2*)(pa + u * 32 * SEG);
                    const float2 yv = ysf[j + 32 * u];
                    ff_madd(av.x, av.y, yv.x, yv.y, h[u], l[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < 3; ++u) {       // at most three columns remain
                if (j + 32 * u < n) {
                    const float2 av = *(const float2*)(pa + u * 32 * SEG);
                    const float2 yv = ysf[j + 32 * u];
                    ff_madd(av.x, av.y, yv.x, yv.y, h[u], l[u]);
                }
            }
            ff_acc(h[0], l[0], h[1], l[1]);
            ff_acc(h[2], l[2], h[3], l[3]);
            ff_acc(h[0], l[0], h[2], l[2]);
#pragma unroll
            for (int o = 8; o < 32; o <<= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, h[0], o);
                const float ol = __shfl_xor_sync(0xffffffffu, l[0], o);
                ff_acc(h[0], l[0], oh, ol);
            }
            if (co == 0) ((float2*)rowred)[warp * 16 + rr] = make_float2(h[0], l[0]);
        }
        __syncthreads();
        if (tid < R) {
            double tsum = 0.0;
            if (c1 != 0.0)
                for (int w = 0; w < 8; ++w) {
                    const float2 v = ((const float2*)rowred)[w * 16 + tid];
                    tsum += (double)v.x + (double)v.y;
                }
            double nv = 0.0;
            if (tid < rows) {
                const int64_t i = i0 + tid;
                const double bi = (c3 != 0.0 || want_b2) ? a.b[i] : 0.0;
                const double old = (c2 != 0.0) ? vec[i] : 0.0;
                nv = c1 * tsum + c2 * old + c3 * bi;
                vec[i] = nv;
                sq = fma(nv, nv, sq);
                if (want_b2) b2 = fma(bi, bi, b2);
            }
            float hh, ll;
            split_ff(nv, hh, ll);
            usf[tid] = make_float2(hh, ll);
        }
        __syncthreads();
        if (accumulate_at) {
            float uh[R], ul[R];
#pragma unroll
            for (int r = 0; r < R; ++r) { const float2 uv = usf[r]; uh[r] = uv.x; ul[r] = uv.y; }
#pragma unroll
            for (int q = 0; q < NACC; ++q) {
                const int64_t j = tid + (int64_t)q * blockDim.x;
                if (j < n) {
                    const uint8_t* seg = tb + j * SEG;
                    const int sw = (int)((j >> 1) & 3);
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const float4 v = *(const float4*)(seg + ((c ^ sw) << 4));   // rows 2c, 2c+1
                        ff_madd(v.x, v.y, uh[2 * c], ul[2 * c], ach[q][0], acl[q][0]);
                        ff_madd(v.z, v.w, uh[2 * c + 1], ul[2 * c + 1], ach[q][1], acl[q][1]);
                    }
                }
            }
        }
        __syncthreads();
    }
    cp_wait<0>();
    if (accumulate_at) {
#pragma unroll
        for (int q = 0; q < NACC; ++q) {
            const int64_t j = tid + (int64_t)q * blockDim.x;
            if (j < n) {
                ff_acc(ach[q][0], acl[q][0], ach[q][1], acl[q][1]);
                a.part[(int64_t)blockIdx.x * n + j] = (double)ach[q][0] + (double)acl[q][0];
            }
        }
    }
    write_partial(sq, a.sp, 0, red);
    if (want_b2) write_partial(b2, a.sp, 3, red);
}

// MODE 0: general staging pass (any n <= 4096), FP64
// MODE 1: streaming pass, FP64 arithmetic, storage TA
// MODE 2: streaming pass, float-float arithmetic, storage float2 (TA = double, split copy) or float
template <typename TA, int NACC, int MODE>
__device__ __forceinline__ void do_pass(const IterArgs& a, double* smem, double c1, double c2, double c3,
                                        double* vec, bool want_b2, bool acc_at) {
    if constexpr (MODE == 0) row_pass<TA, NACC>(a, smem, c1, c2, c3, vec, want_b2, acc_at);
    else if constexpr (MODE == 1) row_pass_stream<TA, false, NACC>(a, smem, c1, c2, c3, vec, want_b2, acc_at);
    else if constexpr (std::is_same<TA, double>::value)
        row_pass_ff2<NACC>(a, smem, c1, c2, c3, vec, want_b2, acc_at);
    else row_pass_stream<float, true, NACC>(a, smem, c1, c2, c3, vec, want_b2, acc_at);
}

__device__ __forceinline__ double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

// solvers.rs:84-102
__device__ __forceinline__ void sym_ortho(double a, double b, double& c, double& s, double& r) {
    if (b == 0.0) { c = sgn(a); s = 0.0; r = fabs(a); return; }
    if (a == 0.0) { c = 0.0; s = sgn(b); r = fabs(b); return; }
    if (fabs(b) > fabs(a)) {
        const double tau = a / b;
        s = sgn(b) / sqrt(1.0 + tau * tau);
        c = s * tau;
        r = b / s;
    } else {
        const double tau = b / a;
        c = sgn(a) / sqrt(1.0 + tau * tau);
        s = c * tau;
        r = a / c;
    }
}

template <typename TA, int NACC, int MODE>
__global__ void __launch_bounds__(IT_THREADS) lsqr_kernel(IterArgs a) {
    extern __shared__ double smem[];
    double* red = smem + a.red_off;
    const int64_t n = a.n;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
    const double eps = 2.220446049250313e-16;
    const double dampsq = a.damp * a.damp;

    // ---- initialisation (solvers.rs:141-182) ----
    for (int64_t j = gt; j < n; j += gthreads) {
        a.x[j] = a.x0 ? a.x0[j] : 0.0;
        if (a.calc_var) a.var[j] = 0.0;
    }
    if (a.x0) trmv_rows(a, a.x0, 1.0, a.y);
    if (!grid_sync(a.bar)) return;
    // u = b - A M x0  (or b), beta^2, ||b||^2, A^T u partials
    do_pass<TA, NACC, MODE>(a, smem, a.x0 ? -1.0 : 0.0, 0.0, 1.0, a.u, true, true);
    if (!grid_sync(a.bar)) return;
    double beta = sqrt(sum_partials(a.sp, 0));
    const double bnorm = sqrt(sum_partials(a.sp, 3));
    reduce_columns(a);
    if (!grid_sync(a.bar)) return;
    {
        const double sc = beta > 0.0 ? 1.0 / beta : 0.0;
        double aq = 0.0;
        trmv_cols(a, a.g, [&](double z, int64_t j, int lane) {
            const double vv = z * sc;
            if (lane == 0) { a.vun[j] = vv; aq = fma(vv, vv, aq); }
        });
        write_partial(aq, a.sp, 1, red);
    }
    if (!grid_sync(a.bar)) return;
    double alfa = sqrt(sum_partials(a.sp, 1));
    double us = beta > 0.0 ? 1.0 / beta : 0.0;     // u is stored unnormalised
    {
        const double sa = alfa > 0.0 ? 1.0 / alfa : 0.0;
        for (int64_t j = gt; j < n; j += gthreads) {
            const double vv = a.vun[j] * sa;
            a.v[j] = vv;
            a.w[j] = vv;
        }
        trmv_rows(a, a.vun, sa, a.y);
    }
    double rhobar = alfa, phibar = beta, rnorm = beta, r1norm = beta, r2norm = beta;
    double anorm = 0.0, acond = 0.0, ddnorm = 0.0, res2 = 0.0, xnorm = 0.0, xxnorm = 0.0, z = 0.0;
    double cs2 = -1.0, sn2 = 0.0;
    double arnorm = alfa * beta;
    int64_t itn = 0;
    int istop = 0;
    if (arnorm == 0.0) {
        if (gt == 0) {
            a.out[0] = 0; a.out[1] = 0; a.out[2] = beta; a.out[3] = beta;
            a.out[4] = 0; a.out[5] = 0; a.out[6] = 0; a.out[7] = 0;
            if (a.arn) a.arn[0] = 0.0;
        }
        return;
    }
    const double ctol = a.conlim > 0.0 ? 1.0 / a.conlim : 0.0;
    if (!grid_sync(a.bar)) return;

    while (itn < a.iter_lim) {
        if (gt == 0 && a.arn) a.arn[itn] = arnorm;
        ++itn;
        // u = A M v - alfa u ; A^T u partials  (solvers.rs:194-195)
        do_pass<TA, NACC, MODE>(a, smem, 1.0, -alfa * us, 0.0, a.u, false, true);
        if (!grid_sync(a.bar)) return;
        beta = sqrt(sum_partials(a.sp, 0));
        reduce_columns(a);
        if (!grid_sync(a.bar)) return;
        // v = M^T A^T u / beta - beta v ; ||v||^2 and ||w||^2 partials (solvers.rs:197-204)
        {
            const double sc = beta > 0.0 ? 1.0 / beta : 0.0;
            double aq = 0.0, wq = 0.0;
            if (beta > 0.0) {
                trmv_cols(a, a.g, [&](double zz, int64_t j, int lane) {
                    if (lane == 0) {
                        const double vv = zz * sc - beta * a.v[j];
                        a.vun[j] = vv;
                        aq = fma(vv, vv, aq);
                    }
                });
            }
            for (int64_t j = gt; j < n; j += gthreads) wq = fma(a.w[j], a.w[j], wq);
            write_partial(aq, a.sp, 1, red);
            write_partial(wq, a.sp, 2, red);
        }
        if (!grid_sync(a.bar)) return;
        const double wsq = sum_partials(a.sp, 2);
        if (beta > 0.0) {
            us = 1.0 / beta;
            anorm = sqrt(anorm * anorm + alfa * alfa + beta * beta + dampsq);
            alfa = sqrt(sum_partials(a.sp, 1));
        }
        // plane rotations (solvers.rs:207-219)
        const double rhobar1 = sqrt(rhobar * rhobar + dampsq);
        const double cs1 = rhobar / rhobar1;
        const double sn1 = a.damp / rhobar1;
        const double psi = sn1 * phibar;
        phibar *= cs1;
        double cs, sn, rho;
        sym_ortho(rhobar1, beta, cs, sn, rho);
        const double theta = sn * alfa;
        rhobar = -cs * alfa;
        const double phi = cs * phibar;
        phibar *= sn;
        const double tau = sn * phi;
        const double t1 = phi / rho;
        const double t2 = -theta / rho;
        // x += t1 w ; w = v + t2 w ; var += (w/rho)^2  (solvers.rs:222-232)
        {
            const double sa = (beta > 0.0) ? (alfa > 0.0 ? 1.0 / alfa : 0.0) : 0.0;
            const double irho = 1.0 / rho;
            for (int64_t j = gt; j < n; j += gthreads) {
                const double vv = (beta > 0.0) ? a.vun[j] * sa : a.v[j];
                a.v[j] = vv;
                const double wj = a.w[j];
                a.x[j] = fma(t1, wj, a.x[j]);
                a.w[j] = fma(t2, wj, vv);
                if (a.calc_var) {
                    const double dk = wj * irho;
                    a.var[j] = fma(dk, dk, a.var[j]);
                }
            }
            if (beta > 0.0) trmv_rows(a, a.vun, sa, a.y);
        }
        ddnorm += wsq / (rho * rho);
        // norm estimates and stopping tests (solvers.rs:235-272)
        const double delta = sn2 * rho;
        const double gambar = -cs2 * rho;
        const double rhs = phi - delta * z;
        const double zbar = rhs / gambar;
        xnorm = sqrt(xxnorm + zbar * zbar);
        const double gamma = sqrt(gambar * gambar + theta * theta);
        cs2 = gambar / gamma;
        sn2 = theta / gamma;
        z = rhs / gamma;
        xxnorm += z * z;
        acond = anorm * sqrt(ddnorm);
        const double res1 = phibar * phibar;
        res2 += psi * psi;
        rnorm = sqrt(res1 + res2);
        arnorm = alfa * fabs(tau);
        const double r1sq = rnorm * rnorm - dampsq * xxnorm;
        r1norm = sqrt(fabs(r1sq));
        r2norm = rnorm;
        const double test1 = rnorm / bnorm;
        const double test2 = arnorm / (anorm * rnorm + eps);
        const double test3 = 1.0 / (acond + eps);
        const double tt1 = test1 / (1.0 + anorm * xnorm / bnorm);
        const double rtol = a.atol + a.btol * (anorm * xnorm / bnorm);
        if (itn >= a.iter_lim) istop = 7;
        if (1.0 + test3 <= 1.0) istop = 6;
        if (1.0 + test2 <= 1.0) istop = 5;
        if (1.0 + tt1 <= 1.0) istop = 4;
        if (test3 <= ctol) istop = 3;
        if (test2 <= a.atol) istop = 2;
        if (test1 <= rtol) istop = 1;
        if (a.abs_tol > 0.0 && arnorm < a.abs_tol && (istop == 0 || istop == 7)) istop = 2;
        if (!grid_sync(a.bar)) return;
        if (istop != 0) break;
    }
    if (gt == 0) {
        a.out[0] = istop; a.out[1] = (double)itn; a.out[2] = r1norm; a.out[3] = r2norm;
        a.out[4] = anorm; a.out[5] = acond; a.out[6] = xnorm; a.out[7] = arnorm;
    }
}

// CGLS (cg.rs:18-61) on A M.  p lives in a.w, s_new in a.vun, ap in a.ap, r in a.u.
template <typename TA, int NACC, int MODE>
__global__ void __launch_bounds__(IT_THREADS) cgls_kernel(IterArgs a) {
    extern __shared__ double smem[];
    double* red = smem + a.red_off;
    const int64_t n = a.n;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
    const double tol = a.abs_tol;

    for (int64_t j = gt; j < n; j += gthreads) a.x[j] = a.x0 ? a.x0[j] : 0.0;
    if (a.x0) trmv_rows(a, a.x0, 1.0, a.y);
    if (!grid_sync(a.bar)) return;
    // r = b - A M x ; partials of A^T r   (cg.rs:32-33)
    do_pass<TA, NACC, MODE>(a, smem, a.x0 ? -1.0 : 0.0, 0.0, 1.0, a.u, false, true);
    if (!grid_sync(a.bar)) return;
    reduce_columns(a);
    if (!grid_sync(a.bar)) return;
    {
        double sq = 0.0;
        trmv_cols(a, a.g, [&](double zz, int64_t j, int lane) {
            if (lane == 0) { a.vun[j] = zz; a.w[j] = zz; sq = fma(zz, zz, sq); }
        });
        write_partial(sq, a.sp, 1, red);
    }
    if (!grid_sync(a.bar)) return;
    double norm_s = sum_partials(a.sp, 1);
    trmv_rows(a, a.w, 1.0, a.y);                 // y = M p
    if (!grid_sync(a.bar)) return;
    int64_t it = 0;
    int converged = 0;
    for (int64_t i = 0; i < a.iter_lim; ++i) {
        // ap = A M p ; ||ap||^2   (cg.rs:38-39)
        do_pass<TA, NACC, MODE>(a, smem, 1.0, 0.0, 0.0, a.ap, false, false);
        if (!grid_sync(a.bar)) return;
        const double apap = sum_partials(a.sp, 0);
        const double alpha = norm_s / apap;
        // x += alpha p ; r -= alpha ap fused with A^T r  (cg.rs:40-42)
        for (int64_t j = gt; j < n; j += gthreads) a.x[j] = fma(alpha, a.w[j], a.x[j]);
        {
            IterArgs b2 = a;
            b2.b = a.ap;   // reuse the "b" slot for ap: new_i = 1 * r_i - alpha * ap_i
            do_pass<TA, NACC, MODE>(b2, smem, 0.0, 1.0, -alpha, a.u, false, true);
        }
        if (!grid_sync(a.bar)) return;
        reduce_columns(a);
        if (!grid_sync(a.bar)) return;
        {
            double sq = 0.0;
            trmv_cols(a, a.g, [&](double zz, int64_t j, int lane) {
                if (lane == 0) { a.vun[j] = zz; sq = fma(zz, zz, sq); }
            });
            write_partial(sq, a.sp, 1, red);
        }
        if (!grid_sync(a.bar)) return;
        const double norm_s_new = sum_partials(a.sp, 1);
        it = i + 1;
        if (sqrt(norm_s_new) < tol) { converged = 1; break; }   // cg.rs:46-50
        const double beta = norm_s_new / norm_s;
        norm_s = norm_s_new;
        // p = s + beta p ; y = M s + beta y   (cg.rs:52-54)
        for (int64_t j = gt; j < n; j += gthreads) a.w[j] = fma(beta, a.w[j], a.vun[j]);
        if (a.Mt) {
            __shared__ double red_y[32];
            for (int64_t r = blockIdx.x; r < n; r += gridDim.x) {
                const double* row = a.Mt + r * n;
                double s = 0.0;
                for (int64_t j = r + threadIdx.x; j < n; j += blockDim.x) s = fma(row[j], a.vun[j], s);
                s = block_sum(s, red_y);
                if (threadIdx.x == 0) a.y[r] = fma(beta, a.y[r], s);
            }
        } else {
            for (int64_t r = gt; r < n; r += gthreads) a.y[r] = fma(beta, a.y[r], a.vun[r]);
        }
        if (!grid_sync(a.bar)) return;
    }
    if (gt == 0) {
        a.out[0] = converged; a.out[1] = (double)it;
    }
}

// ---------------------------------------------------------------------------
// FP64 -> (hi, lo) FP32 split with integer operations (no FP64 arithmetic):
// hi = v rounded to 24 bits, lo = the remainder rounded to 24 bits, so
// hi + lo carries 48 bits of v.  Values outside the FP32 exponent window
// fall back to conversions.
// ---------------------------------------------------------------------------
__global__ void split_ff_kernel(const double* __restrict__ A, int64_t m, int64_t n, int64_t lda,
                                float2* __restrict__ out, int64_t ldo) {
    const int64_t total = m * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % m, j = e / m;
        out[i + j * ldo] = ff_split(A[i + j * lda]);
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int pick_R(int64_t n) {
    const int64_t budget = 96 * 1024 / 8;          // doubles for the staged tile
    int R = 64;
    while (R > 1 && (int64_t)(R + 1) * n > budget) R >>= 1;
    return R;
}

// shared-memory size and reduction-scratch offset of each pass
static size_t iter_smem(int mode, int64_t n, int R, int64_t& red_off) {
    if (mode == 0) red_off = n * (R + 1) + n + 64;
    else red_off = (int64_t)STG * n * (SEG / 8) + n + 16 + 8 * 16;
    return (size_t)(red_off + IT_THREADS + 32) * sizeof(double);
}

struct IterBufs {
    DevBuf<double> u, v, vun, w, y, g, part, sp, ap, out, xbuf, Mt;
    DevBuf<unsigned int> bar;
    DevBuf<float2> aff;
};

static int coop_grid(Ctx& ctx, const void* kernel, size_t smem) {
    if (smem > 48 * 1024)
        set_smem_limit((const void*)kernel, smem);
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, IT_THREADS, smem));
    if (nb < 1) fail(RNLA_ERR_UNSUPPORTED, "iterative kernel does not fit on an SM");
    if (nb > 4) nb = 4;
    return nb * ctx.sm_count;
}

static void setup(Ctx& ctx, IterArgs& a, IterBufs& B, const void* A, int64_t m, int64_t n, int64_t lda,
                  const double* M, int G) {
    cudaStream_t s = ctx.stream;
    B.u.alloc(m, s); B.ap.alloc(m, s);
    B.v.alloc(n, s); B.vun.alloc(n, s); B.w.alloc(n, s); B.y.alloc(n, s); B.g.alloc(n, s);
    B.part.alloc((size_t)G * n, s); B.sp.alloc((size_t)G * 4, s); B.out.alloc(8, s);
    B.bar.alloc(2, s);
    RNLA_CUDA(cudaMemsetAsync(B.bar.get(), 0, 2 * sizeof(unsigned int), s));
    RNLA_CUDA(cudaMemsetAsync(B.out.get(), 0, 8 * sizeof(double), s));
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), s));
    a.A = A; a.m = m; a.n = n; a.lda = lda;
    a.M = M; a.Mt = nullptr;
    if (M) {
        B.Mt.alloc((size_t)n * n, s);
        transpose(ctx, n, n, M, n, B.Mt, n);
        a.Mt = B.Mt.get();
    }
    a.u = B.u; a.ap = B.ap; a.v = B.v; a.vun = B.vun; a.w = B.w; a.y = B.y; a.g = B.g;
    a.part = B.part; a.sp = B.sp; a.out = B.out;
    a.bar.count = B.bar.get(); a.bar.gen = B.bar.get() + 1; a.bar.status = ctx.status;
    a.R = pick_R(n);
}

template <typename TA, int MODE, bool LSQR>
static const void* kernel_for(int64_t n) {
    const int nacc = (int)((n + IT_THREADS - 1) / IT_THREADS);
    if constexpr (MODE == 0) {
        (void)nacc;
        if (LSQR) return (const void*)lsqr_kernel<TA, 16, 0>;
        return (const void*)cgls_kernel<TA, 16, 0>;
    } else {
        if (nacc <= 1) return LSQR ? (const void*)lsqr_kernel<TA, 1, MODE> : (const void*)cgls_kernel<TA, 1, MODE>;
        if (nacc <= 2) return LSQR ? (const void*)lsqr_kernel<TA, 2, MODE> : (const void*)cgls_kernel<TA, 2, MODE>;
        return LSQR ? (const void*)lsqr_kernel<TA, 4, MODE> : (const void*)cgls_kernel<TA, 4, MODE>;
    }
}

template <bool LSQR>
static const void* select_kernel(bool a32, int mode, int64_t n) {
    if (a32) {
        if (mode == 0) return kernel_for<float, 0, LSQR>(n);
        if (mode == 1) return kernel_for<float, 1, LSQR>(n);
        return kernel_for<float, 2, LSQR>(n);
    }
    if (mode == 0) return kernel_for<double, 0, LSQR>(n);
    if (mode == 1) return kernel_for<double, 1, LSQR>(n);
    return kernel_for<double, 2, LSQR>(n);
}

static void launch_coop(Ctx& ctx, const void* kernel, int G, size_t smem, IterArgs& a) {
    void* params[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(G), dim3(IT_THREADS), params, smem, ctx.stream));
    count_launch();
}

// Prepares the kernel choice, the grid and (for float-float on FP64 data) the
// split copy of A; returns the kernel.
static const void* prepare(Ctx& ctx, bool lsqr, IterArgs& a, IterBufs& B, const double* a64, const float* a32,
                           int64_t m, int64_t n, int64_t lda, const double* M, bool ffp, int& G, size_t& smem) {
    const int mode = (n <= STREAM_MAX_N) ? (ffp ? 2 : 1) : 0;
    const void* k = lsqr ? select_kernel<true>(a32 != nullptr, mode, n) : select_kernel<false>(a32 != nullptr, mode, n);
    int64_t red_off = 0;
    smem = iter_smem(mode, n, pick_R(n), red_off);
    G = coop_grid(ctx, k, smem);
    const void* Aptr = a32 ? (const void*)a32 : (const void*)a64;
    int64_t ld = lda;
    if (mode == 2 && !a32) {
        const int64_t ldo = (m + 7) & ~7LL;
        B.aff.alloc((size_t)ldo * n, ctx.stream);
        int g = div_up(m * n, 256);
        if (g > 16 * ctx.sm_count) g = 16 * ctx.sm_count;
        split_ff_kernel<<<g, 256, 0, ctx.stream>>>(a64, m, n, lda, B.aff, ldo);
        RNLA_LAUNCH_CHECK();
        Aptr = B.aff.get();
        ld = ldo;
    }
    setup(ctx, a, B, Aptr, m, n, ld, M, G);
    a.red_off = red_off;
    return k;
}

LsqrResult lsqr_solve(Ctx& ctx, const double* a64, const float* a32, int64_t m, int64_t n,
                      int64_t lda, const double* M, const double* b, const double* x0,
                      const LsqrParams& prm, double* x, double* var, double* arnorms_dev, bool ffp,
                      const LsqrFFInput* pre, LsqrPending* pend) {
    if (n > (int64_t)IT_THREADS * IT_MAXACC)
        fail(RNLA_ERR_UNSUPPORTED, "lsqr: n > 4096 is not supported by the fused kernel");
    if (ffp && lsqr_ff_supported(n)) {
        const void* A = a64 ? (const void*)a64 : (const void*)a32;
        return lsqr_ff_solve(ctx, A, a64 == nullptr, m, n, lda, M, b, x0, prm, x, var, arnorms_dev, pre, pend);
    }
    IterArgs a;
    IterBufs B;
    int G;
    size_t smem;
    const void* k = prepare(ctx, true, a, B, a64, a32, m, n, lda, M, ffp, G, smem);
    a.b = b; a.x0 = x0; a.x = x; a.var = var; a.arn = arnorms_dev;
    a.damp = prm.damp; a.atol = prm.atol; a.btol = prm.btol; a.conlim = prm.conlim;
    a.abs_tol = prm.abs_arnorm_tol;
    a.iter_lim = prm.iter_lim < 0 ? 2 * n : prm.iter_lim;
    a.calc_var = (prm.calc_var && var) ? 1 : 0;
    launch_coop(ctx, k, G, smem, a);
    double out[8];
    RNLA_CUDA(cudaMemcpyAsync(out, B.out.get(), sizeof out, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.check_status("lsqr");
    LsqrResult r;
    r.istop = (int64_t)out[0]; r.itn = (int64_t)out[1];
    r.r1norm = out[2]; r.r2norm = out[3]; r.anorm = out[4]; r.acond = out[5]; r.xnorm = out[6];
    r.arnorm = out[7];
    return r;
}

int64_t cgls_solve(Ctx& ctx, const double* a64, const float* a32, int64_t m, int64_t n, int64_t lda,
                   const double* M, const double* b, const double* x0, double tolerance,
                   int64_t num_iterations, double* x, bool* converged) {
    if (n > (int64_t)IT_THREADS * IT_MAXACC)
        fail(RNLA_ERR_UNSUPPORTED, "cgls: n > 4096 is not supported by the fused kernel");
    IterArgs a;
    IterBufs B;
    int G;
    size_t smem;
    const void* k = prepare(ctx, false, a, B, a64, a32, m, n, lda, M, false, G, smem);
    a.b = b; a.x0 = x0; a.x = x; a.var = nullptr; a.arn = nullptr;
    a.abs_tol = tolerance; a.iter_lim = num_iterations; a.calc_var = 0;
    a.damp = 0; a.atol = 0; a.btol = 0; a.conlim = 0;
    launch_coop(ctx, k, G, smem, a);
    double out[8];
    RNLA_CUDA(cudaMemcpyAsync(out, B.out.get(), sizeof out, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.check_status("cgls");
    if (converged) *converged = out[0] != 0.0;
    return (int64_t)out[1];
}

// Bytes of caller-provided workspace lsqr_run_in_workspace needs for an
// m x n problem on a device with `sm_count` SMs (FP64 arithmetic, no
// preconditioner).  Sets *grid to the cooperative grid it will use.
size_t lsqr_workspace_bytes(int64_t m, int64_t n, int sm_count, int* grid, size_t* smem_out,
                            const void** kernel_out) {
    // the kernels hold each thread's share of the n-vectors in registers:
    // columns beyond IT_THREADS * IT_MAXACC would never be written
    if (n > (int64_t)IT_THREADS * IT_MAXACC)
        fail(RNLA_ERR_UNSUPPORTED, "lsqr: n > 4096 is not supported by the fused kernel");
    const int mode = (n <= STREAM_MAX_N) ? 1 : 0;
    const void* k = select_kernel<true>(false, mode, n);
    int64_t red_off = 0;
    const size_t smem = iter_smem(mode, n, pick_R(n), red_off);
    if (smem > 48 * 1024)
        set_smem_limit((const void*)k, smem);
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, IT_THREADS, smem));
    if (nb < 1) fail(RNLA_ERR_UNSUPPORTED, "iterative kernel does not fit on an SM");
    if (nb > 4) nb = 4;
    const int G = nb * sm_count;
    if (grid) *grid = G;
    if (smem_out) *smem_out = smem;
    if (kernel_out) *kernel_out = k;
    // words (status, barrier) | out[8] | sp[G*4] | u[m] | v, vun, w, y, g [5n] | part[G*n]
    return sizeof(double) * (size_t)(2 + 8 + 4 * (int64_t)G + m + 5 * n + (int64_t)G * n);
}

// LSQR (FP64 arithmetic, no preconditioner) with every scratch buffer carved
// out of `ws` (lsqr_workspace_bytes bytes, 256-byte aligned).  Performs no
// allocation: the status word, barrier words and result record inside `ws`
// are cleared with cudaMemsetAsync, everything else is written by the
// kernel before it is read.
LsqrResult lsqr_run_in_workspace(cudaStream_t stream, int sm_count, void* ws, size_t ws_bytes,
                                 const double* a64, int64_t m, int64_t n, int64_t lda, const double* b,
                                 const double* x0, const LsqrParams& prm, double* x) {
    int G = 0;
    size_t smem = 0;
    const void* k = nullptr;
    const size_t need = lsqr_workspace_bytes(m, n, sm_count, &G, &smem, &k);
    if (need > ws_bytes) fail(RNLA_ERR_INVALID_DIMENSIONS, "workspace too small");
    double* d = static_cast<double*>(ws);
    unsigned int* words = reinterpret_cast<unsigned int*>(d);   // [0] status, [1] count, [2] gen
    double* out = d + 2;
    double* sp = out + 8;
    double* u = sp + 4 * (int64_t)G;
    double* v = u + m;
    double* vun = v + n;
    double* w = vun + n;
    double* y = w + n;
    double* g = y + n;
    double* part = g + n;
    RNLA_CUDA(cudaMemsetAsync(d, 0, sizeof(double) * 10, stream));
    IterArgs a;
    a.A = a64; a.m = m; a.n = n; a.lda = lda;
    a.M = nullptr; a.Mt = nullptr;
    a.b = b; a.x0 = x0;
    a.u = u; a.ap = u; a.v = v; a.vun = vun; a.w = w; a.x = x; a.y = y; a.g = g;
    a.part = part; a.sp = sp; a.var = nullptr; a.arn = nullptr; a.out = out;
    a.damp = prm.damp; a.atol = prm.atol; a.btol = prm.btol; a.conlim = prm.conlim;
    a.abs_tol = prm.abs_arnorm_tol;
    a.iter_lim = prm.iter_lim < 0 ? 2 * n : prm.iter_lim;
    a.calc_var = 0;
    a.bar.status = words;
    a.bar.count = words + 1;
    a.bar.gen = words + 2;
    a.R = pick_R(n);
    const int mode = (n <= STREAM_MAX_N) ? 1 : 0;
    int64_t red_off = 0;
    iter_smem(mode, n, a.R, red_off);
    a.red_off = red_off;
    void* params[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3(G), dim3(IT_THREADS), params, smem, stream));
    count_launch();
    double h[8];
    unsigned int st = 0;
    RNLA_CUDA(cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, stream));
    RNLA_CUDA(cudaMemcpyAsync(&st, words, sizeof st, cudaMemcpyDeviceToHost, stream));
    RNLA_CUDA(cudaStreamSynchronize(stream));
    if (st == KSTATUS_BARRIER_TIMEOUT) fail(RNLA_ERR_TIMEOUT, "lsqr: a grid barrier exceeded its limit");
    if (st != 0) fail(RNLA_ERR_COMPUTATION, "lsqr: device status set");
    LsqrResult r;
    r.istop = (int64_t)h[0]; r.itn = (int64_t)h[1];
    r.r1norm = h[2]; r.r2norm = h[3]; r.anorm = h[4]; r.acond = h[5]; r.xnorm = h[6]; r.arnorm = h[7];
    return r;
}

__global__ void trmv_upper_kernel(const double* __restrict__ M, int64_t n, int64_t ldm,
                                  const double* __restrict__ x, double* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwg = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = gw; i < n; i += nwg) {
        double s = 0.0;
        for (int64_t j = i + lane; j < n; j += 32) s = fma(M[i + j * ldm], x[j], s);
        s = warp_sum(s);
        if (lane == 0) y[i] = s;
    }
}

void trmv_upper(Ctx& ctx, const double* M, int64_t n, int64_t ldm, const double* x, double* y) {
    if (n <= 0) return;
    int g = div_up(n * 32, 256);
    if (g > 4 * ctx.sm_count) g = 4 * ctx.sm_count;
    trmv_upper_kernel<<<g, 256, 0, ctx.stream>>>(M, n, ldm, x, y);
    RNLA_LAUNCH_CHECK();
}

}  // namespace rnla
