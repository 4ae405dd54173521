// Float-float Householder QR and triangular inverse for the BF16X
// precision's preconditioner (sketch_and_precondition.rs:53-55: QR of the
// sketch S A, R^-1).  Arithmetic is float-float on the FP32 pipe: on GB300 a
// dependent FP64 operation takes ~64 cycles and a divide or square root
// several hundred, and a QR of a d x n sketch is a chain of n dependent
// column steps, so the length of that chain sets its time.
//
// QR.  Columns are grouped in blocks of KB = 4; block b is owned by CTA
// b mod G, which keeps its columns in shared memory (512 threads, rows
// strided over the threads).  The owner of a block factors it column by
// column (LAPACK dlarfg reflectors: beta = -sign(alpha) ||(alpha, x)||,
// v = x / (alpha - beta), tau = (beta - alpha) / beta, tau = 0 when x is
// exactly zero), forms the block's triangular factor T (dlarft, forward,
// columnwise) so that H_0 H_1 H_2 H_3 = I - V T V^T, publishes V, T and a
// flag.  On seeing flag rb a CTA bulk-copies V and T of block rb into shared
// memory and applies Q_rb^T = I - V T^T V^T to its later blocks -- the owner
// of block rb + 1 first, which then factors that block (look-ahead).  One
// cross-CTA hand-off and one batched reduction per block of 4 columns sit on
// the critical path.  Flag and copy waits are bounded (2 s) and end the
// kernel with a status code.
//
// Reductions are float-float: a reduce-scatter butterfly inside each warp
// (NV values: each exchange level halves the values a lane keeps), then the
// per-warp partials are summed by NV groups of 16 lanes.
//
// R^-1.  One CTA per column j: column-oriented back substitution
// x_k = t_k / r_kk, t_{<k} -= r_{<k,k} x_k with t = e_j in shared memory,
// the reciprocal pivots precomputed and the next column of R prefetched.
#include "rnla_internal.h"
#include "rnla_ff.cuh"
#include "rnla_async.cuh"

namespace rnla {
namespace qrff {

constexpr int T = 512;
constexpr int W = T / 32;
constexpr int KB = 2;
constexpr int MAX_OWNB = 4;

struct Args {
    double* X;              // m x nc, column-major, ld
    int64_t m, n, nc, ld;
    int64_t ldv;            // m rounded up to even: leading dimension of VF
    float2* VF;             // ldv x n reflectors (column t: rows t+1..m-1)
    float2* TF;             // per reflector block: 4 x 4 T (column-major) then 4 tau
    unsigned int* flags;    // one per reflector block
    unsigned int* status;
};

__device__ __forceinline__ void fail_status(unsigned int* status) {
    atomicCAS(status, 0u, (unsigned int)KSTATUS_BARRIER_TIMEOUT);
}

// Block-wide float-float sums of NV unnormalised accumulators (h, l); the
// normalised totals land in tot[0..NV).  red: W * NV float2 of scratch.
template <int NV>
__device__ __forceinline__ void block_sums(float (&h)[NV], float (&l)[NV], float2* red, float2* tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int off = 16;
#pragma unroll
    for (int half = NV / 2; half >= 1; half /= 2) {
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int k = 0; k < half; ++k) {
            const float sh = up ? h[k] : h[k + half], sl = up ? l[k] : l[k + half];
            float kh = up ? h[k + half] : h[k], kl = up ? l[k + half] : l[k];
            const float rh = __shfl_xor_sync(0xffffffffu, sh, off);
            const float rl = __shfl_xor_sync(0xffffffffu, sl, off);
            ff_acc(kh, kl, rh, rl);
            h[k] = kh;
            l[k] = kl;
        }
        off >>= 1;
    }
    float vh = h[0], vl = l[0];
    for (; off >= 1; off >>= 1) {
        const float rh = __shfl_xor_sync(0xffffffffu, vh, off);
        const float rl = __shfl_xor_sync(0xffffffffu, vl, off);
        ff_acc(vh, vl, rh, rl);
    }
    constexpr int SH = (NV == 1) ? 5 : (NV == 2) ? 4 : (NV == 4) ? 3 : (NV == 8) ? 2 : (NV == 16) ? 1 : 0;
    if ((lane & ((1 << SH) - 1)) == 0) red[warp * NV + (lane >> SH)] = make_float2(vh, vl);
    __syncthreads();
    // NV groups of 16 lanes: group v sums the W = 16 warp partials of value v
    // (whole warps take part; lanes past NV * 16 carry zeros)
    constexpr int PART = (NV * 16 + 31) & ~31;
    if ((int)threadIdx.x < PART) {
        const int v = threadIdx.x >> 4, w = threadIdx.x & 15;
        float sh = 0.f, sl = 0.f;
        if (v < NV) { sh = red[w * NV + v].x; sl = red[w * NV + v].y; }
#pragma unroll
        for (int o = 8; o >= 1; o >>= 1) {
            const float rh = __shfl_xor_sync(0xffffffffu, sh, o);
            const float rl = __shfl_xor_sync(0xffffffffu, sl, o);
            ff_acc(sh, sl, rh, rl);
        }
        if (w == 0 && v < NV) tot[v] = ff_norm(sh, sl);
    }
    __syncthreads();
}

// v_r[i] of a reflector stored in a column with its head at row t: 0 above
// t, 1 at t, the stored value below.
__device__ __forceinline__ float2 vval(const float2* col, int64_t i, int64_t t) {
    return (i > t) ? col[i] : make_float2(i == t ? 1.f : 0.f, 0.f);
}

// Applies Q_b^T = I - V T^T V^T of reflector block b (V: the KB columns at
// vb with stride vs, heads at rows b*KB + r; Tm: 4 x 4 column-major) to the
// KB columns at c (stride m).  nr = reflectors in the block.  Both row
// loops run on packed pairs: W = V^T C pairs reflectors (r, r+1), the
// update pairs columns (q, q+1).
__device__ void apply_block(const float2* vb, int64_t vs, const float2* Tm, int64_t b, int nr, float2* c,
                            int64_t m, float2* red, float2* tot, float2* wsm) {
    const int64_t t0 = b * KB;
    f32x2 ah[KB][KB / 2], al[KB][KB / 2];     // [column q][reflector pair]
#pragma unroll
    for (int q = 0; q < KB; ++q)
#pragma unroll
        for (int k = 0; k < KB / 2; ++k) { ah[q][k] = 0ull; al[q][k] = 0ull; }
    for (int64_t i = t0 + threadIdx.x; i < m; i += T) {
        float2 v[KB];
#pragma unroll
        for (int r = 0; r < KB; ++r) v[r] = (r < nr) ? vval(vb + (size_t)r * vs, i, t0 + r) : make_float2(0.f, 0.f);
        f32x2 vh[KB / 2], vl[KB / 2];
#pragma unroll
        for (int k = 0; k < KB / 2; ++k) {
            vh[k] = pk2(v[2 * k].x, v[2 * k + 1].x);
            vl[k] = pk2(v[2 * k].y, v[2 * k + 1].y);
        }
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            const float2 x = c[(size_t)q * m + i];
            const f32x2 xh = pk2(x.x, x.x), nxh = pk2(-x.x, -x.x), xl = pk2(x.y, x.y);
#pragma unroll
            for (int k = 0; k < KB / 2; ++k) ff2_madd(vh[k], vl[k], xh, nxh, xl, ah[q][k], al[q][k]);
        }
    }
    float h[KB * KB], l[KB * KB];        // [column q][reflector r]
#pragma unroll
    for (int q = 0; q < KB; ++q)
#pragma unroll
        for (int k = 0; k < KB / 2; ++k) {
            const float2 H = upk2(ah[q][k]), L = upk2(al[q][k]);
            h[q * KB + 2 * k] = H.x;
            l[q * KB + 2 * k] = L.x;
            h[q * KB + 2 * k + 1] = H.y;
            l[q * KB + 2 * k + 1] = L.y;
        }
    block_sums<KB * KB>(h, l, red, tot);
    // w'[q][s] = sum_r T[r][s] w[q][r]  (T^T w), one thread per (q, s)
    if ((int)threadIdx.x < KB * KB) {
        const int q = threadIdx.x / KB, s = threadIdx.x % KB;
        float2 acc = make_float2(0.f, 0.f);
        for (int r = 0; r <= s; ++r) acc = ff_add(acc, ff_mul(Tm[r + s * KB], tot[q * KB + r]));
        wsm[q * KB + s] = acc;
    }
    __syncthreads();
    // c_q -= sum_r v_r w'[q][r]: packed over column pairs (q, q+1)
    f32x2 bh[KB / 2][KB], nbh[KB / 2][KB], bl[KB / 2][KB];
#pragma unroll
    for (int k = 0; k < KB / 2; ++k)
#pragma unroll
        for (int r = 0; r < KB; ++r) {
            const float2 w0 = wsm[(2 * k) * KB + r], w1 = wsm[(2 * k + 1) * KB + r];
            bh[k][r] = pk2(-w0.x, -w1.x);
            nbh[k][r] = pk2(w0.x, w1.x);
            bl[k][r] = pk2(-w0.y, -w1.y);
        }
    for (int64_t i = t0 + threadIdx.x; i < m; i += T) {
        f32x2 vh[KB], vl[KB];
#pragma unroll
        for (int r = 0; r < KB; ++r) {
            const float2 v = (r < nr) ? vval(vb + (size_t)r * vs, i, t0 + r) : make_float2(0.f, 0.f);
            vh[r] = pk2(v.x, v.x);
            vl[r] = pk2(v.y, v.y);
        }
#pragma unroll
        for (int k = 0; k < KB / 2; ++k) {
            const float2 x0 = c[(size_t)(2 * k) * m + i], x1 = c[(size_t)(2 * k + 1) * m + i];
            f32x2 xh = pk2(x0.x, x1.x), xl = pk2(x0.y, x1.y);   // unnormalised accumulator
#pragma unroll
            for (int r = 0; r < KB; ++r) ff2_madd(vh[r], vl[r], bh[k][r], nbh[k][r], bl[k][r], xh, xl);
            const float2 H = upk2(xh), L = upk2(xl);
            c[(size_t)(2 * k) * m + i] = ff_norm(H.x, L.x);
            c[(size_t)(2 * k + 1) * m + i] = ff_norm(H.y, L.y);
        }
    }
    __syncthreads();
}

// Factors the block b held at c (KB columns, stride m; columns >= nc are
// absent), writing each reflector to global memory as soon as it is formed;
// then forms T and publishes T, tau and the flag.  One block reduction per
// column t = b*KB + r gathers, over rows i > t, ||c_r||^2 and
// S_q = sum c_q[i] c_r[i] for every other column q of the block: for q < r
// (c_q holds v_q there) they give the Gram entries g_qr = v_q^T v_r that T
// needs, g_qr = v_q[t] + scale * S_q; for q > r the reflector's dot
// v_r^T c_q = c_q[t] + scale * S_q, so H_t is applied to the later columns
// in the same row sweep that scales and publishes v_r.
__device__ void factor_block(const Args& a, float2* c, int64_t b, float2* red, float2* tot, float2* tsm) {
    const int64_t m = a.m, n = a.n, nc = a.nc;
    const int64_t t0 = b * KB;
    const int nr = (int)min((int64_t)KB, n - t0);
    const int ncol = (int)min((int64_t)KB, nc - t0);
    float2* taus = tsm + KB * KB;
    float2 g[KB][KB];                      // g[q][r], q < r (all threads hold the same values)
#pragma unroll
    for (int q = 0; q < KB; ++q)
#pragma unroll
        for (int r = 0; r < KB; ++r) g[q][r] = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < KB; ++r) {
        if (r >= nr) break;
        const int64_t t = t0 + r;
        float2* col = c + (size_t)r * m;
        // slot 0: ||c_r[t+1:]||^2; slot 1 + q: sum_{i>t} c_q[i] c_r[i] (q != r, q < ncol)
        constexpr int NV = 8;
        float h[NV], l[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) { h[k] = 0.f; l[k] = 0.f; }
        for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) {
            const float2 x = col[i];
            ff_madd(x.x, x.y, x.x, x.y, h[0], l[0]);
#pragma unroll
            for (int q = 0; q < KB; ++q)
                if (q != r && q < ncol) {
                    const float2 y = c[(size_t)q * m + i];
                    ff_madd(y.x, y.y, x.x, x.y, h[1 + q], l[1 + q]);
                }
        }
        block_sums<NV>(h, l, red, tot);
        const float2 xn2 = tot[0];
        const float2 alpha = col[t];
        float2 tau = make_float2(0.f, 0.f), beta = alpha, scale = make_float2(0.f, 0.f);
        if (xn2.x != 0.f) {
            const float2 nrm = ff_sqrt(ff_add(ff_mul(alpha, alpha), xn2));
            beta = (alpha.x >= 0.f) ? ff_neg(nrm) : nrm;
            scale = ff_div(make_float2(1.f, 0.f), ff_add(alpha, ff_neg(beta)));
            tau = ff_div(ff_add(beta, ff_neg(alpha)), beta);
        }
        // g[q][r] (q < r) and the update coefficients f_q = -tau v_r^T c_q (q > r)
        float2 f[KB];
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            f[q] = make_float2(0.f, 0.f);
            if (q < r) g[q][r] = ff_add(c[(size_t)q * m + t], ff_mul(scale, tot[1 + q]));
            if (q > r && q < ncol && tau.x != 0.f)
                f[q] = ff_neg(ff_mul(tau, ff_add(c[(size_t)q * m + t], ff_mul(scale, tot[1 + q]))));
        }
        // one row sweep: scale v_r, publish it, apply H_t to the later columns
        const bool scl = xn2.x != 0.f;
        for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) {
            const float2 v = scl ? ff_mul(col[i], scale) : col[i];
            col[i] = v;
            a.VF[i + t * a.ldv] = v;
#pragma unroll
            for (int q = 0; q < KB; ++q)
                if (q > r && q < ncol) {
                    const float2 x = c[(size_t)q * m + i];
                    float xh = x.x, xl = x.y;
                    ff_madd(f[q].x, f[q].y, v.x, v.y, xh, xl);
                    c[(size_t)q * m + i] = ff_norm(xh, xl);
                }
        }
        // row t after every thread has read it (the next column reads rows > t)
        __syncthreads();
        if (threadIdx.x == 0) {
            col[t] = beta;
            taus[r] = tau;
#pragma unroll
            for (int q = 0; q < KB; ++q)
                if (q > r && q < ncol) c[(size_t)q * m + t] = ff_add(c[(size_t)q * m + t], f[q]);
        }
    }
    // T (dlarft, forward, columnwise): T[s][s] = tau_s,
    // T[0:s, s] = -tau_s T[0:s, 0:s] (g[0:s][s]); unrolled, in registers.
    if (threadIdx.x == 0) {
        float2 Tm[KB][KB];
#pragma unroll
        for (int r = 0; r < KB; ++r)
#pragma unroll
            for (int s2 = 0; s2 < KB; ++s2) Tm[r][s2] = make_float2(0.f, 0.f);
#pragma unroll
        for (int s2 = 0; s2 < KB; ++s2) {
            if (s2 < nr) {
                const float2 ts = taus[s2];
                Tm[s2][s2] = ts;
#pragma unroll
                for (int r = 0; r < KB; ++r)
                    if (r < s2) {
                        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                        for (int k = 0; k < KB; ++k)
                            if (k >= r && k < s2) acc = ff_add(acc, ff_mul(Tm[r][k], g[k][s2]));
                        Tm[r][s2] = ff_neg(ff_mul(ts, acc));
                    }
            }
        }
#pragma unroll
        for (int r = 0; r < KB; ++r)
#pragma unroll
            for (int s2 = 0; s2 < KB; ++s2) {
                tsm[r + s2 * KB] = Tm[r][s2];
                a.TF[b * (KB * KB + KB) + r + s2 * KB] = Tm[r][s2];
            }
#pragma unroll
        for (int r = 0; r < KB; ++r) a.TF[b * (KB * KB + KB) + KB * KB + r] = taus[r];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicExch(&a.flags[b], 1u);
    }
}

template <int OWNB>
__global__ void __launch_bounds__(T, 1) qr_ff_kernel(Args a) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ float2 red[W * 16];
    __shared__ float2 tot[16];
    __shared__ float2 wsm[KB * KB];
    __shared__ __align__(16) float2 tsm[KB * KB + KB];      // own T and taus while factoring
    __shared__ __align__(16) float2 tin[KB * KB + KB];      // received T and taus
    __shared__ __align__(8) uint64_t vbar;
    __shared__ int ok_s;
    const int64_t m = a.m, n = a.n, nc = a.nc, G = gridDim.x;
    float2* cols = sm;                                  // OWNB * KB columns of m
    float2* vb = sm + (size_t)OWNB * KB * m;            // received reflector block, KB x ldv
    const int64_t nblk = (nc + KB - 1) / KB, nref = (n + KB - 1) / KB;
    int64_t blk[OWNB];
    int64_t last = -1;
#pragma unroll
    for (int q = 0; q < OWNB; ++q) {
        blk[q] = (int64_t)blockIdx.x + q * G;
        if (blk[q] < nblk) last = blk[q];
    }
#pragma unroll
    for (int q = 0; q < OWNB; ++q)
        for (int r = 0; r < KB; ++r) {
            const int64_t j = blk[q] * KB + r;
            if (blk[q] < nblk)
                for (int64_t i = threadIdx.x; i < m; i += T)
                    cols[(size_t)(q * KB + r) * m + i] = (j < nc) ? ff_split(a.X[i + j * a.ld]) : make_float2(0.f, 0.f);
        }
    if (threadIdx.x == 0) {
        mbar_init(&vbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    volatile int quiet = 0;
    if (blk[0] == 0 && nref > 0) factor_block(a, cols, 0, red, tot, tsm);
    for (int64_t rb = 0; rb < nref && rb < last; ++rb) {
        const int nr = (int)min((int64_t)KB, n - rb * KB);
        // flag, then one bulk copy per reflector column (rows from the block head) and T
        if (threadIdx.x == 0) {
            ok_s = 1;
            const volatile unsigned int* vf = a.flags + rb;
            if (*vf == 0u) {
                const unsigned long long t0 = globaltimer_ns();
                unsigned int spins = 0;
                while (*vf == 0u) {
                    if (*((volatile unsigned int*)a.status) != 0u) { ok_s = 0; break; }
                    if ((++spins & 255u) == 0u && globaltimer_ns() - t0 > MBAR_WAIT_NS) {
                        fail_status(a.status);
                        ok_s = 0;
                        break;
                    }
                }
            }
            __threadfence();
            if (ok_s) {
                const int64_t r0 = (rb * KB) & ~1LL;                 // even row: 16-byte aligned
                const uint32_t bytes = (uint32_t)((a.ldv - r0) * sizeof(float2));
                mbar_expect_tx(&vbar, (uint32_t)nr * bytes + (uint32_t)sizeof(tin));
                for (int r = 0; r < nr; ++r)
                    bulk_g2s(vb + (size_t)r * a.ldv + r0, a.VF + (rb * KB + r) * a.ldv + r0, bytes, &vbar);
                bulk_g2s(tin, a.TF + rb * (KB * KB + KB), (uint32_t)sizeof(tin), &vbar);
                if (!mbar_wait(&vbar, (uint32_t)(rb & 1), &quiet)) {
                    fail_status(a.status);
                    ok_s = 0;
                }
            }
        }
        __syncthreads();
        if (!ok_s) return;
        int la = -1;
#pragma unroll
        for (int q = 0; q < OWNB; ++q)
            if (blk[q] == rb + 1) la = q;
        if (la >= 0) {
            apply_block(vb, a.ldv, tin, rb, nr, cols + (size_t)la * KB * m, m, red, tot, wsm);
            if (rb + 1 < nref) factor_block(a, cols + (size_t)la * KB * m, rb + 1, red, tot, tsm);
        }
#pragma unroll
        for (int q = 0; q < OWNB; ++q)
            if (q != la && blk[q] > rb && blk[q] < nblk)
                apply_block(vb, a.ldv, tin, rb, nr, cols + (size_t)q * KB * m, m, red, tot, wsm);
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < OWNB; ++q)
        for (int r = 0; r < KB; ++r) {
            const int64_t j = blk[q] * KB + r;
            if (blk[q] < nblk && j < nc)
                for (int64_t i = threadIdx.x; i < m; i += T)
                    a.X[i + j * a.ld] = ff_to_double(cols[(size_t)(q * KB + r) * m + i]);
        }
}

// ---- R^-1 ----
constexpr int TI = 128;

// RF = split(R) (upper triangle, column-major n x n)
__global__ void rsplit_kernel(const double* __restrict__ R, int64_t n, int64_t ldr, float2* __restrict__ RF) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        RF[idx] = (i <= j) ? ff_split(R[i + j * ldr]) : make_float2(0.f, 0.f);
    }
}

// One CTA per column j of R^-1: x_k = t_k / r_kk, t_{<k} -= r_{<k,k} x_k,
// k = j .. 0, t = e_j in shared memory.  The thread's entries of the next
// two columns of R are loaded ahead, so the L2 latency overlaps the steps.
__global__ void __launch_bounds__(TI) rinv_ff_kernel(const float2* __restrict__ RF, int64_t n,
                                                     double* __restrict__ Ri, int64_t ldi,
                                                     unsigned int* __restrict__ status) {
    extern __shared__ __align__(16) float2 smi[];
    float2* dinv = smi;          // n reciprocal pivots
    float2* t = smi + n;         // n: right-hand side / solution
    const int64_t j = blockIdx.x;
    for (int64_t k = threadIdx.x; k < n; k += TI) {
        const float2 d = RF[k + k * n];
        if (d.x == 0.f) atomicCAS(status, 0u, (unsigned int)KSTATUS_SINGULAR);
        dinv[k] = (d.x == 0.f) ? make_float2(0.f, 0.f) : ff_div(make_float2(1.f, 0.f), d);
        t[k] = make_float2(k == j ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    constexpr int RPT = 8;       // rows per thread: n <= TI * RPT
    float2 r0[RPT], r1[RPT];     // columns k and k - 1 (thread's rows)
#pragma unroll
    for (int s = 0; s < RPT; ++s) {
        const int64_t i = threadIdx.x + (int64_t)s * TI;
        r0[s] = (i < j) ? RF[i + j * n] : make_float2(0.f, 0.f);
        r1[s] = (j > 0 && i < j - 1) ? RF[i + (j - 1) * n] : make_float2(0.f, 0.f);
    }
    for (int64_t k = j; k >= 0; --k) {
        float2 r2[RPT];          // column k - 2
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
            const int64_t i = threadIdx.x + (int64_t)s * TI;
            r2[s] = (k > 1 && i < k - 2) ? RF[i + (k - 2) * n] : make_float2(0.f, 0.f);
        }
        const float2 xk = ff_mul(t[k], dinv[k]);
        __syncthreads();
        if (threadIdx.x == 0) t[k] = xk;
        const float2 nx = ff_neg(xk);
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
            const int64_t i = threadIdx.x + (int64_t)s * TI;
            if (i < k) {
                const float2 ti = t[i];
                float h = ti.x, l = ti.y;
                ff_madd(r0[s].x, r0[s].y, nx.x, nx.y, h, l);
                t[i] = ff_norm(h, l);
            }
        }
        __syncthreads();
#pragma unroll
        for (int s = 0; s < RPT; ++s) { r0[s] = r1[s]; r1[s] = r2[s]; }
    }
    for (int64_t i = threadIdx.x; i < n; i += TI)
        Ri[i + j * ldi] = (i <= j) ? ff_to_double(t[i]) : 0.0;
}

template <int OWNB>
static const void* qr_kernel() { return (const void*)qr_ff_kernel<OWNB>; }

}  // namespace qrff

// Dynamic shared memory of the QR kernel: the owned blocks (stride m) and
// one received reflector block (stride m rounded up to even).
static size_t qr_ff_smem(int64_t ownb, int64_t m) {
    return ((size_t)ownb * qrff::KB * m + (size_t)qrff::KB * ((m + 1) & ~1LL)) * sizeof(float2);
}

// Owned column blocks per CTA for the float-float QR (0: does not fit): the
// owned blocks and one received reflector block in shared memory, one CTA
// per SM.
static int qr_ff_ownb(const Ctx& ctx, int64_t m, int64_t nc) {
    const int64_t nblk = (nc + qrff::KB - 1) / qrff::KB;
    const int64_t G = nblk < ctx.sm_count ? nblk : ctx.sm_count;
    const int64_t ownb = (nblk + G - 1) / G;
    if (ownb > qrff::MAX_OWNB) return 0;
    const size_t smem = qr_ff_smem(ownb, m);
    if (smem > 200 * 1024) return 0;
    return (int)ownb;
}

bool qr_ff_supported(const Ctx& ctx, int64_t m, int64_t n, int64_t nc) {
    return m >= n && n >= 1 && nc >= n && n <= qrff::TI * 8 && qr_ff_ownb(ctx, m, nc) > 0;
}

void householder_qr_ff(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld) {
    using namespace qrff;
    const int ownb = qr_ff_ownb(ctx, m, nc);
    if (ownb == 0 || m < n) fail(RNLA_ERR_UNSUPPORTED, "float-float QR: the sketch does not fit in shared memory");
    const int64_t nblk = (nc + KB - 1) / KB;
    const int64_t G = nblk < ctx.sm_count ? nblk : ctx.sm_count;
    const size_t smem = qr_ff_smem(ownb, m);
    const void* k = ownb == 1 ? qr_kernel<1>() : ownb == 2 ? qr_kernel<2>() : ownb == 3 ? qr_kernel<3>() : qr_kernel<4>();
    RNLA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, T, smem));
    if ((int64_t)nb * ctx.sm_count < G) fail(RNLA_ERR_UNSUPPORTED, "float-float QR: grid not co-resident");
    cudaStream_t s = ctx.stream;
    const int64_t nref = (n + KB - 1) / KB;
    const int64_t ldv = (m + 1) & ~1LL;
    DevBuf<float2> VF((size_t)ldv * n, s), TF((size_t)nref * (KB * KB + KB), s);
    DevBuf<unsigned int> flags(nref, s);
    RNLA_CUDA(cudaMemsetAsync(flags.get(), 0, nref * sizeof(unsigned int), s));
    ctx.clear_status();
    Args a{X, m, n, nc, ld, ldv, VF.get(), TF.get(), flags.get(), ctx.status};
    void* args[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3((unsigned)G), dim3(T), args, smem, s));
    count_launch();
    ctx.check_status("householder_qr (float-float)");
}

bool upper_inverse_ff(Ctx& ctx, const double* R, int64_t n, int64_t ldr, double* Rinv, int64_t ldi) {
    using namespace qrff;
    if (n <= 0) return true;
    if (n > TI * 8) fail(RNLA_ERR_UNSUPPORTED, "float-float R^-1: n > 1024");
    const size_t smem = (size_t)2 * n * sizeof(float2);
    if (smem > 48 * 1024)
        RNLA_CUDA(cudaFuncSetAttribute(rinv_ff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // a zero pivot is reported through the status word (KSTATUS_SINGULAR):
    // at once, or at the pending check in deferred mode
    ctx.clear_status();
    DevBuf<float2> RF((size_t)n * n, ctx.stream);
    {
        int g = (int)div_up(n * n, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        rsplit_kernel<<<g, 256, 0, ctx.stream>>>(R, n, ldr, RF);
        RNLA_LAUNCH_CHECK();
    }
    rinv_ff_kernel<<<(unsigned)n, TI, smem, ctx.stream>>>(RF, n, Rinv, ldi, ctx.status);
    RNLA_LAUNCH_CHECK();
    if (ctx.deferred) {
        ctx.check_status("R^-1 of the sketch (float-float)");
        return true;
    }
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, ctx.status, sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    return h == 0;
}

}  // namespace rnla
