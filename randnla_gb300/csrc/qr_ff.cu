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
// exactly zero) and writes each reflector v_t and tau_t to global memory as
// soon as it is formed.  Every CTA applies every reflector to the blocks it
// still holds, in order, as the reflector lands: there is no flag -- the
// reflector buffers start filled with a value no arithmetic produces, and a
// reader re-loads an entry until it has been written.  A block's owner
// factors it once all earlier reflectors are applied, so the critical path
// per block is its KB column steps plus one cross-SM hand-off (the last
// reflector of the previous block reaching the next owner), and every other
// CTA's updates overlap it.  All waits are bounded (2 s) and end the kernel
// with a status code.
//
// A column step is one block reduction (the column's norm below the
// diagonal and its dots with the block's later columns, all accumulated
// during the previous step's row sweep) and one row sweep (scale v, publish
// it, apply H_t to the later columns of the block, accumulate the next
// step's reduction).
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
constexpr int KB = 4;
constexpr int MAX_OWNB = 4;

struct Args {
    double* X;              // m x nc, column-major, ld
    int64_t m, n, nc, ld;
    int64_t ldv;            // m rounded up to even: leading dimension of VF
    float2* VF;             // ldv x n reflectors (column t: rows t+1..m-1)
    float2* taug;           // tau_t
    unsigned int* status;
};

// VF and taug start filled with this signalling NaN (as the high word of
// each pair): no arithmetic produces it (results are quiet NaNs), so an
// entry that differs from it has been written.
constexpr uint32_t UNSET = 0x7FBADBADu;

__device__ __forceinline__ float2 ld_relaxed_f2(const float2* p) {
    float2 v;
    asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p) : "memory");
    return v;
}

// Bounded spin until *p has been written; false (status set) on timeout or
// when another CTA has failed.
__device__ __forceinline__ bool ld_written(const Args& a, const float2* p, float2& v) {
    v = ld_relaxed_f2(p);
    if (__float_as_uint(v.x) != UNSET) return true;
    const unsigned long long t0 = globaltimer_ns();
    unsigned int spins = 0;
    while (true) {
        v = ld_relaxed_f2(p);
        if (__float_as_uint(v.x) != UNSET) return true;
        if ((++spins & 31u) == 0u) {
            if (*((volatile unsigned int*)a.status) != 0u) return false;
            if (globaltimer_ns() - t0 > MBAR_WAIT_NS) {
                atomicCAS(a.status, 0u, (unsigned int)KSTATUS_BARRIER_TIMEOUT);
                return false;
            }
        }
    }
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

// Factors the block b held at c (KB columns, stride m; columns >= nc are
// absent), writing each reflector and its tau to global memory as soon as
// it is formed.  Column step r (t = b*KB + r): the block reduction of
// ||c_r[t+1:]||^2 and S_q = sum_{i>t} c_q[i] c_r[i] (q > r), the reflector
// scalars, then one row sweep that scales v_r, publishes it, applies H_t to
// the later columns (v_r^T c_q = c_q[t] + scale S_q) and accumulates the
// next step's reduction on the updated rows.
__device__ void factor_block(const Args& a, float2* c, int64_t b, float2* red, float2* tot) {
    const int64_t m = a.m, n = a.n, nc = a.nc;
    const int64_t t0 = b * KB;
    const int nr = (int)min((int64_t)KB, n - t0);
    const int ncol = (int)min((int64_t)KB, nc - t0);
    // slot 0: ||c_r[t+1:]||^2; slot q (q > r): sum_{i>t} c_q[i] c_r[i]
    float h[KB], l[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) { h[k] = 0.f; l[k] = 0.f; }
    for (int64_t i = t0 + 1 + threadIdx.x; i < m; i += T) {
        const float2 x = c[i];
        ff_madd(x.x, x.y, x.x, x.y, h[0], l[0]);
#pragma unroll
        for (int q = 1; q < KB; ++q)
            if (q < ncol) {
                const float2 y = c[(size_t)q * m + i];
                ff_madd(y.x, y.y, x.x, x.y, h[q], l[q]);
            }
    }
#pragma unroll
    for (int r = 0; r < KB; ++r) {
        if (r >= nr) break;
        const int64_t t = t0 + r;
        float2* col = c + (size_t)r * m;
        block_sums<KB>(h, l, red, tot);
        const float2 xn2 = tot[0];
        const float2 alpha = col[t];
        float2 tau = make_float2(0.f, 0.f), beta = alpha, scale = make_float2(0.f, 0.f);
        if (xn2.x != 0.f) {
            const float2 nrm = ff_sqrt(ff_add(ff_mul(alpha, alpha), xn2));
            beta = (alpha.x >= 0.f) ? ff_neg(nrm) : nrm;
            scale = ff_div(make_float2(1.f, 0.f), ff_add(alpha, ff_neg(beta)));
            tau = ff_div(ff_add(beta, ff_neg(alpha)), beta);
        }
        // update coefficients f_q = -tau v_r^T c_q (q > r)
        float2 f[KB];
#pragma unroll
        for (int q = 0; q < KB; ++q) {
            f[q] = make_float2(0.f, 0.f);
            if (q > r && q < ncol && tau.x != 0.f)
                f[q] = ff_neg(ff_mul(tau, ff_add(c[(size_t)q * m + t], ff_mul(scale, tot[q]))));
        }
        // one row sweep: scale v_r, publish it, apply H_t to the later
        // columns, accumulate the next step's reduction (rows > t + 1)
        const bool scl = xn2.x != 0.f;
        const int rn = r + 1;                    // next column
        const bool nxt = rn < nr;
#pragma unroll
        for (int k = 0; k < KB; ++k) { h[k] = 0.f; l[k] = 0.f; }
        for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) {
            const float2 v = scl ? ff_mul(col[i], scale) : col[i];
            col[i] = v;
            a.VF[i + t * a.ldv] = v;
            float2 y[KB];
#pragma unroll
            for (int q = 0; q < KB; ++q) {
                y[q] = make_float2(0.f, 0.f);
                if (q > r && q < ncol) {
                    const float2 x = c[(size_t)q * m + i];
                    float xh = x.x, xl = x.y;
                    ff_madd(f[q].x, f[q].y, v.x, v.y, xh, xl);
                    y[q] = ff_norm(xh, xl);
                    c[(size_t)q * m + i] = y[q];
                }
            }
            if (nxt && i > t + 1) {
                const float2 x = y[rn < KB ? rn : 0];
                ff_madd(x.x, x.y, x.x, x.y, h[0], l[0]);
#pragma unroll
                for (int q = 0; q < KB; ++q)
                    if (q > rn && q < ncol) ff_madd(y[q].x, y[q].y, x.x, x.y, h[q], l[q]);
            }
        }
        // row t after every thread has read it (the next step reads rows > t)
        __syncthreads();
        if (threadIdx.x == 0) {
            col[t] = beta;
#pragma unroll
            for (int q = 0; q < KB; ++q)
                if (q > r && q < ncol) c[(size_t)q * m + t] = ff_add(c[(size_t)q * m + t], f[q]);
            a.taug[t] = tau;
        }
    }
    __syncthreads();
}

// H_t = I - tau_t v_t v_t^T on the ncol columns at c (stride m), v_t read
// from VF through L2 as it is written (each thread waits for its own
// entries) into vtmp (shared, m entries).  One block reduction of the ncol
// dots v_t^T c_q, one update sweep.  False if a wait failed (all threads
// agree through ok[0..1], shared).
// eager: this CTA owns the block right after the reflector's (critical
// path): every thread loads as soon as it can.  Otherwise thread 0 first
// waits, with back-off, for tau_t, so the CTAs with slack do not crowd the
// L2 lines the critical CTA is reading.
template <int NC>
__device__ bool apply_reflector(const Args& a, int64_t t, float2* c, int64_t m, int ncol, float2* red,
                                float2* tot, float2* vtmp, int* ok, bool eager) {
    constexpr int NP = NC / 2;               // column pairs (packed f32x2 arithmetic)
    float2 ct[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q)
        ct[q] = (q < ncol) ? c[(size_t)q * m + t] : make_float2(0.f, 0.f);   // read before the reduction's barrier
    if (threadIdx.x == 0) {
        int okv = 1;
        if (!eager) {
            float2 tv = ld_relaxed_f2(a.taug + t);
            const unsigned long long t0 = globaltimer_ns();
            while (__float_as_uint(tv.x) == UNSET) {
                __nanosleep(256);
                if (*((volatile unsigned int*)a.status) != 0u) { okv = 0; break; }
                if (globaltimer_ns() - t0 > MBAR_WAIT_NS) {
                    atomicCAS(a.status, 0u, (unsigned int)KSTATUS_BARRIER_TIMEOUT);
                    okv = 0;
                    break;
                }
                tv = ld_relaxed_f2(a.taug + t);
            }
        }
        ok[0] = okv;       // the wait above; read after the barrier below
        ok[1] = 1;         // the loads below; cleared by any thread whose wait fails
    }
    __syncthreads();
    if (!ok[0]) return false;
    bool good = true;
    const int np = (ncol + 1) >> 1;
    f32x2 ah[NP], al[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) { ah[k] = 0ull; al[k] = 0ull; }
    const float2* vg = a.VF + t * a.ldv;
    // tau_t is loaded with the first round of rows (it is written right after
    // them), so it costs no separate L2 round trip
    float2 tau = ld_relaxed_f2(a.taug + t);
    // RB rows per thread per round: their L2 loads are all in flight before
    // any is checked, so a round costs one L2 round trip
    constexpr int RB = (NC <= 8) ? 4 : 2;
    for (int64_t i0 = t + 1 + threadIdx.x; i0 < m; i0 += (int64_t)RB * T) {
        float2 vr[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int64_t i = i0 + (int64_t)u * T;
            vr[u] = (i < m) ? ld_relaxed_f2(vg + i) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int64_t i = i0 + (int64_t)u * T;
            if (i >= m) break;
            float2 v = vr[u];
            if (__float_as_uint(v.x) == UNSET && !ld_written(a, vg + i, v)) { good = false; v = make_float2(0.f, 0.f); }
            vtmp[i] = v;
            const f32x2 vh = pk2(v.x, v.x), nvh = pk2(-v.x, -v.x), vl = pk2(v.y, v.y);
#pragma unroll
            for (int k = 0; k < NP; ++k)
                if (k < np) {
                    const float2 x0 = c[(size_t)(2 * k) * m + i], x1 = c[(size_t)(2 * k + 1) * m + i];
                    ff2_madd(pk2(x0.x, x1.x), pk2(x0.y, x1.y), vh, nvh, vl, ah[k], al[k]);
                }
        }
    }
    if (__float_as_uint(tau.x) == UNSET && !ld_written(a, a.taug + t, tau)) good = false;
    if (!good) ok[1] = 0;
    float h[NC], l[NC];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        const float2 H = upk2(ah[k]), L = upk2(al[k]);
        h[2 * k] = H.x; l[2 * k] = L.x;
        h[2 * k + 1] = H.y; l[2 * k + 1] = L.y;
    }
    block_sums<NC>(h, l, red, tot);
    if (!ok[1]) return false;
    // c_q += f_q v over column pairs: b = (f_q, f_q+1)
    f32x2 bh[NP], nbh[NP], bl[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
        float2 f0 = make_float2(0.f, 0.f), f1 = make_float2(0.f, 0.f);
        if (tau.x != 0.f) {
            if (2 * k < ncol) f0 = ff_neg(ff_mul(tau, ff_add(ct[2 * k], tot[2 * k])));
            if (2 * k + 1 < ncol) f1 = ff_neg(ff_mul(tau, ff_add(ct[2 * k + 1], tot[2 * k + 1])));
        }
        bh[k] = pk2(f0.x, f1.x);
        nbh[k] = pk2(-f0.x, -f1.x);
        bl[k] = pk2(f0.y, f1.y);
    }
    for (int64_t i = t + threadIdx.x; i < m; i += T) {
        const float2 v = (i == t) ? make_float2(1.f, 0.f) : vtmp[i];
        const f32x2 vh = pk2(v.x, v.x), vl = pk2(v.y, v.y);
#pragma unroll
        for (int k = 0; k < NP; ++k)
            if (k < np) {
                float2* p0 = c + (size_t)(2 * k) * m + i;
                float2* p1 = c + (size_t)(2 * k + 1) * m + i;
                const float2 x0 = *p0, x1 = *p1;
                f32x2 xh = pk2(x0.x, x1.x), xl = pk2(x0.y, x1.y);
                ff2_madd(vh, vl, bh[k], nbh[k], bl[k], xh, xl);
                const float2 H = upk2(xh), L = upk2(xl);
                *p0 = ff_norm(H.x, L.x);
                if (2 * k + 1 < ncol) *p1 = ff_norm(H.y, L.y);
            }
    }
    __syncthreads();
    return true;
}

// VF and taug <- UNSET
__global__ void unset_kernel(float2* __restrict__ p, int64_t count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        reinterpret_cast<uint2*>(p)[i] = make_uint2(UNSET, 0u);
}

template <int OWNB>
__global__ void __launch_bounds__(T, 1) qr_ff_kernel(Args a) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ float2 red[W * 16];
    __shared__ float2 tot[16];
    __shared__ int ok_s[2];
    constexpr int NC = (OWNB * KB <= 4) ? 4 : (OWNB * KB <= 8) ? 8 : 16;   // columns one reflector updates
    const int64_t m = a.m, n = a.n, nc = a.nc, G = gridDim.x;
    float2* cols = sm;                                  // OWNB * KB columns of m
    float2* vtmp = sm + (size_t)OWNB * KB * m;          // one reflector (m)
    const int64_t nblk = (nc + KB - 1) / KB;
    int64_t blk[OWNB];
    int nown = 0;
#pragma unroll
    for (int q = 0; q < OWNB; ++q) {
        blk[q] = (int64_t)blockIdx.x + q * G;
        if (blk[q] < nblk) nown = q + 1;
    }
#pragma unroll
    for (int q = 0; q < OWNB; ++q)
        for (int r = 0; r < KB; ++r) {
            const int64_t j = blk[q] * KB + r;
            for (int64_t i = threadIdx.x; i < m; i += T)
                cols[(size_t)(q * KB + r) * m + i] =
                    (blk[q] < nblk && j < nc) ? ff_split(a.X[i + j * a.ld]) : make_float2(0.f, 0.f);
        }
    __syncthreads();
    // reflectors in order: each one to every block still held, the own
    // block factored as soon as every earlier reflector is applied
    int64_t t = 0;
    for (int q = 0; q < nown; ++q) {
        const int64_t t0 = blk[q] * KB;
        const int64_t tend = min(t0, n);
        float2* c = cols + (size_t)q * KB * m;
        const int ncol = (nown - q) * KB;
        for (; t < tend; ++t)
            if (!apply_reflector<NC>(a, t, c, m, ncol, red, tot, vtmp, ok_s, t >= t0 - KB)) return;
        if (t0 < n) factor_block(a, c, blk[q], red, tot);
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
    return ((size_t)ownb * qrff::KB * m + (size_t)m) * sizeof(float2);
}

// Owned column blocks per CTA for the float-float QR (0: does not fit): the
// owned blocks and one reflector in shared memory, one CTA per SM.
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
    set_smem_limit((const void*)k, smem);
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, T, smem));
    if ((int64_t)nb * ctx.sm_count < G) fail(RNLA_ERR_UNSUPPORTED, "float-float QR: grid not co-resident");
    cudaStream_t s = ctx.stream;
    const int64_t ldv = (m + 1) & ~1LL;
    DevBuf<float2> VF((size_t)ldv * n, s), taug(n, s);
    {
        const int64_t cnt = (int64_t)ldv * n;
        int g = (int)div_up(cnt, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        unset_kernel<<<g, 256, 0, s>>>(VF, cnt);
        RNLA_LAUNCH_CHECK();
        unset_kernel<<<(unsigned)div_up(n, 256), 256, 0, s>>>(taug, n);
        RNLA_LAUNCH_CHECK();
    }
    ctx.clear_status();
    Args a{X, m, n, nc, ld, ldv, VF.get(), taug.get(), ctx.status};
    void* args[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3((unsigned)G), dim3(T), args, smem, s));
    count_launch();
    ctx.check_status("householder_qr (float-float)");
}

// T (2n x nc) = the first n rows of the two factored halves of X stacked
// (rows [0, n) of the top half, then of the bottom half starting at row h),
// with the strictly lower parts of their first n columns (the reflector
// storage) zeroed: T = [R_top c_top; R_bot c_bot].
__global__ void tsqr_stack_kernel(const double* __restrict__ X, int64_t ld, int64_t h, int64_t n, int64_t nc,
                                  double* __restrict__ Tm) {
    const int64_t rows = 2 * n;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < rows * nc;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % rows, j = idx / rows;
        const int64_t li = i < n ? i : i - n;
        const int64_t src = (i < n ? i : h + li) + j * ld;
        Tm[i + j * rows] = (j < n && li > j) ? 0.0 : X[src];
    }
}

bool qr_ff_tsqr_supported(const Ctx& ctx, int64_t m, int64_t n, int64_t nc) {
    const int64_t h = (m + 1) / 2;
    return n >= 1 && m - h >= n && qr_ff_supported(ctx, h, n, nc) && qr_ff_supported(ctx, 2 * n, n, nc);
}

// Two-level TSQR in float-float for sketches whose rows do not fit the
// shared memory of one factorization: QR of each row half, then QR of their
// stacked R blocks (with the carried columns n..nc-1).  The first n rows of X
// receive R and (Q^T X)[:n, n:nc], the same contract as householder_qr_ff;
// the rows below n are not meaningful afterwards.
void householder_qr_ff_tsqr(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld) {
    if (!qr_ff_tsqr_supported(ctx, m, n, nc)) fail(RNLA_ERR_UNSUPPORTED, "float-float TSQR: shape not supported");
    const int64_t h = (m + 1) / 2;
    householder_qr_ff(ctx, X, h, n, nc, ld);
    householder_qr_ff(ctx, X + h, m - h, n, nc, ld);
    DevBuf<double> Tm((size_t)2 * n * nc, ctx.stream);
    {
        int g = (int)div_up(2 * n * nc, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        tsqr_stack_kernel<<<g, 256, 0, ctx.stream>>>(X, ld, h, n, nc, Tm);
        RNLA_LAUNCH_CHECK();
    }
    householder_qr_ff(ctx, Tm, 2 * n, n, nc, 2 * n);
    copy_matrix(ctx, n, nc, Tm, 2 * n, X, ld);
}

bool upper_inverse_ff(Ctx& ctx, const double* R, int64_t n, int64_t ldr, double* Rinv, int64_t ldi) {
    using namespace qrff;
    if (n <= 0) return true;
    if (n > TI * 8) fail(RNLA_ERR_UNSUPPORTED, "float-float R^-1: n > 1024");
    const size_t smem = (size_t)2 * n * sizeof(float2);
    if (smem > 48 * 1024)
        set_smem_limit((const void*)rinv_ff_kernel, smem);
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
