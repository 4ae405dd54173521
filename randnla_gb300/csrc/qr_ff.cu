// Float-float Householder QR and triangular inverse for the BF16X
// precision's preconditioner (sketch_and_precondition.rs:53-55: QR of the
// sketch S A, R^-1).  Arithmetic is float-float on the FP32 pipe: on GB300 a
// dependent FP64 operation takes ~64 cycles and a divide or square root
// several hundred, and a QR of a d x n sketch is a chain of n dependent
// column steps, so the FP64 chain length sets its time.
//
// QR.  Columns are grouped in blocks of KB = 4; block b is owned by CTA
// b mod G, which keeps its columns in shared memory.  Reflector block rb is
// published to global memory (float-float v, tau) and announced by a flag.
// On seeing flag rb, a CTA loads the block's reflectors into shared memory;
// if it owns block rb + 1 it applies them there first, factors that block
// (look-ahead) and publishes it, then applies them to its other blocks.  One
// cross-CTA hand-off per KB columns sits on the critical path.
// Reflectors follow LAPACK dlarfg: beta = -sign(alpha) ||(alpha, x)||,
// v = x / (alpha - beta), tau = (beta - alpha) / beta, and tau = 0 when x is
// exactly zero.  Flag waits are bounded (2 s) and end the kernel with a
// status code.
//
// R^-1.  One CTA per column j: column-oriented back substitution
// x_k = t_k / r_kk, t_{<k} -= r_{<k,k} x_k with t = e_j in shared memory and
// the reciprocal pivots precomputed.
#include "rnla_internal.h"
#include "rnla_ff.cuh"

namespace rnla {
namespace qrff {

constexpr int T = 256;
constexpr int W = T / 32;
constexpr int KB = 4;
constexpr int MAX_OWNB = 4;
constexpr int MAXC = MAX_OWNB * KB;

struct Args {
    double* X;              // m x nc, column-major, ld
    int64_t m, n, nc, ld;
    float2* VF;             // m x n reflectors (column t: rows t+1..m-1)
    float2* tauF;           // n
    unsigned int* flags;    // one per reflector block
    unsigned int* status;
};

__device__ bool wait_flag(const unsigned int* f, unsigned int* status) {
    __shared__ int ok_s;
    if (threadIdx.x == 0) {
        ok_s = 1;
        const volatile unsigned int* vf = f;
        if (*vf == 0u) {
            const unsigned long long t0 = globaltimer_ns();
            unsigned int spins = 0;
            while (*vf == 0u) {
                if (*((volatile unsigned int*)status) != 0u) { ok_s = 0; break; }
                if ((++spins & 255u) == 0u && globaltimer_ns() - t0 > 2000000000ull) {
                    atomicCAS(status, 0u, (unsigned int)KSTATUS_BARRIER_TIMEOUT);
                    ok_s = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok_s != 0;
}

// Block sums of cnt unnormalised float-float accumulators; every thread
// receives every total (fixed order: warps 0..W-1).
template <int N>
__device__ __forceinline__ void block_sums(float (&h)[N], float (&l)[N], int cnt, float2* red, float2* tot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < N; ++c)
        if (c < cnt) {
            const float2 s = ff_warp_sum(h[c], l[c]);
            if (lane == 0) red[warp * N + c] = s;
        }
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
        float th = 0.f, tl = 0.f;
        for (int w = 0; w < W; ++w) ff_acc(th, tl, red[w * N + threadIdx.x].x, red[w * N + threadIdx.x].y);
        tot[threadIdx.x] = ff_norm(th, tl);
    }
    __syncthreads();
}

// Applies reflector t (v: row t implicit 1, rows > t in v[]) with tau to the
// columns cols + slot[c] * m, c < cnt.
__device__ void apply_reflector(const Args& a, const float2* v, float2 tau, int64_t t, float2* cols,
                                const int* slot, int cnt, float2* red, float2* tot) {
    const int64_t m = a.m;
    float h[MAXC], l[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; ++c) { h[c] = 0.f; l[c] = 0.f; }
    for (int64_t i = t + threadIdx.x; i < m; i += T) {
        const float2 vi = (i == t) ? make_float2(1.f, 0.f) : v[i];
#pragma unroll
        for (int c = 0; c < MAXC; ++c)
            if (c < cnt) {
                const float2 x = cols[(size_t)slot[c] * m + i];
                ff_madd(vi.x, vi.y, x.x, x.y, h[c], l[c]);
            }
    }
    block_sums<MAXC>(h, l, cnt, red, tot);
    for (int64_t i = t + threadIdx.x; i < m; i += T) {
        const float2 vi = (i == t) ? make_float2(1.f, 0.f) : v[i];
        for (int c = 0; c < cnt; ++c) {
            const float2 f = ff_mul(tau, tot[c]);
            float2* x = cols + (size_t)slot[c] * m + i;
            *x = ff_add(*x, ff_neg(ff_mul(f, vi)));
        }
    }
    __syncthreads();
}

// Factors the KB columns in local slots q*KB.. (block b), publishes them.
__device__ void factor_block(const Args& a, float2* cols, int q, int64_t b, float2* red, float2* tot,
                             float2* taus_local) {
    const int64_t m = a.m, n = a.n, nc = a.nc;
    for (int r = 0; r < KB; ++r) {
        const int64_t t = b * KB + r;
        if (t >= n) break;
        float2* col = cols + (size_t)(q * KB + r) * m;
        float h[1] = {0.f}, l[1] = {0.f};
        for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) ff_madd(col[i].x, col[i].y, col[i].x, col[i].y, h[0], l[0]);
        block_sums<1>(h, l, 1, red, tot);
        const float2 xn2 = tot[0];
        const float2 alpha = col[t];
        float2 tau = make_float2(0.f, 0.f), beta = alpha;
        if (xn2.x != 0.f) {
            const float2 nrm = ff_sqrt(ff_add(ff_mul(alpha, alpha), xn2));
            beta = (alpha.x >= 0.f) ? ff_neg(nrm) : nrm;
            const float2 scale = ff_div(make_float2(1.f, 0.f), ff_add(alpha, ff_neg(beta)));
            for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) col[i] = ff_mul(col[i], scale);
            tau = ff_div(ff_add(beta, ff_neg(alpha)), beta);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            col[t] = beta;
            taus_local[r] = tau;
        }
        __syncthreads();
        // apply to the rest of the block (v = (1, col[t+1..]))
        int slot[MAXC];
        int cnt = 0;
        for (int rr = r + 1; rr < KB && cnt < MAXC; ++rr)
            if (b * KB + rr < nc) slot[cnt++] = q * KB + rr;
        if (cnt > 0 && tau.x != 0.f) {
            // the reflector's v: row t implicit 1 (col[t] now holds beta)
            float hh[MAXC], ll[MAXC];
#pragma unroll
            for (int c = 0; c < MAXC; ++c) { hh[c] = 0.f; ll[c] = 0.f; }
            for (int64_t i = t + threadIdx.x; i < m; i += T) {
                const float2 vi = (i == t) ? make_float2(1.f, 0.f) : col[i];
#pragma unroll
                for (int c = 0; c < MAXC; ++c)
                    if (c < cnt) {
                        const float2 x = cols[(size_t)slot[c] * m + i];
                        ff_madd(vi.x, vi.y, x.x, x.y, hh[c], ll[c]);
                    }
            }
            block_sums<MAXC>(hh, ll, cnt, red, tot);
            for (int64_t i = t + threadIdx.x; i < m; i += T) {
                const float2 vi = (i == t) ? make_float2(1.f, 0.f) : col[i];
                for (int c = 0; c < cnt; ++c) {
                    const float2 f = ff_mul(tau, tot[c]);
                    float2* x = cols + (size_t)slot[c] * m + i;
                    *x = ff_add(*x, ff_neg(ff_mul(f, vi)));
                }
            }
            __syncthreads();
        }
    }
    // publish: reflectors and tau to global memory, then the flag
    for (int r = 0; r < KB; ++r) {
        const int64_t t = b * KB + r;
        if (t >= n) break;
        const float2* col = cols + (size_t)(q * KB + r) * m;
        for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) a.VF[i + t * m] = col[i];
        if (threadIdx.x == 0) a.tauF[t] = taus_local[r];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicExch(&a.flags[b], 1u);
    }
}

template <int OWNB>
__global__ void __launch_bounds__(T) qr_ff_kernel(Args a) {
    extern __shared__ __align__(16) float2 sm[];
    __shared__ float2 red[W * MAXC];
    __shared__ float2 tot[MAXC];
    __shared__ float2 taus[KB];
    __shared__ float2 taus_local[KB];
    const int64_t m = a.m, n = a.n, nc = a.nc, G = gridDim.x;
    float2* cols = sm;                                  // OWNB*KB columns of m
    float2* vb = sm + (size_t)OWNB * KB * m;            // the current reflector block, KB x m
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
            if (blk[q] < nblk && j < nc)
                for (int64_t i = threadIdx.x; i < m; i += T)
                    cols[(size_t)(q * KB + r) * m + i] = ff_split(a.X[i + j * a.ld]);
        }
    __syncthreads();
    if (blk[0] == 0 && nref > 0) factor_block(a, cols, 0, 0, red, tot, taus_local);
    for (int64_t rb = 0; rb < nref && rb < last; ++rb) {
        if (!wait_flag(&a.flags[rb], a.status)) return;
        for (int r = 0; r < KB; ++r) {
            const int64_t t = rb * KB + r;
            if (t >= n) break;
            for (int64_t i = t + 1 + threadIdx.x; i < m; i += T) vb[(size_t)r * m + i] = __ldcg(a.VF + i + t * m);
            if (threadIdx.x == 0) {
                const float2 tv = __ldcg(a.tauF + t);
                taus[r] = tv;
            }
        }
        __syncthreads();
        int la = -1;
#pragma unroll
        for (int q = 0; q < OWNB; ++q)
            if (blk[q] == rb + 1) la = q;
        // look-ahead: block rb + 1 first, factor and publish it
        if (la >= 0) {
            int slot[MAXC];
            int cnt = 0;
            for (int r = 0; r < KB; ++r)
                if ((rb + 1) * KB + r < nc) slot[cnt++] = la * KB + r;
            for (int r = 0; r < KB; ++r) {
                const int64_t t = rb * KB + r;
                if (t >= n) break;
                if (taus[r].x != 0.f) apply_reflector(a, vb + (size_t)r * m, taus[r], t, cols, slot, cnt, red, tot);
            }
            if (rb + 1 < nref) factor_block(a, cols, la, rb + 1, red, tot, taus_local);
        }
        // the other owned blocks after rb
        {
            int slot[MAXC];
            int cnt = 0;
#pragma unroll
            for (int q = 0; q < OWNB; ++q)
                if (q != la && blk[q] > rb && blk[q] < nblk)
                    for (int r = 0; r < KB; ++r)
                        if (blk[q] * KB + r < nc) slot[cnt++] = q * KB + r;
            if (cnt > 0)
                for (int r = 0; r < KB; ++r) {
                    const int64_t t = rb * KB + r;
                    if (t >= n) break;
                    if (taus[r].x != 0.f)
                        apply_reflector(a, vb + (size_t)r * m, taus[r], t, cols, slot, cnt, red, tot);
                }
        }
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

__global__ void __launch_bounds__(TI) rinv_ff_kernel(const double* __restrict__ R, int64_t n, int64_t ldr,
                                                     double* __restrict__ Ri, int64_t ldi,
                                                     unsigned int* __restrict__ singular) {
    extern __shared__ __align__(16) float2 smi[];
    float2* dinv = smi;          // n reciprocal pivots
    float2* t = smi + n;         // n: right-hand side / solution
    const int64_t j = blockIdx.x;
    for (int64_t k = threadIdx.x; k < n; k += TI) {
        const float2 d = ff_split(R[k + k * ldr]);
        if (d.x == 0.f) atomicExch(singular, 1u);
        dinv[k] = (d.x == 0.f) ? make_float2(0.f, 0.f) : ff_div(make_float2(1.f, 0.f), d);
        t[k] = make_float2(k == j ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    for (int64_t k = j; k >= 0; --k) {
        const float2 xk = ff_mul(t[k], dinv[k]);
        __syncthreads();
        if (threadIdx.x == 0) t[k] = xk;
        for (int64_t i = threadIdx.x; i < k; i += TI) {
            const float2 r = ff_split(R[i + k * ldr]);
            t[i] = ff_add(t[i], ff_neg(ff_mul(r, xk)));
        }
        __syncthreads();
    }
    for (int64_t i = threadIdx.x; i < n; i += TI)
        Ri[i + j * ldi] = (i <= j) ? ff_to_double(t[i]) : 0.0;
}

template <int OWNB>
static const void* qr_kernel() { return (const void*)qr_ff_kernel<OWNB>; }

}  // namespace qrff

// Whether the float-float QR fits: the owned column blocks and one
// reflector block in shared memory, one CTA per SM.
static int qr_ff_ownb(const Ctx& ctx, int64_t m, int64_t nc) {
    const int64_t nblk = (nc + qrff::KB - 1) / qrff::KB;
    const int64_t G = nblk < ctx.sm_count ? nblk : ctx.sm_count;
    const int64_t ownb = (nblk + G - 1) / G;
    if (ownb > qrff::MAX_OWNB) return 0;
    const size_t smem = (size_t)(ownb + 1) * qrff::KB * m * sizeof(float2);
    if (smem > 200 * 1024) return 0;
    return (int)ownb;
}

bool qr_ff_supported(const Ctx& ctx, int64_t m, int64_t n, int64_t nc) {
    return m >= n && n >= 1 && nc >= n && qr_ff_ownb(ctx, m, nc) > 0;
}

void householder_qr_ff(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld) {
    using namespace qrff;
    const int ownb = qr_ff_ownb(ctx, m, nc);
    if (ownb == 0 || m < n) fail(RNLA_ERR_UNSUPPORTED, "float-float QR: the sketch does not fit in shared memory");
    const int64_t nblk = (nc + KB - 1) / KB;
    const int64_t G = nblk < ctx.sm_count ? nblk : ctx.sm_count;
    const size_t smem = (size_t)(ownb + 1) * KB * m * sizeof(float2);
    const void* k = ownb == 1 ? qr_kernel<1>() : ownb == 2 ? qr_kernel<2>() : ownb == 3 ? qr_kernel<3>() : qr_kernel<4>();
    RNLA_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, T, smem));
    if ((int64_t)nb * ctx.sm_count < G) fail(RNLA_ERR_UNSUPPORTED, "float-float QR: grid not co-resident");
    cudaStream_t s = ctx.stream;
    const int64_t nref = (n + KB - 1) / KB;
    DevBuf<float2> VF((size_t)m * n, s), tauF(n, s);
    DevBuf<unsigned int> flags(nref, s);
    RNLA_CUDA(cudaMemsetAsync(flags.get(), 0, nref * sizeof(unsigned int), s));
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), s));
    Args a{X, m, n, nc, ld, VF.get(), tauF.get(), flags.get(), ctx.status};
    void* args[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3((unsigned)G), dim3(T), args, smem, s));
    count_launch();
    ctx.check_status("householder_qr (float-float)");
}

bool upper_inverse_ff(Ctx& ctx, const double* R, int64_t n, int64_t ldr, double* Rinv, int64_t ldi) {
    using namespace qrff;
    if (n <= 0) return true;
    const size_t smem = (size_t)2 * n * sizeof(float2);
    if (smem > 200 * 1024) fail(RNLA_ERR_UNSUPPORTED, "float-float R^-1: n too large");
    if (smem > 48 * 1024)
        RNLA_CUDA(cudaFuncSetAttribute(rinv_ff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    DevBuf<unsigned int> sing(1, ctx.stream);
    RNLA_CUDA(cudaMemsetAsync(sing.get(), 0, sizeof(unsigned int), ctx.stream));
    rinv_ff_kernel<<<(unsigned)n, TI, smem, ctx.stream>>>(R, n, ldr, Rinv, ldi, sing.get());
    RNLA_LAUNCH_CHECK();
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, sing.get(), sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    return h == 0;
}

}  // namespace rnla
