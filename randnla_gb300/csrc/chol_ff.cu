// Blocked Cholesky G = R^T R in float-float on the FP32 pipe, for the
// tensor-core paths whose Grams are themselves float-float (~2^-48): the
// CholeskyQR passes and the final basis of the tensor-core rand_svd, the
// Gram-based small SVD, the CholeskyQR R of wide least-squares sketches.
//
// Same data flow as cholesky_blocked_kernel (factor.cu) -- panels of 32
// rows, every CTA factors the panel's diagonal block redundantly (all of its
// threads, in shared memory, one __syncthreads per pivot), forms the panel
// rows of its own columns by forward substitution, grid barrier, subtracts
// R[K][i]^T R[K][j] from its own columns, grid barrier -- with every
// operation a float-float one (exact products through FMA, TwoSum accumulation): on GB300 a
// dependent FP64 operation costs ~64 cycles and a warp's FP64 FMA occupies a
// sub-partition's FP64 unit for 64 cycles, so the FP64 kernel spends ~30 us
// per panel in the diagonal block alone.  The matrix lives as (hi, lo)
// pairs in a workspace for the duration of the factorization.
#include "rnla_internal.h"
#include "rnla_ff.cuh"

namespace rnla {
namespace cff {

constexpr int CB = 32;
constexpr int CT = 256;
constexpr int MAXQ = 32;                 // owned columns per CTA: n <= MAXQ x grid

// 1 / sqrt(d), d > 0: FP32 estimate, one Newton step y + y (1 - d y^2) / 2
// with the residual 1 - d y^2 formed in float-float (~44 bits)
__device__ __forceinline__ float2 ff_rsqrt(float2 d) {
    const float y = rsqrtf(d.x);
    const float p = __fmul_rn(y, y);
    const float pe = __fmaf_rn(y, y, -p);
    const float2 dy2 = ff_mul(d, make_float2(p, pe));
    const float2 e = ff_add(make_float2(1.f, 0.f), ff_neg(dy2));
    return ff_norm(y, __fmul_rn(__fmul_rn(y, 0.5f), e.x));
}

// c - a b
__device__ __forceinline__ float2 ff_fms(float2 c, float2 a, float2 b) { return ff_add(c, ff_neg(ff_mul(a, b))); }

__device__ __forceinline__ float2 ff_shfl(float2 v, int src) {
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

__global__ void __launch_bounds__(CT) chol_ff_kernel(float2* __restrict__ F, int64_t n, int64_t npd,
                                                     unsigned int* status, GridBarrier bar) {
    __shared__ float2 Ds[CB][CB + 1];
    __shared__ float2 ris[CB];
    __shared__ float2 Ps[CB][64 + 1];
    __shared__ float2 Rjs[MAXQ][CB];
    __shared__ int bad_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Gc = gridDim.x, c = blockIdx.x;
    const float2 z2 = make_float2(0.f, 0.f);
    for (int64_t k0 = 0; k0 < npd; k0 += CB) {
        const int kb = (int)(npd - k0 < CB ? npd - k0 : CB);
        const int64_t k1 = k0 + kb;
        // (1) diagonal block
        for (int e = tid; e < CB * CB; e += CT) {
            const int i = e % CB, j = e / CB;
            Ds[i][j] = (i <= j && j < kb) ? F[(k0 + i) + (k0 + j) * n] : z2;
        }
        if (tid == 0) bad_s = 0;
        __syncthreads();
        // every thread takes up to two entries (i, c), t < i <= c, of the block
        // per step and subtracts (G[t][i] / sqrt(d)) (G[t][c] / sqrt(d)) with the
        // unscaled pivot row (no one writes row t during step t); row t is
        // scaled once the pivots are known.  One __syncthreads per pivot.
        for (int t = 0; t < kb; ++t) {
            const float2 d = Ds[t][t];
            if (!(d.x > 0.f)) {
                if (tid == 0) bad_s = 1;
                break;
            }
            const float2 ri = ff_rsqrt(d);
            if (tid == 0) ris[t] = ri;
            const int w = kb - t - 1;                     // trailing block size
            for (int e = tid; e < w * w; e += CT) {
                const int i = t + 1 + e % w, cc = t + 1 + e / w;
                if (i <= cc) Ds[i][cc] = ff_fms(Ds[i][cc], ff_mul(Ds[t][i], ri), ff_mul(Ds[t][cc], ri));
            }
            __syncthreads();
        }
        __syncthreads();
        if (!bad_s)
            for (int e = tid; e < kb * kb; e += CT) {
                const int t = e % kb, cc = e / kb;
                if (t <= cc) Ds[t][cc] = ff_mul(Ds[t][cc], ris[t]);     // R[t][c]; R[t][t] = d / sqrt(d)
            }
        __syncthreads();
        if (bad_s) {
            if (tid == 0) atomicCAS(status, 0u, (unsigned int)KSTATUS_NOT_PD);
            return;
        }
        // (2) panel rows of the owned trailing columns: R_KK^T x = g
        const int64_t jfirst = k1 + ((c - k1 % Gc) % Gc + Gc) % Gc;
        for (int64_t j = jfirst + (int64_t)warp * Gc; j < n; j += (int64_t)(CT / 32) * Gc) {
            float2 g = lane < kb ? F[(k0 + lane) + j * n] : z2;
            for (int s = 0; s < kb; ++s) {
                const float2 xs = ff_mul(ff_shfl(g, s), ris[s]);
                if (lane == s) g = xs;
                else if (lane > s && lane < kb) g = ff_fms(g, Ds[s][lane], xs);
            }
            if (lane < kb) F[(k0 + lane) + j * n] = g;
        }
        if (!grid_sync(bar)) return;
        // every CTA has read the diagonal block: R_KK replaces it
        if (c == 0)
            for (int e = tid; e < kb * kb; e += CT) {
                const int i = e % kb, j = e / kb;
                if (i <= j) F[(k0 + i) + (k0 + j) * n] = Ds[i][j];
            }
        // (3) trailing update of the owned columns j = jfirst + q Gc
        if (jfirst < n) {
            const int nq = (int)((n - 1 - jfirst) / Gc) + 1;
            const int64_t jlast = jfirst + (int64_t)(nq - 1) * Gc;
            for (int e = tid; e < nq * CB; e += CT) {
                const int q = e / CB, t = e % CB;
                Rjs[q][t] = t < kb ? F[(k0 + t) + (jfirst + (int64_t)q * Gc) * n] : z2;
            }
            const int r = tid & 63, cg = tid >> 6;
            // the panel rows of the next 64 columns are loaded into registers
            // while the current block is applied (their L2 round trip
            // overlaps the multiply-adds), then staged into shared memory
            constexpr int PRE = CB * 64 / CT;
            float2 pre[PRE];
#pragma unroll
            for (int u = 0; u < PRE; ++u) {
                const int e = tid + u * CT;
                const int t = e % CB, rr = e / CB;
                pre[u] = (t < kb && k1 + rr < n) ? F[(k0 + t) + (k1 + rr) * n] : z2;
            }
            for (int64_t i0 = k1; i0 <= jlast; i0 += 64) {
                __syncthreads();
#pragma unroll
                for (int u = 0; u < PRE; ++u) {
                    const int e = tid + u * CT;
                    Ps[e % CB][e / CB] = pre[u];
                }
                __syncthreads();
                const int64_t i1 = i0 + 64;
                if (i1 <= jlast) {
#pragma unroll
                    for (int u = 0; u < PRE; ++u) {
                        const int e = tid + u * CT;
                        const int t = e % CB, rr = e / CB;
                        pre[u] = (t < kb && i1 + rr < n) ? F[(k0 + t) + (i1 + rr) * n] : z2;
                    }
                }
                const int64_t i = i0 + r;
                const int q0 = i0 > jfirst ? (int)((i0 - jfirst + Gc - 1) / Gc) : 0;
                for (int q = q0 + cg; q < nq; q += 4) {
                    const int64_t j = jfirst + (int64_t)q * Gc;
                    if (i > j) continue;
                    float sh = 0.f, sl = 0.f;
#pragma unroll 8
                    for (int t = 0; t < CB; ++t) {
                        const float2 a = Ps[t][r], b = Rjs[q][t];
                        ff_madd(a.x, a.y, b.x, b.y, sh, sl);
                    }
                    F[i + j * n] = ff_add(F[i + j * n], ff_neg(ff_norm(sh, sl)));
                }
            }
        }
        if (!grid_sync(bar)) return;
    }
}

// F (n x n float-float, ld n) <- upper triangle of G; strict lower zero
__global__ void to_ff_kernel(const double* __restrict__ G, int64_t n, int64_t ld, float2* __restrict__ F) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % n, j = e / n;
        F[e] = i <= j ? ff_split(G[i + j * ld]) : make_float2(0.f, 0.f);
    }
}

// G <- R (upper, strict lower zero); the diagonal of columns beyond npd is
// the residual norm sqrt(max(0, .)) of the bordered column
__global__ void from_ff_kernel(const float2* __restrict__ F, int64_t n, int64_t npd, double* __restrict__ G,
                               int64_t ld) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % n, j = e / n;
        double v = 0.0;
        if (i < j || (i == j && i < npd)) v = ff_to_double(F[e]);
        else if (i == j) v = sqrt(fmax(ff_to_double(F[e]), 0.0));
        G[i + j * ld] = v;
    }
}

}  // namespace cff

bool cholesky_upper_ff(Ctx& ctx, double* G, int64_t n, int64_t ld, int64_t npd) {
    using namespace cff;
    if (npd < 0) npd = n;
    if (n <= 0) return true;
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, chol_ff_kernel, CT, 0));
    int Gs = ctx.sm_count;
    if (Gs > nb * ctx.sm_count) Gs = nb * ctx.sm_count;
    if (Gs > n) Gs = (int)n;
    if (Gs < 1) Gs = 1;
    if (n > (int64_t)MAXQ * Gs) fail(RNLA_ERR_INVALID_DIMENSIONS, "float-float Cholesky: n above the kernel's limit");
    DevBuf<float2> F((size_t)n * n, ctx.stream);
    int g = div_up(n * n, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    to_ff_kernel<<<g, 256, 0, ctx.stream>>>(G, n, ld, F);
    RNLA_LAUNCH_CHECK();
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    DevBuf<unsigned int> bw(2, ctx.stream);
    RNLA_CUDA(cudaMemsetAsync(bw.get(), 0, 2 * sizeof(unsigned int), ctx.stream));
    GridBarrier bar{bw.get(), bw.get() + 1, ctx.status};
    float2* Fp = F.get();
    void* args[] = {&Fp, &n, &npd, &ctx.status, &bar};
    RNLA_CUDA(cudaLaunchCooperativeKernel((const void*)chol_ff_kernel, dim3((unsigned)Gs), dim3(CT), args, 0,
                                          ctx.stream));
    count_launch();
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, ctx.status, sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    if (h == KSTATUS_NOT_PD) return false;
    if (h != KSTATUS_OK) throw Error(RNLA_ERR_TIMEOUT, "float-float Cholesky: a grid barrier exceeded its limit");
    from_ff_kernel<<<g, 256, 0, ctx.stream>>>(F, n, npd, G, ld);
    RNLA_LAUNCH_CHECK();
    return true;
}

}  // namespace rnla
