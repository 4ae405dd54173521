// Eigenvectors of a small SPD Gram G = B B^T (p x p, 2 <= p <= 320) for the
// Gram-based small SVD of the tensor-core rand_svd, in two stages:
//
//  1. one-sided Jacobi in FP32 on W = R^T (R = chol(G)) on one thread-block
//     cluster of 8 CTAs whose shared memories hold W: column c lives in CTA
//     c % 8 at slot c / 8, each warp of the cluster owns one position of the
//     round-robin pairing, reads its two columns through distributed shared
//     memory, reduces alpha, beta, gamma with shuffles and rotates.  A round
//     ends with a cluster barrier (hardware, a few hundred cycles) where the
//     FP64 grid version pays a global-memory barrier and FP64 arithmetic at
//     1/64 of the FP32 rate -- about 10 us per round on GB300 against well
//     under 1 us here, with ~300 rounds per sweep and 8-11 sweeps.  The
//     normalised columns of W approximate the eigenvectors of G to FP32
//     accuracy (R^T = W V^T with V orthogonal gives G = R^T R = W W^T).
//  2. float-float Rayleigh-Ritz refinement (every product on gram_ff):
//     Newton-Schulz orthonormalisation U <- U (3 I - U^T U) / 2, H = U^T G U,
//     and the rotation U <- U (I + E) with E_ij the Jacobi tangent of
//     (H_ii, H_jj, H_ij) -- to first order H_ij / (H_jj - H_ii), bounded by 1
//     when the two are close -- which squares the eigenvector error per
//     step; three steps take FP32 accuracy past float-float, a final
//     orthonormalisation and Rayleigh quotient give U and sigma^2 = diag(H).
// The caller falls back to the FP64 Jacobi when the refined H keeps an
// off-diagonal entry above 2^-40 of its diagonal (plus the products' own
// rounding level): clusters the tangent step does not resolve.
#include "rnla_internal.h"
#include <cooperative_groups.h>

namespace rnla {
namespace eigr {

constexpr int JC = 8;                // CTAs of the cluster
constexpr int JE = 10;               // column entries per lane (p <= 320)
constexpr int PMAX = 32 * JE;

__global__ void __cluster_dims__(JC, 1, 1) __launch_bounds__(640, 1)
    jacobi_f32_cluster_kernel(float* __restrict__ W, int s, int max_sweeps, unsigned int* __restrict__ sweeps_out) {
    namespace cg = cooperative_groups;
    extern __shared__ float wsm[];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int cw = (s + JC - 1) / JC;
    float* Ws = wsm;
    unsigned int* cnt = (unsigned int*)(wsm + (size_t)cw * s);
    for (int e = threadIdx.x; e < cw * s; e += blockDim.x) {
        const int slot = e / s, i = e % s, c = slot * JC + rank;
        Ws[e] = c < s ? W[i + (int64_t)c * s] : 0.f;
    }
    if (threadIdx.x < 2) cnt[threadIdx.x] = 0u;
    cl.sync();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int sp = (s + 1) & ~1, npairs = sp / 2;
    const int pr = rank * nwarps + warp;
    // FP32 rounding of an s-term dot product
    const float tol = (float)s * 0x1p-24f;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        for (int round = 0; round < sp - 1; ++round) {
            int a = s, b = s;
            if (pr < npairs) {
                if (pr == 0) { a = 0; b = 1 + (round % (sp - 1)); }
                else {
                    a = 1 + ((round + pr) % (sp - 1));
                    b = 1 + ((round + sp - 1 - pr) % (sp - 1));
                }
                if (a > b) { const int t = a; a = b; b = t; }
            }
            if (a < s && b < s) {                        // uniform over the warp
                float* wa = cl.map_shared_rank(Ws + (size_t)(a / JC) * s, (unsigned)(a % JC));
                float* wb = cl.map_shared_rank(Ws + (size_t)(b / JC) * s, (unsigned)(b % JC));
                float x[JE], y[JE];
                float al = 0.f, be = 0.f, ga = 0.f;
#pragma unroll
                for (int e = 0; e < JE; ++e) {
                    const int i = lane + 32 * e;
                    x[e] = i < s ? wa[i] : 0.f;
                    y[e] = i < s ? wb[i] : 0.f;
                }
#pragma unroll
                for (int e = 0; e < JE; ++e) {
                    al = fmaf(x[e], x[e], al);
                    be = fmaf(y[e], y[e], be);
                    ga = fmaf(x[e], y[e], ga);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    al += __shfl_xor_sync(0xffffffffu, al, o);
                    be += __shfl_xor_sync(0xffffffffu, be, o);
                    ga += __shfl_xor_sync(0xffffffffu, ga, o);
                }
                if (ga != 0.f && fabsf(ga) > tol * sqrtf(al * be)) {
                    // t = tan of the rotation angle, the root of t^2 + 2 zeta t - 1 with
                    // |t| <= 1, zeta = (beta - alpha) / (2 gamma)
                    const float tau = be - al;
                    const float h = sqrtf(fmaf(tau, tau, 4.f * ga * ga));
                    const float t = 2.f * ga / (tau >= 0.f ? tau + h : tau - h);
                    const float c = rsqrtf(fmaf(t, t, 1.f));
                    const float sn = c * t;
#pragma unroll
                    for (int e = 0; e < JE; ++e) {
                        const int i = lane + 32 * e;
                        if (i < s) {
                            wa[i] = c * x[e] - sn * y[e];
                            wb[i] = sn * x[e] + c * y[e];
                        }
                    }
                    if (lane == 0) atomicAdd(&cnt[sweep & 1], 1u);
                }
            }
            cl.sync();
        }
        unsigned int tot = 0u;
        for (int r = 0; r < JC; ++r) tot += *((volatile unsigned int*)cl.map_shared_rank(&cnt[sweep & 1], (unsigned)r));
        cl.sync();
        if (threadIdx.x == 0) cnt[sweep & 1] = 0u;
        if (tot == 0u) break;
    }
    if (rank == 0 && threadIdx.x == 0 && sweeps_out) *sweeps_out = (unsigned int)(sweep < max_sweeps ? sweep + 1 : sweep);
    cl.sync();
    for (int e = threadIdx.x; e < cw * s; e += blockDim.x) {
        const int slot = e / s, i = e % s, c = slot * JC + rank;
        if (c < s) W[i + (int64_t)c * s] = Ws[e];
    }
}

// W (FP32, p x p) <- R^T, R the upper triangle of G (FP64, ld p)
__global__ void rt_f32_kernel(const double* __restrict__ R, int64_t p, float* __restrict__ W) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < p * p; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % p, j = e / p;          // W[i][j] = R[j][i]
        W[e] = j <= i ? (float)R[j + i * p] : 0.f;
    }
}

// U (FP64) <- the columns of W normalised (one CTA per column)
__global__ void normalize_cols_kernel(const float* __restrict__ W, int64_t p, double* __restrict__ U) {
    __shared__ double red[8];
    const int64_t j = blockIdx.x;
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < p; i += blockDim.x) {
        const double v = W[i + j * p];
        acc = fma(v, v, acc);
    }
    acc = block_sum(acc, red);
    const double inv = acc > 0.0 ? 1.0 / sqrt(acc) : 0.0;
    for (int64_t i = threadIdx.x; i < p; i += blockDim.x) U[i + j * p] = acc > 0.0 ? W[i + j * p] * inv : (i == j ? 1.0 : 0.0);
}

// N = (3 I - S) / 2
__global__ void ns_factor_kernel(double* __restrict__ S, int64_t p) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < p * p; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % p, j = e / p;
        S[e] = 0.5 * ((i == j ? 3.0 : 0.0) - S[e]);
    }
}

// Convergence of H: the largest |H_ij| / (2^-40 sqrt(H_ii H_jj) + 2^-44 max_k H_kk)
// over i != j (the second term is the float-float products' own rounding
// level on the small eigenvalues); one value per block in off_out
__global__ void offdiag_kernel(const double* __restrict__ H, int64_t p, double* __restrict__ off_out) {
    __shared__ double red[256];
    double hm = 0.0;
    for (int64_t k = threadIdx.x; k < p; k += blockDim.x) hm = fmax(hm, H[k + k * p]);
    red[threadIdx.x] = hm;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    hm = red[0];
    __syncthreads();
    double mx = 0.0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < p * p; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % p, j = e / p;
        if (i == j) continue;
        const double hij = 0.5 * (H[i + j * p] + H[j + i * p]);
        const double hii = H[i + i * p], hjj = H[j + j * p];
        mx = fmax(mx, fabs(hij) / (0x1p-40 * sqrt(fabs(hii * hjj)) + 0x1p-44 * hm));
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) off_out[blockIdx.x] = red[0];
}
__global__ void tangent_apply_kernel(const double* __restrict__ H, int64_t p, double* __restrict__ IE) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < p * p; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % p, j = e / p;
        if (i == j) { IE[e] = 1.0; continue; }
        // rotation of columns (i, j) of U that zeroes the (i, j) entry of H:
        // U_i' = U_i - t U_j, U_j' = t U_i + U_j with t the tangent below, so
        // (I + E)[j][i] = -t, (I + E)[i][j] = t for i < j
        const int64_t a = i < j ? i : j, b = i < j ? j : i;
        const double hab = 0.5 * (H[a + b * p] + H[b + a * p]);
        const double tau = H[b + b * p] - H[a + a * p];
        double t = 0.0;
        if (hab != 0.0) {
            const double h = sqrt(fma(tau, tau, 4.0 * hab * hab));
            t = 2.0 * hab / (tau >= 0.0 ? tau + h : tau - h);
        }
        IE[e] = (i < j) ? t : -t;
    }
}

// sigma_r = sqrt(H_cc) in descending order, U_B[:, r] = U[:, c] (one CTA)
__global__ void order_kernel(const double* __restrict__ H, const double* __restrict__ U, int64_t p,
                             double* __restrict__ UB, int64_t ldu, double* __restrict__ sigma) {
    extern __shared__ double dg[];
    for (int64_t c = threadIdx.x; c < p; c += blockDim.x) dg[c] = sqrt(fmax(H[c + c * p], 0.0));
    __syncthreads();
    for (int64_t c = threadIdx.x; c < p; c += blockDim.x) {
        int64_t rank = 0;
        for (int64_t d = 0; d < p; ++d)
            if (dg[d] > dg[c] || (dg[d] == dg[c] && d < c)) ++rank;
        sigma[rank] = dg[c];
        for (int64_t i = 0; i < p; ++i) UB[i + rank * ldu] = U[i + c * p];
    }
}

}  // namespace eigr

bool eig_gram_refined(Ctx& ctx, const double* G, const double* R, int64_t p, double* UB, int64_t ldu, double* sigma,
                      int* sweeps) {
    using namespace eigr;
    if (p < 2 || p > PMAX) return false;
    DevBuf<float> W32((size_t)p * p, ctx.stream);
    int g = div_up(p * p, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    rt_f32_kernel<<<g, 256, 0, ctx.stream>>>(R, p, W32);
    RNLA_LAUNCH_CHECK();
    DevBuf<unsigned int> nsw(1, ctx.stream);
    RNLA_CUDA(cudaMemsetAsync(nsw.get(), 0, sizeof(unsigned int), ctx.stream));
    {
        const int cw = (int)((p + JC - 1) / JC);
        const size_t smem = (size_t)cw * p * sizeof(float) + 16;
        const int npairs = (int)((p + 1) / 2);
        const int nwarps = (npairs + JC - 1) / JC;
        set_smem_limit((const void*)jacobi_f32_cluster_kernel, smem);
        jacobi_f32_cluster_kernel<<<JC, 32 * nwarps, smem, ctx.stream>>>(W32, (int)p, 40, nsw);
        RNLA_LAUNCH_CHECK();
    }
    const size_t pp = (size_t)p * p;
    DevBuf<double> U(pp, ctx.stream), Ut(pp, ctx.stream), S(pp, ctx.stream), T(pp, ctx.stream), H(pp, ctx.stream),
        offb(64, ctx.stream);
    normalize_cols_kernel<<<(unsigned)p, 256, 0, ctx.stream>>>(W32, p, U);
    RNLA_LAUNCH_CHECK();
    // U <- U N with N = (3 I - U^T U) / 2
    auto orthonormalize_ns = [&]() {
        gram_ff(ctx, U, p, p, U, p, p, p, S, p);
        ns_factor_kernel<<<g, 256, 0, ctx.stream>>>(S, p);
        RNLA_LAUNCH_CHECK();
        transpose(ctx, p, p, U, p, Ut, p);
        gram_ff(ctx, Ut, p, p, S, p, p, p, U, p);
    };
    auto rayleigh = [&]() {
        gram_ff(ctx, G, p, p, U, p, p, p, T, p);                 // G U (G symmetric)
        gram_ff(ctx, U, p, p, T, p, p, p, H, p);                 // U^T G U
    };
    for (int it = 0; it < 3; ++it) {
        orthonormalize_ns();
        rayleigh();
        tangent_apply_kernel<<<g, 256, 0, ctx.stream>>>(H, p, S);
        RNLA_LAUNCH_CHECK();
        transpose(ctx, p, p, U, p, Ut, p);
        gram_ff(ctx, Ut, p, p, S, p, p, p, U, p);                // U (I + E)
    }
    orthonormalize_ns();
    orthonormalize_ns();
    rayleigh();
    const int gb = 64;
    offdiag_kernel<<<gb, 256, 0, ctx.stream>>>(H, p, offb);
    RNLA_LAUNCH_CHECK();
    double offh[64];
    unsigned int hsw = 0;
    RNLA_CUDA(cudaMemcpyAsync(offh, offb.get(), gb * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaMemcpyAsync(&hsw, nsw.get(), sizeof hsw, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    if (sweeps) *sweeps = (int)hsw;
    double off = 0.0;
    for (int i = 0; i < gb; ++i) off = off > offh[i] ? off : offh[i];
    if (!(off <= 1.0)) return false;
    order_kernel<<<1, 256, (size_t)p * sizeof(double), ctx.stream>>>(H, U, p, UB, ldu, sigma);
    RNLA_LAUNCH_CHECK();
    return true;
}

}  // namespace rnla
