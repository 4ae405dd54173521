// Sketch-and-precondition CholeskyQR with column pivoting
// (cqrrpt.rs:27-58, sap_chol_qrcp) and the column-pivoted Householder QR it
// uses (pivot_decompositions.rs:106-174, qrcp).
//
//   S a (d x m sketch, Gaussian)  ->  QRCP of S a: R_sk, pivots j
//   k = #{ i : |R_sk[i][i]| > 1e-10 }, a_pre = a[:, j[:k]] R_sk[:k,:k]^-1
//   R_pre = chol(a_pre^T a_pre),  Q = a_pre R_pre^-1,  R = R_pre R_sk[:k, :]
//
// QRCP follows the reference's rule step by step, in FP64: at step k the
// column with the largest remaining norm (strictly larger; the first index
// on ties) moves to position k, v = x + sign(x_0) ||x|| e_0 normalised,
// every column from k on is reflected (c -= 2 v (v^T c)), and the norms of
// the later columns are recomputed below row k.  It runs in one CTA: the
// sketch is small (d x n with n <= d << m) and the pivot choice is a chain of
// n dependent steps.  Warps own columns, lanes own rows, so every dot
// product is a fixed-order warp reduction and the run is reproducible.
#include "rnla_internal.h"

namespace rnla {
namespace cq {

constexpr int T = 1024;
constexpr int NWARP = T / 32;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ||R[r0:d, j]|| by one warp
__device__ double col_norm(const double* R, int64_t d, int64_t ld, int64_t j, int64_t r0, int lane) {
    double s = 0.0;
    for (int64_t i = r0 + lane; i < d; i += 32) {
        const double x = R[i + j * ld];
        s = fma(x, x, s);
    }
    return sqrt(warp_sum_d(s));
}

__global__ void __launch_bounds__(T, 1) qrcp_kernel(double* __restrict__ R, int64_t d, int64_t n, int64_t ld,
                                                    int64_t* __restrict__ jpvt, double* __restrict__ norms,
                                                    double* __restrict__ v) {
    __shared__ double red_v[NWARP];
    __shared__ int64_t red_i[NWARP];
    __shared__ int64_t piv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int64_t j = warp; j < n; j += NWARP) {
        const double nr = col_norm(R, d, ld, j, 0, lane);
        if (lane == 0) {
            norms[j] = nr;
            jpvt[j] = j;
        }
    }
    __syncthreads();
    const int64_t steps = d < n ? d : n;
    for (int64_t k = 0; k < steps; ++k) {
        // argmax of norms[k..n): strictly larger wins, so the first index
        // stays on ties (pivot_decompositions.rs:119-127)
        double best = -1.0;
        int64_t bi = n;
        for (int64_t j = k + tid; j < n; j += T) {
            const double x = norms[j];
            if (x > best) { best = x; bi = j; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { red_v[warp] = best; red_i[warp] = bi; }
        __syncthreads();
        if (tid == 0) {
            double b = red_v[0];
            int64_t i = red_i[0];
            for (int w = 1; w < NWARP; ++w)
                if (red_v[w] > b || (red_v[w] == b && red_i[w] < i)) { b = red_v[w]; i = red_i[w]; }
            // the reference compares against norms[k] first: a later column
            // must be strictly larger to move
            if (!(norms[i] > norms[k])) i = k;
            piv = i;
        }
        __syncthreads();
        const int64_t p = piv;
        if (p != k) {
            for (int64_t i = tid; i < d; i += T) {
                const double a = R[i + k * ld];
                R[i + k * ld] = R[i + p * ld];
                R[i + p * ld] = a;
            }
            if (tid == 0) {
                const int64_t t = jpvt[k]; jpvt[k] = jpvt[p]; jpvt[p] = t;
                const double x = norms[k]; norms[k] = norms[p]; norms[p] = x;
            }
            __syncthreads();
        }
        // Householder vector of R[k:d, k]
        double s = 0.0;
        for (int64_t i = k + tid; i < d; i += T) {
            const double x = R[i + k * ld];
            s = fma(x, x, s);
        }
        s = block_sum(s, red_v);
        const double nx = sqrt(s);
        if (nx == 0.0) continue;                       // uniform: every thread has the same nx
        const double x0 = R[k + k * ld];
        const double v0 = x0 + (x0 >= 0.0 ? nx : -nx);
        // ||v||^2 = ||x||^2 - x0^2 + v0^2
        double vs = 0.0;
        for (int64_t i = k + 1 + tid; i < d; i += T) {
            const double x = R[i + k * ld];
            vs = fma(x, x, vs);
        }
        vs = block_sum(vs, red_v);
        const double inv = 1.0 / sqrt(fma(v0, v0, vs));
        for (int64_t i = k + tid; i < d; i += T) v[i] = (i == k ? v0 : R[i + k * ld]) * inv;
        __syncthreads();
        // reflect columns k..n-1 (warp per column), then the later columns' norms
        for (int64_t j = k + warp; j < n; j += NWARP) {
            double dp = 0.0;
            for (int64_t i = k + lane; i < d; i += 32) dp = fma(v[i], R[i + j * ld], dp);
            dp = warp_sum_d(dp);
            for (int64_t i = k + lane; i < d; i += 32) R[i + j * ld] -= 2.0 * v[i] * dp;
            __syncwarp();
            if (j > k) {
                const double nr = col_norm(R, d, ld, j, k + 1, lane);
                if (lane == 0) norms[j] = nr;
            }
        }
        __syncthreads();
    }
}

// out[:, c] = A[:, jpvt[c]], c < k
__global__ void gather_columns_kernel(const double* __restrict__ A, int64_t m, int64_t lda,
                                      const int64_t* __restrict__ jpvt, int64_t k, double* __restrict__ out,
                                      int64_t ldo) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < m * k;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % m, c = idx / m;
        out[i + c * ldo] = A[i + jpvt[c] * lda];
    }
}

// number of |R[i][i]| > tol, i < s
__global__ void count_rank_kernel(const double* __restrict__ R, int64_t s, int64_t ld, double tol,
                                  int64_t* __restrict__ k) {
    __shared__ double red[32];
    double c = 0.0;
    for (int64_t i = threadIdx.x; i < s; i += blockDim.x) c += (fabs(R[i + i * ld]) > tol) ? 1.0 : 0.0;
    c = block_sum(c, red);
    if (threadIdx.x == 0) *k = (int64_t)c;
}

// dst = upper triangle of src (n x n), zeros below
__global__ void upper_copy_kernel(const double* __restrict__ src, int64_t lds, int64_t n,
                                  double* __restrict__ dst, int64_t ldd) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        dst[i + j * ldd] = (i <= j) ? src[i + j * lds] : 0.0;
    }
}

}  // namespace cq

static void copy_upper(Ctx& ctx, int64_t n, const double* src, int64_t lds, double* dst, int64_t ldd) {
    int g = (int)div_up(n * n, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    cq::upper_copy_kernel<<<g, 256, 0, ctx.stream>>>(src, lds, n, dst, ldd);
    RNLA_LAUNCH_CHECK();
}

void qrcp(Ctx& ctx, double* R, int64_t d, int64_t n, int64_t ld, int64_t* jpvt) {
    if (d <= 0 || n <= 0) return;
    DevBuf<double> norms(n, ctx.stream), v(d, ctx.stream);
    cq::qrcp_kernel<<<1, cq::T, 0, ctx.stream>>>(R, d, n, ld, jpvt, norms, v);
    RNLA_LAUNCH_CHECK();
}

void sap_chol_qrcp(Ctx& ctx, const RngKey& key, int precision, int digits, const double* A, int64_t m,
                   int64_t n, int64_t lda, int64_t d, double* Q, int64_t ldq, double* Rout, int64_t ldr,
                   int64_t* jpvt_dev) {
    if (!(n <= d && d <= m) || n <= 0)
        fail(RNLA_ERR_INVALID_PARAMETERS, "d must satisfy n <= d << m");
    // S a (cqrrpt.rs:31-33)
    DevBuf<double> SA((size_t)d * n, ctx.stream);
    if (precision == RNLA_PREC_FP64) {
        DevBuf<double> S((size_t)d * m, ctx.stream);
        sketch_fill_f64(ctx, DIST_GAUSSIAN, key, d, m, S, d);
        gemm_f64(ctx, 'N', 'N', d, n, m, 1.0, S, d, A, lda, 0.0, SA, d);
    } else {
        if (!tc_available(ctx)) fail(RNLA_ERR_UNSUPPORTED, "sm_103a tensor-core kernels unavailable");
        tc_sketch_apply(ctx, key, A, false, m, n, lda, nullptr, d, digits, SA, d);
    }
    // QRCP of the sketch, numerical rank with the reference's 1e-10 (lines 35-43)
    qrcp(ctx, SA, d, n, d, jpvt_dev);
    DevBuf<int64_t> kdev(1, ctx.stream);
    cq::count_rank_kernel<<<1, 256, 0, ctx.stream>>>(SA, n < d ? n : d, d, 1e-10, kdev);
    RNLA_LAUNCH_CHECK();
    int64_t k = 0;
    RNLA_CUDA(cudaMemcpyAsync(&k, kdev.get(), sizeof k, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    if (k < n)
        fail(RNLA_ERR_SINGULAR_MATRIX, "the sketch's pivoted R has numerical rank below n (the reference "
                                       "panics on the dimension mismatch that follows)");
    // a_pre = a[:, j] R_sk^-1 (lines 45-48)
    DevBuf<double> Ap((size_t)m * n, ctx.stream), Rk((size_t)n * n, ctx.stream), Rki((size_t)n * n, ctx.stream),
        Apre((size_t)m * n, ctx.stream);
    {
        int g = (int)div_up(m * n, 256);
        if (g > 16 * ctx.sm_count) g = 16 * ctx.sm_count;
        cq::gather_columns_kernel<<<g, 256, 0, ctx.stream>>>(A, m, lda, jpvt_dev, n, Ap, m);
        RNLA_LAUNCH_CHECK();
    }
    copy_upper(ctx, n, SA, d, Rk, n);
    if (!upper_inverse(ctx, Rk, n, n, Rki, n)) fail(RNLA_ERR_SINGULAR_MATRIX, "the sketch's R is singular");
    gemm_f64(ctx, 'N', 'N', m, n, n, 1.0, Ap, m, Rki, n, 0.0, Apre, m);
    // R_pre = chol(a_pre^T a_pre)^T (lines 50-52)
    DevBuf<double> G((size_t)n * n, ctx.stream), Gi((size_t)n * n, ctx.stream);
    gemm_f64(ctx, 'T', 'N', n, n, m, 1.0, Apre, m, Apre, m, 0.0, G, n);
    if (!cholesky_upper(ctx, G, n, n))
        fail(RNLA_ERR_MATRIX_DECOMPOSITION, "Cholesky decomposition failed");
    // Q = a_pre R_pre^-1, R = R_pre R_sk[:k, :] (lines 53-55)
    if (!upper_inverse(ctx, G, n, n, Gi, n)) fail(RNLA_ERR_SINGULAR_MATRIX, "R_pre is singular");
    gemm_f64(ctx, 'N', 'N', m, n, n, 1.0, Apre, m, Gi, n, 0.0, Q, ldq);
    DevBuf<double> Gu((size_t)n * n, ctx.stream);
    copy_upper(ctx, n, G, n, Gu, n);
    gemm_f64(ctx, 'N', 'N', n, n, n, 1.0, Gu, n, Rk, n, 0.0, Rout, ldr);
}

}  // namespace rnla
