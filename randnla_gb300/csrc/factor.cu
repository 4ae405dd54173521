// Dense FP64 factorizations used by the hot path:
//   * Householder QR (lora_helpers.rs:132 `qr().q()`; sketch_and_precondition.rs:53)
//   * triangular inverse / solves (sketch_and_precondition.rs:55; solvers.rs:22-41)
//   * Cholesky and CholeskyQR2 with a Householder fallback (range basis)
//   * complete-pivoting LU, L factor only (lora_helpers.rs:144-146)
//   * one-sided Jacobi SVD of a small matrix (lora_drivers.rs:53 `B.svd`)
// All run on the GPU in FP64.
#include "rnla_internal.h"
#include <vector>

namespace rnla {

// ---------------------------------------------------------------------------
// Householder QR, one launch per column.  Launch t applies reflector t-1 to
// every column j >= t and, in the CTA that owns column t, builds reflector t
// (LAPACK dlarfg convention: tau = 0 when the sub-column is exactly zero).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) hh_step_kernel(double* __restrict__ X, int64_t m, int64_t n,
                                                      int64_t ld, int64_t t, int64_t jfirst,
                                                      double* __restrict__ tau) {
    __shared__ double red[8];
    const int64_t j = jfirst + blockIdx.x;
    double* col = X + j * ld;
    if (t > 0) {
        const int64_t p = t - 1;
        const double tp = tau[p];
        if (tp != 0.0) {
            const double* v = X + p * ld;
            double s = 0.0;
            for (int64_t i = p + 1 + threadIdx.x; i < m; i += blockDim.x) s = fma(v[i], col[i], s);
            s = block_sum(s, red) + col[p];
            const double f = tp * s;
            if (threadIdx.x == 0) col[p] -= f;
            for (int64_t i = p + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] = fma(-f, v[i], col[i]);
        }
    }
    if (j == t && t < n) {
        __syncthreads();
        double s = 0.0;
        for (int64_t i = t + 1 + threadIdx.x; i < m; i += blockDim.x) s = fma(col[i], col[i], s);
        const double xn2 = block_sum(s, red);
        const double alpha = col[t];
        if (xn2 == 0.0) {
            if (threadIdx.x == 0) tau[t] = 0.0;
        } else {
            const double beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
            const double scale = 1.0 / (alpha - beta);
            for (int64_t i = t + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] *= scale;
            if (threadIdx.x == 0) {
                tau[t] = (beta - alpha) / beta;
                col[t] = beta;
            }
        }
    }
}

// The same factorization as one cooperative launch: CTA c owns columns
// c, c + G, ... (at most QR_OWN); step t applies reflector t-1 to the owned
// columns j >= t, the owner of column t then builds reflector t, and a
// bounded grid barrier publishes it.  n + 1 barriers instead of n + 1 launches.
constexpr int QR_OWN = 4;

__global__ void __launch_bounds__(256) hh_qr_coop_kernel(double* __restrict__ X, int64_t m, int64_t n,
                                                         int64_t nc, int64_t ld, double* __restrict__ tau,
                                                         GridBarrier bar) {
    __shared__ double red[8];
    const int64_t G = gridDim.x;
    for (int64_t t = 0; t <= n; ++t) {
        if (t > 0) {
            const int64_t p = t - 1;
            const double tp = tau[p];
            if (tp != 0.0) {
                const double* v = X + p * ld;
                double dot[QR_OWN];
#pragma unroll
                for (int q = 0; q < QR_OWN; ++q) dot[q] = 0.0;
                for (int64_t i = p + 1 + threadIdx.x; i < m; i += blockDim.x) {
                    const double vi = v[i];
#pragma unroll
                    for (int q = 0; q < QR_OWN; ++q) {
                        const int64_t j = blockIdx.x + q * G;
                        if (j >= t && j < nc) dot[q] = fma(vi, X[i + j * ld], dot[q]);
                    }
                }
#pragma unroll
                for (int q = 0; q < QR_OWN; ++q) {
                    const int64_t j = blockIdx.x + q * G;
                    if (j >= t && j < nc) {                       // uniform across the CTA
                        double* col = X + j * ld;
                        const double s = block_sum(dot[q], red) + col[p];
                        const double f = tp * s;
                        if (threadIdx.x == 0) col[p] -= f;
                        for (int64_t i = p + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] = fma(-f, v[i], col[i]);
                    }
                }
            }
        }
        if (t < n && (t % G) == (int64_t)blockIdx.x) {
            __syncthreads();
            double* col = X + t * ld;
            double sacc = 0.0;
            for (int64_t i = t + 1 + threadIdx.x; i < m; i += blockDim.x) sacc = fma(col[i], col[i], sacc);
            const double xn2 = block_sum(sacc, red);
            const double alpha = col[t];
            if (xn2 == 0.0) {
                if (threadIdx.x == 0) tau[t] = 0.0;
            } else {
                const double beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
                const double scale = 1.0 / (alpha - beta);
                for (int64_t i = t + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] *= scale;
                if (threadIdx.x == 0) {
                    tau[t] = (beta - alpha) / beta;
                    col[t] = beta;
                }
            }
        }
        if (t < n && !grid_sync(bar)) return;
    }
}

// Flag-pipelined variant: each CTA keeps its owned columns (c, c + G, ...)
// in shared memory.  Step t: wait until reflector t-1 is published
// (flags[t-1], bounded wait), apply it to the owned columns -- the owner of
// column t first, which then builds reflector t, writes it to global memory
// and raises flags[t] before updating its other columns.  No grid-wide
// barrier sits on the critical path: a step costs one flag hand-off plus
// one column update.
__device__ __forceinline__ bool wait_flag(const unsigned int* f, unsigned int* status) {
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

template <int OWN>
__global__ void __launch_bounds__(256) hh_qr_flag_kernel(double* __restrict__ X, int64_t m, int64_t n,
                                                         int64_t nc, int64_t ld, double* __restrict__ tau,
                                                         unsigned int* __restrict__ flags,
                                                         unsigned int* status) {
    extern __shared__ double cols[];                      // OWN x m
    __shared__ double red[8 * (OWN + 1)];
    const int64_t G = gridDim.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int64_t jq[OWN];
#pragma unroll
    for (int q = 0; q < OWN; ++q) {
        jq[q] = blockIdx.x + q * G;
        if (jq[q] < nc)
            for (int64_t i = tid; i < m; i += blockDim.x) cols[q * m + i] = X[i + jq[q] * ld];
    }
    __syncthreads();
    // block sums of up to OWN values at once (fixed order)
    auto block_sums = [&](double (&v)[OWN], int cnt) {
#pragma unroll
        for (int q = 0; q < OWN; ++q) if (q < cnt) v[q] = warp_sum(v[q]);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < OWN; ++q) if (q < cnt) red[warp * OWN + q] = v[q];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < OWN; ++q)
            if (q < cnt) {
                double s = 0.0;
                for (int w = 0; w < 8; ++w) s += red[w * OWN + q];
                v[q] = s;
            }
        __syncthreads();
    };
    // applies reflector p (v from global memory, tau) to owned column q if it is >= p + 1
    auto reflector_norm_and_publish = [&](int q, int64_t t) {
        double* col = cols + q * m;
        double a[1];
        a[0] = 0.0;
        for (int64_t i = t + 1 + tid; i < m; i += blockDim.x) a[0] = fma(col[i], col[i], a[0]);
        double tmp[OWN];
#pragma unroll
        for (int r = 0; r < OWN; ++r) tmp[r] = (r == 0) ? a[0] : 0.0;
        block_sums(tmp, 1);
        const double xn2 = tmp[0];
        const double alpha = col[t];
        double tt = 0.0, beta = alpha;
        if (xn2 != 0.0) {
            beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
            const double scale = 1.0 / (alpha - beta);
            for (int64_t i = t + 1 + tid; i < m; i += blockDim.x) col[i] *= scale;
            tt = (beta - alpha) / beta;
        }
        __syncthreads();
        if (tid == 0) { col[t] = beta; tau[t] = tt; }
        __syncthreads();
        for (int64_t i = t + tid; i < m; i += blockDim.x) X[i + t * ld] = col[i];
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            atomicExch(&flags[t], 1u);
        }
    };
    // owner of column 0 starts the chain
    if (blockIdx.x == 0 && n > 0) reflector_norm_and_publish(0, 0);
    for (int64_t p = 0; p < n; ++p) {
        if (!wait_flag(&flags[p], status)) return;
        const double tp = tau[p];
        const int64_t t = p + 1;                           // the next reflector's column
        if (tp != 0.0) {
            const double* v = X + p * ld;
            // the owner of column t updates it first (look-ahead)
            int first = -1;
#pragma unroll
            for (int q = 0; q < OWN; ++q) if (jq[q] == t && t < n) first = q;
            for (int pass = 0; pass < 2; ++pass) {
                double dot[OWN];
                int sel[OWN];
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < OWN; ++q) {
                    const bool mine = jq[q] < nc && jq[q] > p;
                    const bool in_pass = (pass == 0) ? (q == first) : (q != first);
                    if (mine && in_pass) sel[cnt++] = q;
                }
                for (int c = cnt; c < OWN; ++c) sel[c] = -1;
                if (cnt == 0) continue;
#pragma unroll
                for (int c = 0; c < OWN; ++c) dot[c] = 0.0;
                for (int64_t i = p + 1 + tid; i < m; i += blockDim.x) {
                    const double vi = v[i];
#pragma unroll
                    for (int c = 0; c < OWN; ++c)
                        if (c < cnt) dot[c] = fma(vi, cols[sel[c] * m + i], dot[c]);
                }
                block_sums(dot, cnt);
#pragma unroll
                for (int c = 0; c < OWN; ++c) {
                    if (c >= cnt) break;
                    double* col = cols + sel[c] * m;
                    const double f = tp * (dot[c] + col[p]);
                    for (int64_t i = p + 1 + tid; i < m; i += blockDim.x) col[i] = fma(-f, v[i], col[i]);
                    __syncthreads();
                    if (tid == 0) col[p] -= f;
                    __syncthreads();
                }
                if (pass == 0 && first >= 0) reflector_norm_and_publish(first, t);
            }
        } else if (t < n) {
#pragma unroll
            for (int q = 0; q < OWN; ++q)
                if (jq[q] == t) reflector_norm_and_publish(q, t);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < OWN; ++q)
        if (jq[q] < nc)
            for (int64_t i = tid; i < m; i += blockDim.x) X[i + jq[q] * ld] = cols[q * m + i];
}

void householder_qr(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld, double* tau) {
    if (n <= 0) return;
    if (m < n) fail(RNLA_ERR_INVALID_DIMENSIONS, "householder_qr needs m >= n");
    {
        // flag-pipelined kernel when the owned columns fit in shared memory
        int64_t G = 2LL * ctx.sm_count;
        if (G > nc) G = nc;
        const int own = (int)((nc + G - 1) / G);
        const size_t smem = (size_t)own * m * sizeof(double);
        if (n >= 8 && own <= 4 && smem <= 200 * 1024) {
            const void* k = own == 1 ? (const void*)hh_qr_flag_kernel<1>
                          : own == 2 ? (const void*)hh_qr_flag_kernel<2>
                          : own == 3 ? (const void*)hh_qr_flag_kernel<3>
                                     : (const void*)hh_qr_flag_kernel<4>;
            set_smem_limit((const void*)k, smem);
            int nb = 0;
            RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 256, smem));
            if ((int64_t)nb * ctx.sm_count >= G) {
                DevBuf<unsigned int> flags(n, ctx.stream);
                RNLA_CUDA(cudaMemsetAsync(flags.get(), 0, n * sizeof(unsigned int), ctx.stream));
                RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
                unsigned int* fl = flags.get();
                unsigned int* st = ctx.status;
                void* args[] = {&X, &m, &n, &nc, &ld, &tau, &fl, &st};
                RNLA_CUDA(cudaLaunchCooperativeKernel(k, dim3((unsigned)G), dim3(256), args, smem, ctx.stream));
                count_launch();
                ctx.check_status("householder_qr");
                return;
            }
        }
    }
    {
        int nb = 0;
        RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, hh_qr_coop_kernel, 256, 0));
        int64_t G = (int64_t)(nb < 2 ? nb : 2) * ctx.sm_count;
        if (G > nc) G = nc;
        if (nb >= 1 && n >= 32 && (nc + G - 1) / G <= QR_OWN) {
            DevBuf<unsigned int> bw(2, ctx.stream);
            RNLA_CUDA(cudaMemsetAsync(bw.get(), 0, 2 * sizeof(unsigned int), ctx.stream));
            RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
            GridBarrier bar{bw.get(), bw.get() + 1, ctx.status};
            void* args[] = {&X, &m, &n, &nc, &ld, &tau, &bar};
            RNLA_CUDA(cudaLaunchCooperativeKernel((const void*)hh_qr_coop_kernel, dim3((unsigned)G), dim3(256),
                                                  args, 0, ctx.stream));
            count_launch();
            ctx.check_status("householder_qr");
            return;
        }
    }
    for (int64_t t = 0; t <= n; ++t) {
        const int64_t jfirst = (t < n) ? t : n;
        const int64_t cnt = nc - jfirst;
        if (cnt <= 0) break;
        hh_step_kernel<<<(unsigned)cnt, 256, 0, ctx.stream>>>(X, m, n, ld, t, jfirst, tau);
        RNLA_LAUNCH_CHECK();
    }
}

// Applies reflector t (stored in V) to columns j >= t of Q.
__global__ void __launch_bounds__(256) hh_apply_kernel(const double* __restrict__ V, int64_t ldv,
                                                       const double* __restrict__ tau, int64_t m,
                                                       int64_t t, double* __restrict__ Q, int64_t ldq) {
    __shared__ double red[8];
    const double tp = tau[t];
    if (tp == 0.0) return;
    const int64_t j = t + blockIdx.x;
    double* q = Q + j * ldq;
    const double* v = V + t * ldv;
    double s = 0.0;
    for (int64_t i = t + 1 + threadIdx.x; i < m; i += blockDim.x) s = fma(v[i], q[i], s);
    s = block_sum(s, red) + q[t];
    const double f = tp * s;
    if (threadIdx.x == 0) q[t] -= f;
    for (int64_t i = t + 1 + threadIdx.x; i < m; i += blockDim.x) q[i] = fma(-f, v[i], q[i]);
}

void householder_form_q(Ctx& ctx, const double* V, int64_t m, int64_t n, int64_t ldv,
                        const double* tau, double* Q, int64_t ldq) {
    fill_identity(ctx, m, n, Q, ldq);
    for (int64_t t = n - 1; t >= 0; --t) {
        hh_apply_kernel<<<(unsigned)(n - t), 256, 0, ctx.stream>>>(V, ldv, tau, m, t, Q, ldq);
        RNLA_LAUNCH_CHECK();
    }
}

// ---------------------------------------------------------------------------
// Triangular inverse and solves (column-oriented back substitution)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) upper_inverse_kernel(const double* __restrict__ R, int64_t n,
                                                            int64_t ldr, double* __restrict__ Ri,
                                                            int64_t ldi, unsigned int* status) {
    extern __shared__ double b[];
    const int64_t j = blockIdx.x;
    for (int64_t i = threadIdx.x; i <= j; i += blockDim.x) b[i] = (i == j) ? 1.0 : 0.0;
    __shared__ double xi_s;
    __syncthreads();
    for (int64_t i = j; i >= 0; --i) {
        if (threadIdx.x == 0) {
            const double d = R[i + i * ldr];
            if (d == 0.0) atomicCAS(status, 0u, (unsigned int)KSTATUS_SINGULAR);
            xi_s = b[i] / d;
            b[i] = xi_s;
        }
        __syncthreads();
        const double xi = xi_s;
        const double* rc = R + i * ldr;
        for (int64_t r = threadIdx.x; r < i; r += blockDim.x) b[r] = fma(-xi, rc[r], b[r]);
        __syncthreads();
    }
    double* out = Ri + j * ldi;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) out[i] = (i <= j) ? b[i] : 0.0;
}

bool upper_inverse(Ctx& ctx, const double* R, int64_t n, int64_t ldr, double* Rinv, int64_t ldi) {
    if (n <= 0) return true;
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    const size_t smem = (size_t)n * sizeof(double);
    if (smem > 48 * 1024)
        set_smem_limit((const void*)upper_inverse_kernel, smem);
    upper_inverse_kernel<<<(unsigned)n, 256, smem, ctx.stream>>>(R, n, ldr, Rinv, ldi, ctx.status);
    RNLA_LAUNCH_CHECK();
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, ctx.status, sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    return h == 0;
}

// solvers.rs:22-41: x_i = (y_i - sum_{j>i} u_ij x_j) / u_ii, skipped (x_i = 0) when u_ii == 0.
__global__ void __launch_bounds__(256) upper_solve_skip_kernel(const double* __restrict__ U, int64_t n,
                                                               int64_t ldu, const double* __restrict__ y,
                                                               double* __restrict__ x) {
    extern __shared__ double b[];
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) b[i] = y[i];
    __shared__ double xi_s;
    __syncthreads();
    for (int64_t i = n - 1; i >= 0; --i) {
        if (threadIdx.x == 0) {
            const double d = U[i + i * ldu];
            xi_s = (d != 0.0) ? b[i] / d : 0.0;
            b[i] = xi_s;
        }
        __syncthreads();
        const double xi = xi_s;
        if (xi != 0.0) {
            const double* uc = U + i * ldu;
            for (int64_t r = threadIdx.x; r < i; r += blockDim.x) b[r] = fma(-xi, uc[r], b[r]);
        }
        __syncthreads();
    }
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
}

void upper_solve_skip_zero(Ctx& ctx, const double* U, int64_t n, int64_t ldu, const double* y,
                           double* x) {
    if (n <= 0) return;
    const size_t smem = (size_t)n * sizeof(double);
    if (smem > 48 * 1024)
        set_smem_limit((const void*)upper_solve_skip_kernel, smem);
    upper_solve_skip_kernel<<<1, 256, smem, ctx.stream>>>(U, n, ldu, y, x);
    RNLA_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// Cholesky (right-looking, one CTA): G = R^T R, R upper, written in place.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) cholesky_kernel(double* __restrict__ G, int64_t n, int64_t ld,
                                                        unsigned int* status) {
    __shared__ double rkk_s;
    __shared__ int bad_s;
    if (threadIdx.x == 0) bad_s = 0;
    for (int64_t k = 0; k < n; ++k) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const double d = G[k + k * ld];
            if (!(d > 0.0)) {
                bad_s = 1;
                atomicCAS(status, 0u, (unsigned int)KSTATUS_NOT_PD);
            }
            rkk_s = sqrt(d);
            G[k + k * ld] = rkk_s;
        }
        __syncthreads();
        if (bad_s) return;
        const double rkk = rkk_s;
        for (int64_t j = k + 1 + threadIdx.x; j < n; j += blockDim.x) G[k + j * ld] /= rkk;
        __syncthreads();
        // trailing update of the upper triangle: G[i][j] -= R[k][i] R[k][j], k < i <= j
        const int64_t w = n - k - 1;
        const int64_t tot = w * w;
        for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
            const int64_t ii = k + 1 + e % w, jj = k + 1 + e / w;
            if (ii <= jj) G[ii + jj * ld] = fma(-G[k + ii * ld], G[k + jj * ld], G[ii + jj * ld]);
        }
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int64_t i = e % n, j = e / n;
        if (i > j) G[i + j * ld] = 0.0;
    }
}

// Blocked right-looking Cholesky G = R^T R over a cooperative grid (upper
// triangle read, R written over it, strict lower triangle zeroed).  Panels
// of CHB = 32 rows; CTA c owns the columns j = c, c + G, ...  Per panel K:
//   (1) every CTA loads the panel's diagonal block and factors it in shared
//       memory (warp 0; the other warps wait): redundant work, but no grid
//       barrier between the diagonal block and its use;
//   (2) each CTA forms the panel rows R[K][j] = R_KK^-T G[K][j] of its own
//       trailing columns (one warp per column, forward substitution with
//       the pivots' reciprocals); CTA 0 writes R_KK;
//   grid barrier (the panel rows of every column are now in G);
//   (3) each CTA subtracts R[K][i]^T R[K][j] from its own columns j, rows
//       k1 <= i <= j, with 64-row chunks of the panel rows staged in shared
//       memory;
//   grid barrier.
// Two barriers per 32 columns instead of one per column.  Columns at or
// beyond npd (npd = n or n - 1) need no positive pivot: a bordered Gram
// [X c]^T [X c] gives R of X and, in column n - 1, R^-T X^T c and the
// residual norm sqrt(max(0, .)).  Every CTA factors the same diagonal block
// from the same data, so a non-positive pivot ends all of them at the same
// panel.
constexpr int CHB = 32;
constexpr int CH_THREADS = 256;
constexpr int CH_MAXQ = 32;                 // owned columns per CTA: n <= CH_MAXQ x grid

__global__ void __launch_bounds__(CH_THREADS) cholesky_blocked_kernel(double* __restrict__ G, int64_t n, int64_t npd,
                                                                      int64_t ld, unsigned int* status,
                                                                      GridBarrier bar) {
    __shared__ double Ds[CHB][CHB + 1];           // diagonal block, R_KK after step (1)
    __shared__ double ris[CHB];                   // 1 / R[t][t]
    __shared__ double Ps[CHB][64 + 1];            // panel rows of a 64-row chunk
    __shared__ double Rjs[CH_MAXQ][CHB];          // panel rows of the owned trailing columns
    __shared__ int bad_s;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Gc = gridDim.x, c = blockIdx.x;
    for (int64_t k0 = 0; k0 < npd; k0 += CHB) {
        const int kb = (int)(npd - k0 < CHB ? npd - k0 : CHB);
        const int64_t k1 = k0 + kb;
        // (1) diagonal block
        for (int e = tid; e < CHB * CHB; e += CH_THREADS) {
            const int i = e % CHB, j = e / CHB;
            Ds[i][j] = (i <= j && j < kb) ? G[(k0 + i) + (k0 + j) * ld] : 0.0;
        }
        if (tid == 0) bad_s = 0;
        __syncthreads();
        if (warp == 0) {
            // lane c holds column c of the block in registers; step t scales
            // row t by 1 / sqrt(pivot) and subtracts R[t][i] R[t][c] from rows
            // t < i <= c, R[t][i] arriving from lane i by shuffle
            double col[CHB];
#pragma unroll
            for (int i = 0; i < CHB; ++i) col[i] = Ds[i][lane];
            bool bad = false;
#pragma unroll
            for (int t = 0; t < CHB; ++t) {
                if (t < kb && !bad) {
                    const double d = __shfl_sync(0xffffffffu, col[t], t);
                    if (!(d > 0.0)) {
                        bad = true;
                    } else {
                        const double ri = rsqrt(d);
                        const double rt = col[t] * ri;               // R[t][lane] (R[t][t] = d ri)
                        col[t] = rt;
                        if (lane == 0) ris[t] = ri;
#pragma unroll
                        for (int i = t + 1; i < CHB; ++i) {
                            const double rti = __shfl_sync(0xffffffffu, rt, i);
                            if (i <= lane) col[i] = fma(-rti, rt, col[i]);
                        }
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < CHB; ++i) Ds[i][lane] = col[i];
            if (bad && lane == 0) bad_s = 1;
        }
        __syncthreads();
        if (bad_s) {
            if (tid == 0) atomicCAS(status, 0u, (unsigned int)KSTATUS_NOT_PD);
            return;
        }
        // (2) panel rows of the owned trailing columns: R_KK^T x = g
        {
            int64_t j = k1 + ((c - k1 % Gc) % Gc + Gc) % Gc;        // first owned column >= k1
            j += (int64_t)warp * Gc;
            for (; j < n; j += (int64_t)(CH_THREADS / 32) * Gc) {
                double g = lane < kb ? G[(k0 + lane) + j * ld] : 0.0;
                for (int s = 0; s < kb; ++s) {
                    const double xs = __shfl_sync(0xffffffffu, g, s) * ris[s];
                    if (lane == s) g = xs;
                    else if (lane > s && lane < kb) g = fma(-Ds[s][lane], xs, g);
                }
                if (lane < kb) G[(k0 + lane) + j * ld] = g;
            }
        }
        if (!grid_sync(bar)) return;
        // every CTA has read the diagonal block: R_KK replaces it
        if (c == 0)
            for (int e = tid; e < kb * kb; e += CH_THREADS) {
                const int i = e % kb, j = e / kb;
                if (i <= j) G[(k0 + i) + (k0 + j) * ld] = Ds[i][j];
            }
        // (3) trailing update of the owned columns q = 0, 1, ... (j = jfirst + q Gc),
        // their panel rows staged in shared memory
        const int64_t jfirst = k1 + ((c - k1 % Gc) % Gc + Gc) % Gc;
        if (jfirst < n) {
            const int nq = (int)((n - 1 - jfirst) / Gc) + 1;
            const int64_t jlast = jfirst + (int64_t)(nq - 1) * Gc;
            for (int e = tid; e < nq * CHB; e += CH_THREADS) {
                const int q = e / CHB, t = e % CHB;
                Rjs[q][t] = t < kb ? G[(k0 + t) + (jfirst + (int64_t)q * Gc) * ld] : 0.0;
            }
            const int r = tid & 63, cg = tid >> 6;          // row within the chunk, column group
            for (int64_t i0 = k1; i0 <= jlast; i0 += 64) {
                __syncthreads();
                for (int e = tid; e < CHB * 64; e += CH_THREADS) {
                    const int t = e % CHB, rr = e / CHB;
                    Ps[t][rr] = (t < kb && i0 + rr < n) ? G[(k0 + t) + (i0 + rr) * ld] : 0.0;
                }
                __syncthreads();
                const int64_t i = i0 + r;
                // owned columns j >= i0, handed to the four column groups in turn
                const int q0 = i0 > jfirst ? (int)((i0 - jfirst + Gc - 1) / Gc) : 0;
                for (int q = q0 + cg; q < nq; q += 4) {
                    const int64_t j = jfirst + (int64_t)q * Gc;
                    if (i > j) continue;
                    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;     // four independent chains
#pragma unroll
                    for (int t = 0; t < CHB; t += 4) {
                        a0 = fma(Ps[t][r], Rjs[q][t], a0);
                        a1 = fma(Ps[t + 1][r], Rjs[q][t + 1], a1);
                        a2 = fma(Ps[t + 2][r], Rjs[q][t + 2], a2);
                        a3 = fma(Ps[t + 3][r], Rjs[q][t + 3], a3);
                    }
                    G[i + j * ld] -= (a0 + a1) + (a2 + a3);
                }
            }
        }
        if (!grid_sync(bar)) return;
    }
    // trailing columns beyond npd: the residual norm on the diagonal
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = gt; e < n * n; e += gs) {
        const int64_t i = e % n, j = e / n;
        if (i > j) G[i + j * ld] = 0.0;
        else if (i == j && i >= npd) G[i + j * ld] = sqrt(fmax(G[i + j * ld], 0.0));
    }
}

bool cholesky_upper(Ctx& ctx, double* G, int64_t n, int64_t ld, int64_t npd) {
    if (npd < 0) npd = n;
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    if (n >= 128 || npd < n) {
        int nb = 0;
        RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, cholesky_blocked_kernel, CH_THREADS, 0));
        int Gs = ctx.sm_count;
        if (Gs > nb * ctx.sm_count) Gs = nb * ctx.sm_count;
        if (Gs > n) Gs = (int)n;
        if (Gs < 1) Gs = 1;
        if (n > (int64_t)CH_MAXQ * Gs) fail(RNLA_ERR_INVALID_DIMENSIONS, "Cholesky: n above the blocked kernel's limit");
        DevBuf<unsigned int> bw(2, ctx.stream);
        RNLA_CUDA(cudaMemsetAsync(bw.get(), 0, 2 * sizeof(unsigned int), ctx.stream));
        GridBarrier bar{bw.get(), bw.get() + 1, ctx.status};
        void* args[] = {&G, &n, &npd, &ld, &ctx.status, &bar};
        RNLA_CUDA(cudaLaunchCooperativeKernel((const void*)cholesky_blocked_kernel, dim3((unsigned)Gs),
                                              dim3(CH_THREADS), args, 0, ctx.stream));
        count_launch();
    } else {
        cholesky_kernel<<<1, 1024, 0, ctx.stream>>>(G, n, ld, ctx.status);
        RNLA_LAUNCH_CHECK();
    }
    unsigned int h = 0;
    RNLA_CUDA(cudaMemcpyAsync(&h, ctx.status, sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_CUDA(cudaMemsetAsync(ctx.status, 0, sizeof(unsigned int), ctx.stream));
    if (h == KSTATUS_NOT_PD) return false;
    if (h != KSTATUS_OK) throw Error(RNLA_ERR_TIMEOUT, "Cholesky: a grid barrier exceeded its limit");
    return true;
}

// ---------------------------------------------------------------------------
// Orthonormal basis: CholeskyQR2, Householder fallback
// ---------------------------------------------------------------------------
static void householder_orth_inplace(Ctx& ctx, double* Y, int64_t m, int64_t n, int64_t ld) {
    DevBuf<double> tau(n, ctx.stream), Q((size_t)m * n, ctx.stream);
    householder_qr(ctx, Y, m, n, n, ld, tau);
    householder_form_q(ctx, Y, m, n, ld, tau, Q, m);
    copy_matrix(ctx, m, n, Q, m, Y, ld);
}

int orthonormalize(Ctx& ctx, double* Y, int64_t m, int64_t n, int64_t ld, bool force_householder) {
    if (m <= 0 || n <= 0) return 0;
    if (force_householder || m < n) {
        householder_orth_inplace(ctx, Y, m, n, ld);
        return 0;
    }
    DevBuf<double> G((size_t)n * n, ctx.stream), Ri((size_t)n * n, ctx.stream),
        T((size_t)m * n, ctx.stream);
    for (int pass = 0; pass < 2; ++pass) {
        gemm_f64(ctx, 'T', 'N', n, n, m, 1.0, Y, ld, Y, ld, 0.0, G, n);
        if (!cholesky_upper(ctx, G, n, n) || !upper_inverse(ctx, G, n, n, Ri, n)) {
            householder_orth_inplace(ctx, Y, m, n, ld);
            return 1;
        }
        gemm_f64(ctx, 'N', 'N', m, n, n, 1.0, Y, ld, Ri, n, 0.0, T, m);
        copy_matrix(ctx, m, n, T, m, Y, ld);
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Complete-pivoting LU (one CTA), L only.  Arithmetic uses explicitly
// rounded operations (no contraction) so the pivot sequence is exactly that
// of a scalar restatement of the same algorithm.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) full_piv_lu_kernel(double* __restrict__ W, int64_t m, int64_t n,
                                                           int64_t ld) {
    __shared__ double bv[32];
    __shared__ long long bi[32];
    __shared__ long long piv_s;
    __shared__ double pval_s;
    const int64_t p = m < n ? m : n;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t k = 0; k < p; ++k) {
        const int64_t rows = m - k, cols = n - k, tot = rows * cols;
        double best = -1.0;
        long long bidx = 0x7fffffffffffffffLL;
        for (int64_t e = threadIdx.x; e < tot; e += blockDim.x) {
            const int64_t i = k + e % rows, j = k + e / rows;
            const double a = fabs(W[i + j * ld]);
            if (a > best) { best = a; bidx = e; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, best, o);
            const long long oi = __shfl_xor_sync(0xffffffffu, bidx, o);
            if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
        }
        if (lane == 0) { bv[wid] = best; bi[wid] = bidx; }
        __syncthreads();
        if (wid == 0) {
            best = lane < nw ? bv[lane] : -1.0;
            bidx = lane < nw ? bi[lane] : 0x7fffffffffffffffLL;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, best, o);
                const long long oi = __shfl_xor_sync(0xffffffffu, bidx, o);
                if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
            }
            if (lane == 0) { piv_s = bidx; pval_s = best; }
        }
        __syncthreads();
        if (pval_s == 0.0) break;   // remaining block is zero: L keeps identity columns
        const int64_t r = k + piv_s % rows, c = k + piv_s / rows;
        if (r != k)
            for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
                const double t = W[k + j * ld];
                W[k + j * ld] = W[r + j * ld];
                W[r + j * ld] = t;
            }
        __syncthreads();   // the column swap below touches rows k and r too
        if (c != k)
            for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
                const double t = W[i + k * ld];
                W[i + k * ld] = W[i + c * ld];
                W[i + c * ld] = t;
            }
        __syncthreads();
        const double pv = W[k + k * ld];
        for (int64_t i = k + 1 + threadIdx.x; i < m; i += blockDim.x)
            W[i + k * ld] = __ddiv_rn(W[i + k * ld], pv);
        __syncthreads();
        const int64_t tr = m - k - 1, tc = n - k - 1;
        for (int64_t e = threadIdx.x; e < tr * tc; e += blockDim.x) {
            const int64_t i = k + 1 + e % tr, j = k + 1 + e / tr;
            W[i + j * ld] = __dsub_rn(W[i + j * ld], __dmul_rn(W[i + k * ld], W[k + j * ld]));
        }
        __syncthreads();
    }
}

__global__ void extract_unit_lower_kernel(const double* __restrict__ W, int64_t m, int64_t p,
                                          int64_t ldw, double* __restrict__ L, int64_t ldl) {
    const int64_t tot = m * p;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % m, c = e / m;
        L[i + c * ldl] = (i > c) ? W[i + c * ldw] : (i == c ? 1.0 : 0.0);
    }
}

void full_piv_lu_l(Ctx& ctx, const double* X, int64_t m, int64_t n, int64_t ldx, double* L,
                   int64_t ldl) {
    if (m <= 0 || n <= 0) return;
    DevBuf<double> W((size_t)m * n, ctx.stream);
    copy_matrix(ctx, m, n, X, ldx, W, m);
    full_piv_lu_kernel<<<1, 1024, 0, ctx.stream>>>(W, m, n, m);
    RNLA_LAUNCH_CHECK();
    const int64_t p = m < n ? m : n;
    int g = div_up(m * p, 256);
    if (g > 4096) g = 4096;
    extract_unit_lower_kernel<<<g, 256, 0, ctx.stream>>>(W, m, p, m, L, ldl);
    RNLA_LAUNCH_CHECK();
}

// ---------------------------------------------------------------------------
// One-sided (Hestenes) Jacobi on a small s x s matrix W, rotations
// accumulated into V.  One CTA; each warp takes pairs of a round-robin
// tournament round, so the pairs of a round touch disjoint columns.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) jacobi_kernel(double* __restrict__ W, double* __restrict__ V,
                                                      int s, int max_sweeps) {
    __shared__ int rot_s;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int sp = (s + 1) & ~1;     // players, padded to even (a bye when s is odd)
    const double tol = 1e-15;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) rot_s = 0;
        __syncthreads();
        for (int round = 0; round < sp - 1; ++round) {
            for (int pr = wid; pr < sp / 2; pr += nw) {
                // circle method: player 0 fixed, the others rotate
                int a, b;
                if (pr == 0) { a = 0; b = 1 + (round % (sp - 1)); }
                else {
                    a = 1 + ((round + pr) % (sp - 1));
                    b = 1 + ((round + sp - 1 - pr) % (sp - 1));
                }
                if (a >= s || b >= s) continue;
                if (a > b) { const int t = a; a = b; b = t; }
                double* wa = W + (int64_t)a * s;
                double* wb = W + (int64_t)b * s;
                double al = 0.0, be = 0.0, ga = 0.0;
                for (int i = lane; i < s; i += 32) {
                    const double x = wa[i], y = wb[i];
                    al = fma(x, x, al);
                    be = fma(y, y, be);
                    ga = fma(x, y, ga);
                }
                al = warp_sum(al); be = warp_sum(be); ga = warp_sum(ga);
                if (ga == 0.0 || fabs(ga) <= tol * sqrt(al * be)) continue;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
                const double c = 1.0 / sqrt(fma(t, t, 1.0));
                const double sn = c * t;
                for (int i = lane; i < s; i += 32) {
                    const double x = wa[i], y = wb[i];
                    wa[i] = c * x - sn * y;
                    wb[i] = sn * x + c * y;
                }
                double* va = V + (int64_t)a * s;
                double* vb = V + (int64_t)b * s;
                for (int i = lane; i < s; i += 32) {
                    const double x = va[i], y = vb[i];
                    va[i] = c * x - sn * y;
                    vb[i] = sn * x + c * y;
                }
                if (lane == 0) atomicAdd(&rot_s, 1);
            }
            __syncthreads();
        }
        if (rot_s == 0) break;
        __syncthreads();
    }
}

// The same one-sided Jacobi spread over a cooperative grid: in each round
// of the circle-method tournament the s/2 disjoint column pairs go one per
// CTA (256 threads reduce the three dot products over the s rows and apply
// the rotation to W and V; short FP64 dependency chains per thread), and a
// bounded grid barrier separates rounds.  Same rotation formulae and
// tolerance as jacobi_kernel; a sweep without a rotation ends the iteration
// (all CTAs read the same counter).  (A warp per pair measured slower: the
// 64-cycle FP64 dependent latency over s / 32 rows per lane dominates.)
__global__ void __launch_bounds__(256) jacobi_coop_kernel(double* __restrict__ W, double* __restrict__ V, int s,
                                                          int max_sweeps, unsigned int* __restrict__ rot,
                                                          unsigned int* __restrict__ sweeps_out, GridBarrier bar) {
    __shared__ double red[3][8];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int sp = (s + 1) & ~1;
    // rotations stop at |gamma| <= s 2^-53 sqrt(alpha beta): below that, gamma is
    // the rounding of its own s-term dot product
    const double tol = fmax(1e-15, (double)s * 0x1p-53);
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        for (int round = 0; round < sp - 1; ++round) {
            for (int pr = blockIdx.x; pr < sp / 2; pr += gridDim.x) {
                int a, b;
                if (pr == 0) { a = 0; b = 1 + (round % (sp - 1)); }
                else {
                    a = 1 + ((round + pr) % (sp - 1));
                    b = 1 + ((round + sp - 1 - pr) % (sp - 1));
                }
                if (a >= s || b >= s) continue;          // the bye of an odd s (uniform over the CTA)
                if (a > b) { const int t = a; a = b; b = t; }
                double* wa = W + (int64_t)a * s;
                double* wb = W + (int64_t)b * s;
                double al = 0.0, be = 0.0, ga = 0.0;
                for (int i = tid; i < s; i += blockDim.x) {
                    const double x = wa[i], y = wb[i];
                    al = fma(x, x, al);
                    be = fma(y, y, be);
                    ga = fma(x, y, ga);
                }
                al = warp_sum(al); be = warp_sum(be); ga = warp_sum(ga);
                if (lane == 0) { red[0][wid] = al; red[1][wid] = be; red[2][wid] = ga; }
                __syncthreads();
                al = 0.0; be = 0.0; ga = 0.0;
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { al += red[0][w]; be += red[1][w]; ga += red[2][w]; }
                __syncthreads();
                if (ga == 0.0 || fabs(ga) <= tol * sqrt(al * be)) continue;
                const double zeta = (be - al) / (2.0 * ga);
                const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.0)));
                const double c = 1.0 / sqrt(fma(t, t, 1.0));
                const double sn = c * t;
                for (int i = tid; i < s; i += blockDim.x) {
                    const double x = wa[i], y = wb[i];
                    wa[i] = c * x - sn * y;
                    wb[i] = sn * x + c * y;
                }
                if (V) {
                    double* va = V + (int64_t)a * s;
                    double* vb = V + (int64_t)b * s;
                    for (int i = tid; i < s; i += blockDim.x) {
                        const double x = va[i], y = vb[i];
                        va[i] = c * x - sn * y;
                        vb[i] = sn * x + c * y;
                    }
                }
                if (tid == 0) atomicAdd(&rot[sweep & 1], 1u);
            }
            if (!grid_sync(bar)) return;
        }
        // every CTA reads this sweep's count after the last round's barrier;
        // the other slot is cleared for the next sweep before anyone uses it
        const unsigned int n_rot = *((volatile unsigned int*)&rot[sweep & 1]);
        if (blockIdx.x == 0 && tid == 0) {
            rot[(sweep + 1) & 1] = 0u;
            if (sweeps_out) *sweeps_out = (unsigned int)(sweep + 1);
        }
        if (!grid_sync(bar)) return;
        if (n_rot == 0u) break;
    }
}

// sigma_i = ||W_i||, descending order; U_R = W_i / sigma_i (zero columns
// completed with the first coordinate vectors orthogonal to the others);
// V columns permuted alike.  One CTA.
__global__ void __launch_bounds__(256) jacobi_finish_kernel(const double* __restrict__ W,
                                                            const double* __restrict__ V, int s,
                                                            double* __restrict__ UR,
                                                            double* __restrict__ VS,
                                                            double* __restrict__ sigma, int* order) {
    __shared__ double red[8];
    extern __shared__ double nrm[];
    for (int c = 0; c < s; ++c) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < s; i += blockDim.x) acc = fma(W[i + (int64_t)c * s], W[i + (int64_t)c * s], acc);
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) nrm[c] = sqrt(acc);
    }
    __syncthreads();
    // stable descending rank
    for (int c = threadIdx.x; c < s; c += blockDim.x) {
        int rank = 0;
        for (int d = 0; d < s; ++d)
            if (nrm[d] > nrm[c] || (nrm[d] == nrm[c] && d < c)) ++rank;
        order[rank] = c;
    }
    __syncthreads();
    for (int r = 0; r < s; ++r) {
        const int c = order[r];
        const double sg = nrm[c];
        if (threadIdx.x == 0) sigma[r] = sg;
        for (int i = threadIdx.x; i < s; i += blockDim.x) {
            UR[i + (int64_t)r * s] = (sg > 0.0) ? W[i + (int64_t)c * s] / sg : 0.0;
            if (V) VS[i + (int64_t)r * s] = V[i + (int64_t)c * s];
        }
    }
    __syncthreads();
    // complete the zero-sigma columns of UR with coordinate vectors
    int cand = 0;
    for (int r = 0; r < s; ++r) {
        if (nrm[order[r]] > 0.0) continue;
        while (cand < s) {
            // u = e_cand - sum_q (UR_q . e_cand) UR_q over the columns already set
            for (int i = threadIdx.x; i < s; i += blockDim.x) UR[i + (int64_t)r * s] = (i == cand) ? 1.0 : 0.0;
            __syncthreads();
            for (int q = 0; q < s; ++q) {
                if (q == r) continue;
                const bool set = (nrm[order[q]] > 0.0) || (q < r);
                if (!set) continue;
                double d = 0.0;
                for (int i = threadIdx.x; i < s; i += blockDim.x)
                    d = fma(UR[i + (int64_t)q * s], UR[i + (int64_t)r * s], d);
                d = block_sum(d, red);
                for (int i = threadIdx.x; i < s; i += blockDim.x)
                    UR[i + (int64_t)r * s] = fma(-d, UR[i + (int64_t)q * s], UR[i + (int64_t)r * s]);
                __syncthreads();
            }
            double nn = 0.0;
            for (int i = threadIdx.x; i < s; i += blockDim.x)
                nn = fma(UR[i + (int64_t)r * s], UR[i + (int64_t)r * s], nn);
            nn = sqrt(block_sum(nn, red));
            ++cand;
            if (nn > 0.5) {
                for (int i = threadIdx.x; i < s; i += blockDim.x) UR[i + (int64_t)r * s] /= nn;
                __syncthreads();
                break;
            }
        }
    }
}

__global__ void triu_copy_kernel(const double* __restrict__ src, int64_t lds, int64_t s,
                                 double* __restrict__ dst) {
    const int64_t tot = s * s;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % s, j = e / s;
        dst[e] = (i <= j) ? src[i + j * lds] : 0.0;
    }
}

// One-sided Jacobi of W (s x s) with the rotations accumulated into V (V may
// be null from s = 64 on): one CTA for small s, the cooperative grid version
// from s = 64 on.
void jacobi_sweeps(Ctx& ctx, double* W, double* V, int64_t s, unsigned int* sweeps_dev) {
    if (s < 64) {
        if (!V) fail(RNLA_ERR_COMPUTATION, "single-CTA Jacobi needs V");
        jacobi_kernel<<<1, 1024, 0, ctx.stream>>>(W, V, (int)s, 60);
        RNLA_LAUNCH_CHECK();
        return;
    }
    int nb = 0;
    RNLA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, jacobi_coop_kernel, 256, 0));
    int G = (int)((s + 1) / 2);                      // a CTA per column pair
    if (G > nb * ctx.sm_count) G = nb * ctx.sm_count;
    if (G > ctx.sm_count) G = ctx.sm_count;
    DevBuf<unsigned int> words(4, ctx.stream);       // rotation counts [2], barrier count, generation
    RNLA_CUDA(cudaMemsetAsync(words.get(), 0, 4 * sizeof(unsigned int), ctx.stream));
    ctx.clear_status();
    GridBarrier bar{words.get() + 2, words.get() + 3, ctx.status};
    int si = (int)s, sweeps = 60;
    unsigned int* rot = words.get();
    void* args[] = {&W, &V, &si, &sweeps, &rot, &sweeps_dev, &bar};
    RNLA_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_coop_kernel, dim3((unsigned)G), dim3(256), args, 0,
                                          ctx.stream));
    count_launch();
    ctx.check_status("Jacobi SVD");
}

// V[:, j] /= sigma_j (rows q, columns p)
__global__ void scale_columns_inv_kernel(int64_t q, int64_t p, double* __restrict__ V, int64_t ldv,
                                         const double* __restrict__ sigma) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < q * p; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % q, j = e / q;
        V[i + j * ldv] /= sigma[j];
    }
}
static void scale_columns_inv(Ctx& ctx, int64_t q, int64_t p, double* V, int64_t ldv, const double* sigma) {
    int g = div_up(q * p, 256);
    if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
    scale_columns_inv_kernel<<<g, 256, 0, ctx.stream>>>(q, p, V, ldv, sigma);
    RNLA_LAUNCH_CHECK();
}

// U_B = VS (eigenvectors of B B^T, descending sigma), sigma, V_B = B^T VS
// Sigma^-1 (float-float product); false -- nothing the caller keeps written
// -- when sigma_p / sigma_1 < 1e-5 (the Gram route loses the small ones)
static bool finish_gram_svd(Ctx& ctx, const double* B, int64_t p, int64_t q, int64_t ldb, const double* VS,
                            const double* sg, double* U, int64_t ldu, double* sigma, double* V, int64_t ldv) {
    double ext[2];
    RNLA_CUDA(cudaMemcpyAsync(&ext[0], sg, sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaMemcpyAsync(&ext[1], sg + p - 1, sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    if (!(ext[0] > 0.0) || !(ext[1] >= 1e-5 * ext[0])) return false;
    copy_matrix(ctx, p, p, VS, p, U, ldu);
    RNLA_CUDA(cudaMemcpyAsync(sigma, sg, p * sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    gram_ff(ctx, B, ldb, q, VS, p, p, p, V, ldv);
    scale_columns_inv(ctx, q, p, V, ldv, sg);
    return true;
}

// SVD of a wide B (p x q, p <= q) from R = chol(B B^T): the Gram is formed
// in float-float (gram_ff), R's right singular vectors (one-sided Jacobi on
// R) are B's left ones U_B, the column norms its singular values, and
// V_B = B^T U_B Sigma^-1 (float-float product).  Squaring B loses accuracy
// in the small singular values (relative error ~ 2^-48 (sigma_1 / sigma_i)^2),
// so this returns false -- and writes nothing the caller keeps -- when the
// Cholesky fails or sigma_p / sigma_1 < 1e-5; the caller then takes
// small_svd.  Synchronises once (to read the two extreme sigmas).
bool small_svd_gram(Ctx& ctx, const double* B, int64_t p, int64_t q, int64_t ldb, double* U, int64_t ldu,
                    double* sigma, double* V, int64_t ldv, int* sweeps) {
    if (p <= 0 || p > q) return false;
    DevBuf<double> Bt((size_t)q * p, ctx.stream), G((size_t)p * p, ctx.stream);
    transpose(ctx, p, q, B, ldb, Bt, q);
    gram_ff(ctx, Bt, q, p, Bt, q, p, q, G, p);                 // B B^T
    DevBuf<double> G0((size_t)p * p, ctx.stream);
    copy_matrix(ctx, p, p, G, p, G0, p);
    if (!cholesky_upper_ff(ctx, G, p, p)) return false;
    DevBuf<double> W((size_t)p * p, ctx.stream), UR((size_t)p * p, ctx.stream), sg(p, ctx.stream);
    DevBuf<double> VS((size_t)p * p, ctx.stream);
    DevBuf<int> order(p, ctx.stream);
    // FP32 cluster Jacobi + float-float Rayleigh-Ritz (eig_refine.cu), else
    // the FP64 grid Jacobi below
    if (eig_gram_refined(ctx, G0, G, p, VS, p, sg, sweeps)) return finish_gram_svd(ctx, B, p, q, ldb, VS, sg, U, ldu, sigma, V, ldv);
    int g = div_up(p * p, 256);
    if (g > 1024) g = 1024;
    // Jacobi on R^T (the rows of R): R^T V' = W' with orthogonal columns, so
    // B B^T = R^T R = (W' Sigma^-1) Sigma^2 (W' Sigma^-1)^T and U_B is W' with
    // normalised columns -- no rotation accumulation
    triu_copy_kernel<<<g, 256, 0, ctx.stream>>>(G, p, p, UR);
    RNLA_LAUNCH_CHECK();
    transpose(ctx, p, p, UR, p, W, p);
    DevBuf<double> VR;
    if (p < 64) {                                    // the single-CTA Jacobi accumulates V regardless
        VR.alloc((size_t)p * p, ctx.stream);
        fill_identity(ctx, p, p, VR, p);
    }
    DevBuf<unsigned int> nsw(1, ctx.stream);
    RNLA_CUDA(cudaMemsetAsync(nsw.get(), 0, sizeof(unsigned int), ctx.stream));
    jacobi_sweeps(ctx, W, p < 64 ? VR.get() : nullptr, p, nsw);
    const size_t smem = (size_t)p * sizeof(double);
    if (smem > 48 * 1024)
        set_smem_limit((const void*)jacobi_finish_kernel, smem);
    jacobi_finish_kernel<<<1, 256, smem, ctx.stream>>>(W, nullptr, (int)p, VS, nullptr, sg, order);
    RNLA_LAUNCH_CHECK();
    unsigned int hsw = 0;
    RNLA_CUDA(cudaMemcpyAsync(&hsw, nsw.get(), sizeof hsw, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    if (sweeps) *sweeps = (int)hsw;
    return finish_gram_svd(ctx, B, p, q, ldb, VS, sg, U, ldu, sigma, V, ldv);
}

void small_svd(Ctx& ctx, const double* B, int64_t p, int64_t q, int64_t ldb, double* U, int64_t ldu,
               double* sigma, double* V, int64_t ldv) {
    const int64_t s = p < q ? p : q;
    if (s <= 0) return;
    const bool wide = p <= q;
    const int64_t big = wide ? q : p;      // rows of G = B^T (wide) or B (tall)
    DevBuf<double> G((size_t)big * s, ctx.stream), tau(s, ctx.stream), QG((size_t)big * s, ctx.stream);
    if (wide) transpose(ctx, p, q, B, ldb, G, big);
    else copy_matrix(ctx, p, q, B, ldb, G, big);
    householder_qr(ctx, G, big, s, s, big, tau);
    householder_form_q(ctx, G, big, s, big, tau, QG, big);
    DevBuf<double> W((size_t)s * s, ctx.stream), VR((size_t)s * s, ctx.stream);
    int g = div_up(s * s, 256);
    if (g > 1024) g = 1024;
    triu_copy_kernel<<<g, 256, 0, ctx.stream>>>(G, big, s, W);
    RNLA_LAUNCH_CHECK();
    fill_identity(ctx, s, s, VR, s);
    // R VR = W with orthogonal columns -> R = UR diag(sigma) VR^T
    jacobi_sweeps(ctx, W, VR, s);
    DevBuf<double> UR((size_t)s * s, ctx.stream), VS((size_t)s * s, ctx.stream);
    DevBuf<int> order(s, ctx.stream);
    const size_t smem = (size_t)s * sizeof(double);
    if (smem > 48 * 1024)
        set_smem_limit((const void*)jacobi_finish_kernel, smem);
    jacobi_finish_kernel<<<1, 256, smem, ctx.stream>>>(W, VR, (int)s, UR, VS, sigma, order);
    RNLA_LAUNCH_CHECK();
    // G = QG R = (QG UR) diag(sigma) VS^T
    if (wide) {
        // B = G^T = VS diag(sigma) (QG UR)^T: U_B = VS (p x s), V_B = QG UR (q x s)
        copy_matrix(ctx, s, s, VS, s, U, ldu);
        gemm_f64(ctx, 'N', 'N', q, s, s, 1.0, QG, big, UR, s, 0.0, V, ldv);
    } else {
        gemm_f64(ctx, 'N', 'N', p, s, s, 1.0, QG, big, UR, s, 0.0, U, ldu);
        copy_matrix(ctx, s, s, VS, s, V, ldv);
    }
}

}  // namespace rnla
