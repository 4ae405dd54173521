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
#include <cooperative_groups.h>

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
    int R;              // rows per staged tile (power of two, <= 64)
};

template <typename TA>
__device__ __forceinline__ double ld_a(const TA* A, int64_t idx) { return (double)A[idx]; }

// y_i = sum_{j>=i} M_ij x_j (row i of M = column i of Mt); identity when M is null.
// Distributed over all warps of the grid.
__device__ void trmv_rows(const IterArgs& a, const double* __restrict__ xin, double scale,
                          double* __restrict__ yout) {
    const int64_t n = a.n;
    const int lane = threadIdx.x & 31;
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwg = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = gw; i < n; i += nwg) {
        double s;
        if (a.Mt) {
            const double* row = a.Mt + i * n;
            s = 0.0;
            for (int64_t j = i + lane; j < n; j += 32) s = fma(row[j], xin[j], s);
            s = warp_sum(s);
        } else {
            s = xin[i];
        }
        if (lane == 0) yout[i] = s * scale;
    }
}

// z_j = sum_{i<=j} M_ij g_i (column j of M); identity when M is null.  Each
// warp handles whole j's; returns through the callback-free path: writes
// f(z_j, j) via the lambda-like functor below.
template <typename F>
__device__ void trmv_cols(const IterArgs& a, const double* __restrict__ gin, F f) {
    const int64_t n = a.n;
    const int lane = threadIdx.x & 31;
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwg = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = gw; j < n; j += nwg) {
        double s;
        if (a.M) {
            const double* col = a.M + j * n;
            s = 0.0;
            for (int64_t i = lane; i <= j; i += 32) s = fma(col[i], gin[i], s);
            s = warp_sum(s);
        } else {
            s = gin[j];
        }
        f(s, j, lane);
    }
}

// Sum of per-CTA partial slot `slot` in a fixed order (identical in every CTA).
__device__ __forceinline__ double sum_partials(const double* sp, int slot) {
    __shared__ double v_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (unsigned c = 0; c < gridDim.x; ++c) s += ((volatile double*)sp)[c * 4 + slot];
        v_s = s;
    }
    __syncthreads();
    const double r = v_s;
    __syncthreads();
    return r;
}

// Block sum of a per-thread value, written by thread 0 to sp[cta*4 + slot].
__device__ __forceinline__ void write_partial(double v, double* sp, int slot, double* red) {
    v = block_sum(v, red);
    if (threadIdx.x == 0) sp[blockIdx.x * 4 + slot] = v;
}

// g_j = sum over CTAs of part[c][j]
__device__ void reduce_columns(const IterArgs& a) {
    const int64_t n = a.n;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
         j += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (unsigned c = 0; c < gridDim.x; ++c) s += a.part[(int64_t)c * n + j];
        a.g[j] = s;
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

template <typename TA, int NACC>
__global__ void __launch_bounds__(IT_THREADS) lsqr_kernel(IterArgs a) {
    extern __shared__ double smem[];
    double* red = smem + (size_t)a.n * (a.R + 1) + a.n + 64;
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
    row_pass<TA, NACC>(a, smem, a.x0 ? -1.0 : 0.0, 0.0, 1.0, a.u, true, true);
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
        row_pass<TA, NACC>(a, smem, 1.0, -alfa * us, 0.0, a.u, false, true);
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
template <typename TA, int NACC>
__global__ void __launch_bounds__(IT_THREADS) cgls_kernel(IterArgs a) {
    extern __shared__ double smem[];
    double* red = smem + (size_t)a.n * (a.R + 1) + a.n + 64;
    const int64_t n = a.n;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
    const double tol = a.abs_tol;

    for (int64_t j = gt; j < n; j += gthreads) a.x[j] = a.x0 ? a.x0[j] : 0.0;
    if (a.x0) trmv_rows(a, a.x0, 1.0, a.y);
    if (!grid_sync(a.bar)) return;
    // r = b - A M x ; partials of A^T r   (cg.rs:32-33)
    row_pass<TA, NACC>(a, smem, a.x0 ? -1.0 : 0.0, 0.0, 1.0, a.u, false, true);
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
        row_pass<TA, NACC>(a, smem, 1.0, 0.0, 0.0, a.ap, false, false);
        if (!grid_sync(a.bar)) return;
        const double apap = sum_partials(a.sp, 0);
        const double alpha = norm_s / apap;
        // x += alpha p ; r -= alpha ap fused with A^T r  (cg.rs:40-42)
        for (int64_t j = gt; j < n; j += gthreads) a.x[j] = fma(alpha, a.w[j], a.x[j]);
        {
            IterArgs b2 = a;
            b2.b = a.ap;   // reuse the "b" slot for ap: new_i = 1 * r_i - alpha * ap_i
            row_pass<TA, NACC>(b2, smem, 0.0, 1.0, -alpha, a.u, false, true);
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
        {
            const int lane = threadIdx.x & 31;
            const int64_t gw = gt >> 5, nwg = gthreads >> 5;
            for (int64_t r = gw; r < n; r += nwg) {
                double s;
                if (a.Mt) {
                    const double* row = a.Mt + r * n;
                    s = 0.0;
                    for (int64_t j = r + lane; j < n; j += 32) s = fma(row[j], a.vun[j], s);
                    s = warp_sum(s);
                } else {
                    s = a.vun[r];
                }
                if (lane == 0) a.y[r] = fma(beta, a.y[r], s);
            }
        }
        if (!grid_sync(a.bar)) return;
    }
    if (gt == 0) {
        a.out[0] = converged; a.out[1] = (double)it;
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

static size_t iter_smem(int64_t n, int R) {
    return ((size_t)n * (R + 1) + (size_t)n + 64 + IT_THREADS + 32) * sizeof(double);
}

struct IterBufs {
    DevBuf<double> u, v, vun, w, y, g, part, sp, ap, out, xbuf, Mt;
    DevBuf<unsigned int> bar;
};

template <typename K>
static int coop_grid(Ctx& ctx, K kernel, size_t smem) {
    if (smem > 48 * 1024)
        RNLA_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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

template <typename TA>
static void* lsqr_kernel_for(int64_t n) {
    const int nacc = (int)((n + IT_THREADS - 1) / IT_THREADS);
    if (nacc <= 1) return (void*)lsqr_kernel<TA, 1>;
    if (nacc <= 2) return (void*)lsqr_kernel<TA, 2>;
    if (nacc <= 4) return (void*)lsqr_kernel<TA, 4>;
    if (nacc <= 8) return (void*)lsqr_kernel<TA, 8>;
    return (void*)lsqr_kernel<TA, 16>;
}
template <typename TA>
static void* cgls_kernel_for(int64_t n) {
    const int nacc = (int)((n + IT_THREADS - 1) / IT_THREADS);
    if (nacc <= 1) return (void*)cgls_kernel<TA, 1>;
    if (nacc <= 2) return (void*)cgls_kernel<TA, 2>;
    if (nacc <= 4) return (void*)cgls_kernel<TA, 4>;
    if (nacc <= 8) return (void*)cgls_kernel<TA, 8>;
    return (void*)cgls_kernel<TA, 16>;
}

static void launch_coop(Ctx& ctx, void* kernel, int G, size_t smem, IterArgs& a) {
    void* params[] = {&a};
    RNLA_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(G), dim3(IT_THREADS), params, smem, ctx.stream));
    count_launch();
}

LsqrResult lsqr_solve(Ctx& ctx, const double* a64, const float* a32, int64_t m, int64_t n,
                      int64_t lda, const double* M, const double* b, const double* x0,
                      const LsqrParams& prm, double* x, double* var, double* arnorms_dev, bool ffp) {
    (void)ffp;
    if (n > (int64_t)IT_THREADS * IT_MAXACC)
        fail(RNLA_ERR_UNSUPPORTED, "lsqr: n > 4096 is not supported by the fused kernel");
    IterArgs a;
    IterBufs B;
    const int R = pick_R(n);
    const size_t smem = iter_smem(n, R);
    void* k = a32 ? lsqr_kernel_for<float>(n) : lsqr_kernel_for<double>(n);
    const int G = coop_grid(ctx, k, smem);
    setup(ctx, a, B, a32 ? (const void*)a32 : (const void*)a64, m, n, lda, M, G);
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
    const int R = pick_R(n);
    const size_t smem = iter_smem(n, R);
    void* k = a32 ? cgls_kernel_for<float>(n) : cgls_kernel_for<double>(n);
    const int G = coop_grid(ctx, k, smem);
    setup(ctx, a, B, a32 ? (const void*)a32 : (const void*)a64, m, n, lda, M, G);
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
