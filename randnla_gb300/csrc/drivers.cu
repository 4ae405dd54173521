// C entry points of the hot path: solvers.rs, cg.rs, lora_helpers.rs,
// lora_drivers.rs and sketch_and_precondition.rs, orchestrated on the GPU.
#include "rnla_abi.h"
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace rnla {

// Stage timer on the call's stream (device-timed).
struct StageTimer {
    cudaStream_t s;
    cudaEvent_t e[5];
    int n = 0;
    explicit StageTimer(cudaStream_t st) : s(st) {
        for (auto& x : e) RNLA_CUDA(cudaEventCreate(&x));
    }
    ~StageTimer() {
        for (auto& x : e) cudaEventDestroy(x);
    }
    void mark() {
        if (n < 5) RNLA_CUDA(cudaEventRecord(e[n++], s));
    }
    double ms(int a, int b) {
        if (b >= n) return 0.0;
        float t = 0.f;
        RNLA_CUDA(cudaEventSynchronize(e[b]));
        RNLA_CUDA(cudaEventElapsedTime(&t, e[a], e[b]));
        return t;
    }
};

// RNLA_PREC_BF16 is the tensor-core path with a single 8-bit digit per
// operand; any other value than the three precisions is an error.
static void resolve_precision(int32_t& prec, int32_t& digits_a, int32_t& digits_b) {
    if (prec == RNLA_PREC_BF16) {
        prec = RNLA_PREC_BF16X;
        digits_a = 1;
        digits_b = 1;
    } else if (prec != RNLA_PREC_FP64 && prec != RNLA_PREC_BF16X) {
        fail(RNLA_ERR_INVALID_PARAMETERS, "unknown precision");
    }
}

// The caller's options (or the defaults) with the precision resolved and
// the enumerations checked.
static rnla_options opts_or_default(const rnla_options* o) {
    rnla_options d;
    rnla_options_default(&d);
    if (o) d = *o;
    resolve_precision(d.precision, d.digits_a, d.digits_b);
    if (d.mode != RNLA_MODE_REFERENCE && d.mode != RNLA_MODE_RANDNLA)
        fail(RNLA_ERR_INVALID_PARAMETERS, "unknown rand_svd mode");
    if (d.inner_solver != RNLA_SOLVER_CGLS && d.inner_solver != RNLA_SOLVER_LSQR)
        fail(RNLA_ERR_INVALID_PARAMETERS, "unknown inner solver");
    return d;
}

static void check_mat(int64_t m, int64_t n, int64_t ld) {
    if (m < 0 || n < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "negative dimension");
    if (ld < (m > 0 ? m : 1)) fail(RNLA_ERR_INVALID_PARAMETERS, "leading dimension smaller than rows");
}

// ---------------------------------------------------------------------------
// Reference-mode range finder (lora_helpers.rs:17-105)
// ---------------------------------------------------------------------------
struct DMat {
    DevBuf<double> buf;
    int64_t rows = 0, cols = 0;
    double* p() const { return buf.get(); }
};

static void stabilize(Ctx& ctx, DMat& X) {
    const int64_t c = X.rows < X.cols ? X.rows : X.cols;
    DMat L;
    L.buf.alloc((size_t)X.rows * c, ctx.stream);
    L.rows = X.rows;
    L.cols = c;
    full_piv_lu_l(ctx, X.p(), X.rows, X.cols, X.rows, L.p(), X.rows);
    X = std::move(L);
}

// product with the zero S1 of lora_helpers.rs:63: exactly zero for finite A;
// with non-finite entries the FP64 GEMM reproduces the NaNs the reference gets.
static void times_zero(Ctx& ctx, const double* A, int64_t m, int64_t n, int64_t lda, int64_t k,
                       bool finite, DMat& out) {
    out.buf.alloc((size_t)m * k, ctx.stream);
    out.rows = m;
    out.cols = k;
    if (finite) {
        fill_zero(ctx, m, k, out.p(), m);
    } else {
        DevBuf<double> Z((size_t)n * k, ctx.stream);
        fill_zero(ctx, n, k, Z, n);
        gemm_f64(ctx, 'N', 'N', m, k, n, 1.0, A, lda, Z, n, 0.0, out.p(), m);
    }
}

static DMat tsog1_ref(Ctx& ctx, const double* A, int64_t m, int64_t n, int64_t lda, int64_t k,
                      int num_passes, int passes_per_stab, bool finite) {
    if (passes_per_stab == 0) fail(RNLA_ERR_INVALID_PARAMETERS, "passes_per_stab must be nonzero");
    int passes_done = 0;
    DMat S;                 // current S (lora_helpers.rs:67)
    bool s1_zero = true;    // S1 is the zero n x k matrix of line 63 unless replaced
    DMat S1;
    RngKey key0{GEN_PHILOX4X32, 0, 0};
    if (num_passes % 2 == 0) {
        S.buf.alloc((size_t)n * k, ctx.stream);
        S.rows = n;
        S.cols = k;
        sketch_fill_f64(ctx, DIST_GAUSSIAN, key0, n, k, S.p(), n);   // line 71
    } else {
        DMat G;
        G.buf.alloc((size_t)m * k, ctx.stream);
        G.rows = m;
        G.cols = k;
        sketch_fill_f64(ctx, DIST_GAUSSIAN, key0, m, k, G.p(), m);   // line 74
        S1.buf.alloc((size_t)n * k, ctx.stream);
        S1.rows = n;
        S1.cols = k;
        gemm_f64(ctx, 'T', 'N', n, k, m, 1.0, A, lda, G.p(), m, 0.0, S1.p(), n);   // line 76
        s1_zero = false;
        passes_done += 1;
        // line 78-81: the stabilised copy _S2 is never used
    }
    int diff = num_passes - passes_done;
    while (diff >= 2) {
        if (s1_zero) times_zero(ctx, A, m, n, lda, k, finite, S);      // line 89
        else {
            S.buf.alloc((size_t)m * S1.cols, ctx.stream);
            S.rows = m;
            S.cols = S1.cols;
            gemm_f64(ctx, 'N', 'N', m, S1.cols, n, 1.0, A, lda, S1.p(), n, 0.0, S.p(), m);
        }
        passes_done += 1;
        if (passes_done % passes_per_stab == 0) stabilize(ctx, S);      // line 93
        DMat T;
        T.buf.alloc((size_t)n * S.cols, ctx.stream);
        T.rows = n;
        T.cols = S.cols;
        gemm_f64(ctx, 'T', 'N', n, S.cols, m, 1.0, A, lda, S.p(), m, 0.0, T.p(), n);   // line 95
        S = std::move(T);
        passes_done += 1;
        if (passes_done % passes_per_stab == 0) stabilize(ctx, S);      // line 99
        diff -= 2;
    }
    return S;
}

static DMat orth_of(Ctx& ctx, const double* X, int64_t m, int64_t n, int64_t ldx) {
    // lora_helpers.rs:131-133: Householder QR, thin Q m x min(m,n)
    const int64_t c = m < n ? m : n;
    DMat Q;
    Q.rows = m;
    Q.cols = c;
    Q.buf.alloc((size_t)m * (c ? c : 1), ctx.stream);
    if (c == 0) return Q;
    DevBuf<double> W((size_t)m * n, ctx.stream), tau(c, ctx.stream);
    copy_matrix(ctx, m, n, X, ldx, W, m);
    // only the first c columns are factored (m < n: the trailing columns do not change Q)
    householder_qr(ctx, W, m, c, c, m, tau);
    householder_form_q(ctx, W, m, c, m, tau, Q.p(), m);
    return Q;
}

static DMat rf1_ref(Ctx& ctx, const double* A, int64_t m, int64_t n, int64_t lda, int64_t k,
                    bool finite) {
    DMat S = tsog1_ref(ctx, A, m, n, lda, k, 2, 1, finite);          // line 40
    DevBuf<double> Y((size_t)m * S.cols, ctx.stream);
    gemm_f64(ctx, 'N', 'N', m, S.cols, n, 1.0, A, lda, S.p(), S.rows, 0.0, Y, m);   // line 41
    return orth_of(ctx, Y, m, S.cols, m);                                            // line 42
}

// ---------------------------------------------------------------------------
// Symmetric eigenpairs and the eigenvalue drivers (lora_drivers.rs:84-213)
// ---------------------------------------------------------------------------
// lambda_i = sigma_i sign(u_i . v_i): for a symmetric matrix the SVD's
// left and right singular vectors agree up to the eigenvalue's sign
__global__ void eig_sign_kernel(const double* __restrict__ U, const double* __restrict__ V, int64_t p,
                                int64_t c, const double* __restrict__ sigma, double* __restrict__ lambda) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t j = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); j < c; j += nw) {
        double d = 0.0;
        for (int64_t i = lane; i < p; i += 32) d = fma(U[i + j * p], V[i + j * p], d);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == 0) lambda[j] = (d < 0.0) ? -sigma[j] : sigma[j];
    }
}

// count of A[i][j] != A[j][i] (exact comparison, as lora_drivers.rs:103)
__global__ void asym_count_kernel(const double* __restrict__ A, int64_t n, int64_t lda,
                                  unsigned long long* __restrict__ cnt) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % n, j = e / n;
        if (i < j && !(A[i + j * lda] == A[j + i * lda])) atomicAdd(cnt, 1ull);
    }
}

// y = y + nu x (n x c, same ld)
__global__ void axpy_mat_kernel(double* __restrict__ Y, const double* __restrict__ X, int64_t count, double nu) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
        Y[e] = fma(nu, X[e], Y[e]);
}

// symmetric eigenpairs of C (p x p): lambda ordered by decreasing |lambda|,
// eigenvectors the right singular vectors
static void sym_eig(Ctx& ctx, const double* C, int64_t p, double* lambda, double* W) {
    DevBuf<double> U((size_t)p * p, ctx.stream), sg(p, ctx.stream);
    small_svd(ctx, C, p, p, p, U, p, sg, W, p);
    eig_sign_kernel<<<(unsigned)div_up(p, 8), 256, 0, ctx.stream>>>(U, W, p, p, sg, lambda);
    RNLA_LAUNCH_CHECK();
}

static void rand_evd1_impl(Ctx& ctx, const double* A, int64_t n, int64_t lda, int64_t k, double eps, int64_t s,
                           double* v, int64_t ldv, double* lambda_host, int64_t* r_out) {
    if (k <= 0) fail(RNLA_ERR_INVALID_PARAMETERS, "Rank k must be positive");
    if (!(eps > 0.0)) fail(RNLA_ERR_INVALID_PARAMETERS, "Epsilon must be positive");
    if (s <= 0) fail(RNLA_ERR_INVALID_PARAMETERS, "Oversampling parameter s must be positive");
    {
        DevBuf<unsigned long long> cnt(1, ctx.stream);
        RNLA_CUDA(cudaMemsetAsync(cnt.get(), 0, sizeof(unsigned long long), ctx.stream));
        int g = (int)div_up(n * n, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        asym_count_kernel<<<g, 256, 0, ctx.stream>>>(A, n, lda, cnt);
        RNLA_LAUNCH_CHECK();
        unsigned long long h = 0;
        RNLA_CUDA(cudaMemcpyAsync(&h, cnt.get(), sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
        RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
        if (h) fail(RNLA_ERR_NOT_HERMITIAN, "Input matrix is not Hermitian");
    }
    const bool finite = all_finite(ctx, n, n, A, lda);
    DMat Q = rf1_ref(ctx, A, n, n, lda, k + s, finite);              // QB1: Q
    const int64_t c = Q.cols;
    DevBuf<double> B((size_t)c * n, ctx.stream), C((size_t)c * c, ctx.stream), W((size_t)c * c, ctx.stream),
        lam(c, ctx.stream);
    gemm_f64(ctx, 'T', 'N', c, n, n, 1.0, Q.p(), n, A, lda, 0.0, B, c);     // B = Q^T A
    gemm_f64(ctx, 'N', 'N', c, c, n, 1.0, B, c, Q.p(), n, 0.0, C, c);       // C = B Q
    sym_eig(ctx, C, c, lam, W);
    const int64_t r = k < c ? k : c;
    gemm_f64(ctx, 'N', 'N', n, r, c, 1.0, Q.p(), n, W, c, 0.0, v, ldv);      // V = Q U
    RNLA_CUDA(cudaMemcpyAsync(lambda_host, lam.get(), r * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    *r_out = r;
}

static double frob_norm(Ctx& ctx, const double* X, int64_t count) {
    DevBuf<double> out(1, ctx.stream);
    gemm_f64(ctx, 'T', 'N', 1, 1, count, 1.0, X, count, X, count, 0.0, out, 1);
    double h = 0.0;
    RNLA_CUDA(cudaMemcpyAsync(&h, out.get(), sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    return sqrt(h);
}

static void rand_evd2_impl(Ctx& ctx, const double* A, int64_t n, int64_t lda, int64_t k, int64_t s, double* v,
                           int64_t ldv, double* lambda_host, int64_t* r_out) {
    if (k <= 0) fail(RNLA_ERR_INVALID_PARAMETERS, "Rank k must be positive");
    // every eigenvalue of A must be >= 0 (lora_drivers.rs:166-172)
    {
        DevBuf<double> W((size_t)n * n, ctx.stream), lam(n, ctx.stream);
        DevBuf<double> Ac((size_t)n * n, ctx.stream);
        copy_matrix(ctx, n, n, A, lda, Ac, n);
        sym_eig(ctx, Ac, n, lam, W);
        std::vector<double> h(n);
        RNLA_CUDA(cudaMemcpyAsync(h.data(), lam.get(), n * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
        RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
        for (double x : h)
            if (x < 0.0) fail(RNLA_ERR_NOT_POSITIVE_SEMIDEFINITE, "Matrix is not positive semi-definite");
    }
    const bool finite = all_finite(ctx, n, n, A, lda);
    DMat S = tsog1_ref(ctx, A, n, n, lda, k + s, 3, 1, finite);        // lines 174
    const int64_t l = S.cols;
    DevBuf<double> Y((size_t)n * l, ctx.stream), SY((size_t)l * l, ctx.stream), Ri((size_t)l * l, ctx.stream),
        B((size_t)n * l, ctx.stream), U((size_t)n * l, ctx.stream), sg(l, ctx.stream), Vs((size_t)l * l, ctx.stream);
    gemm_f64(ctx, 'N', 'N', n, l, n, 1.0, A, lda, S.p(), n, 0.0, Y, n);     // Y = A S
    const double nu = sqrt((double)n) * 2.220446049250313e-16 * frob_norm(ctx, Y, n * l);
    {
        int g = (int)div_up(n * l, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        axpy_mat_kernel<<<g, 256, 0, ctx.stream>>>(Y, S.p(), n * l, nu);     // Y_new = Y + nu S
        RNLA_LAUNCH_CHECK();
    }
    gemm_f64(ctx, 'T', 'N', l, l, n, 1.0, S.p(), n, Y, n, 0.0, SY, l);      // S^T Y_new
    if (!cholesky_upper(ctx, SY, l, l))
        fail(RNLA_ERR_MATRIX_DECOMPOSITION, "Cholesky Decomposition Failed");
    if (!upper_inverse(ctx, SY, l, l, Ri, l)) fail(RNLA_ERR_MATRIX_DECOMPOSITION, "Matrix Inverse Failed");
    gemm_f64(ctx, 'N', 'N', n, l, l, 1.0, Y, n, Ri, l, 0.0, B, n);          // B = Y_new R^-1
    small_svd(ctx, B, n, l, n, U, n, sg, Vs, l);
    std::vector<double> sh(l);
    RNLA_CUDA(cudaMemcpyAsync(sh.data(), sg.get(), l * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    std::vector<double> lam;
    for (double x : sh)
        if (x > 0.0) lam.push_back(x * x);
    int64_t above = 0;
    for (double x : lam)
        if (x > nu) ++above;
    const int64_t r = k < above ? k : above;
    for (int64_t i = 0; i < r; ++i) lambda_host[i] = lam[(size_t)i] - nu;
    if (r > 0) copy_matrix(ctx, n, r, U, n, v, ldv);
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    *r_out = r;
}

// ---------------------------------------------------------------------------
// Shared helpers for the randomized drivers
// ---------------------------------------------------------------------------
// C (MM x NN) = X^T Y with X (K x MM), Y (K x NN) in the requested precision.
static void product_tn(Ctx& ctx, int prec, const double* X, int64_t K, int64_t MM, int64_t ldx,
                       const double* Y, int64_t NN, int64_t ldy, int dx, int dy, double* C,
                       int64_t ldc) {
    if (prec == RNLA_PREC_FP64) gemm_f64(ctx, 'T', 'N', MM, NN, K, 1.0, X, ldx, Y, ldy, 0.0, C, ldc);
    else tc_gemm_tn(ctx, X, K, MM, ldx, Y, NN, ldy, dx, dy, C, ldc);
}

struct SvdOut {
    int64_t r = 0;
};

// SVD finish of lora_drivers.rs:51-68 from Q (m x cq) and B (cq x n).
static int64_t svd_finish(Ctx& ctx, int prec, const double* Q, int64_t m, int64_t cq, const double* B,
                          int64_t n, int64_t k, double* U, int64_t ldu, double* sig, double* Vt,
                          int64_t ldvt) {
    const int64_t r = k < cq ? k : cq;
    const int64_t t = cq < n ? cq : n;
    DevBuf<double> UB((size_t)cq * t, ctx.stream), VB((size_t)n * t, ctx.stream), sg(t, ctx.stream);
    small_svd(ctx, B, cq, n, cq, UB, cq, sg, VB, n);
    // U = Q U_B[:, :r]
    gemm_f64(ctx, 'N', 'N', m, r, cq, 1.0, Q, m, UB, cq, 0.0, U, ldu);
    (void)prec;
    RNLA_CUDA(cudaMemcpyAsync(sig, sg.get(), r * sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    transpose(ctx, n, r, VB, n, Vt, ldvt);
    return r;
}

// Orthonormal basis of Y (m x l, ld m, m >= l) in place: CholeskyQR2 with
// the Grams and the triangular products on the split-bf16 tensor-core GEMM
// at level 3 (FP32 accumulation over K = m), Cholesky in float-float, R^-1 in FP64; the
// FP64 Householder basis when a Cholesky pivot fails.  Returns 1 on
// fallback.
static int orthonormalize_bfx(Ctx& ctx, double* Y, int64_t m, int64_t l, int passes = 2) {
    if (m < l) return orthonormalize(ctx, Y, m, l, m, true), 1;
    DevBuf<double> G((size_t)l * l, ctx.stream), Ri((size_t)l * l, ctx.stream), T((size_t)m * l, ctx.stream);
    for (int pass = 0; pass < passes; ++pass) {
        {
            BfxPlanes ya, yb;
            bfx_planes(ctx, ya, Y, false, l, m, m, 1, bfx_tile_rows(3, true), 3);     // columns of Y
            bfx_planes(ctx, yb, Y, false, l, m, m, 1, bfx_tile_rows(3, false), 3);
            bfx_gemm(ctx, 3, ya, yb, G, l, false);                                    // G = Y^T Y
        }
        if (!cholesky_upper_ff(ctx, G, l, l) || !upper_inverse(ctx, G, l, l, Ri, l)) {
            orthonormalize(ctx, Y, m, l, m, true);
            return 1;
        }
        {
            BfxPlanes yr, wr;
            bfx_planes(ctx, yr, Y, false, m, l, 1, m, bfx_tile_rows(3, true), 3);     // rows of Y
            bfx_planes(ctx, wr, Ri, false, l, l, l, 1, bfx_tile_rows(3, false), 3);   // columns of R^-1
            bfx_gemm(ctx, 3, yr, wr, T, m, false);                                    // T = Y R^-1
        }
        copy_matrix(ctx, m, l, T, m, Y, m);
    }
    return 0;
}

// The RandNLA-mode range finder and projection on the tensor cores
// (lora_helpers.rs:17-44 with a Gaussian Omega and q power iterations):
// Y = A Omega, q times {Z = orth(A^T Y), Y = orth(A Z)}, B = Q^T A, then the
// small-SVD finish of lora_drivers.rs:51-68.  A is read as bf16 planes made
// once (its rows for the A Z products, its columns for A^T Y, level 2); the
// projection B = Q^T A is an exact digit product (tc_exact_tn).  Omega is
// the FP64 Gaussian of the FP64 path (same key).
static int64_t rand_svd_bfx(Ctx& ctx, const void* Av, bool a_f32, int64_t m, int64_t n, int64_t lda, int64_t k,
                            int64_t l, const rnla_options& o, double* U, int64_t ldu, double* sig, double* Vt,
                            int64_t ldvt, int& fallbacks, int& sweeps, StageTimer& tm) {
    const int LP = (o.digits_a >= 1 && o.digits_a <= 3) ? o.digits_a : 2;   // power-iteration level
    const RngKey key = key_of(&o.rng);
    BfxPlanes arow, acol;
    bfx_planes(ctx, arow, Av, a_f32, m, n, 1, lda, bfx_tile_rows(LP, true), LP);   // A(i, k) = A[i + k lda]
    bfx_planes(ctx, acol, Av, a_f32, n, m, lda, 1, bfx_tile_rows(LP, true), LP);  // A^T(i, k) = A[k + i lda]
    DevBuf<double> Y((size_t)m * l, ctx.stream), Z((size_t)n * l, ctx.stream);
    {
        DevBuf<double> Om((size_t)n * l, ctx.stream);
        sketch_fill_f64(ctx, DIST_GAUSSIAN, key, n, l, Om, n);
        BfxPlanes op;
        bfx_planes(ctx, op, Om, false, l, n, n, 1, bfx_tile_rows(LP, false), LP);
        bfx_gemm(ctx, LP, arow, op, Y, m, false);                                    // Y = A Omega
    }
    // between products the basis only has to stay well conditioned (its span
    // is what the next product uses): one CholeskyQR pass; the projection
    // below makes the final one orthonormal in float-float
    fallbacks += orthonormalize_bfx(ctx, Y, m, l, 1);
    for (int it = 0; it < o.power_iters; ++it) {
        {
            BfxPlanes yp;
            bfx_planes(ctx, yp, Y, false, l, m, m, 1, bfx_tile_rows(LP, false), LP);
            bfx_gemm(ctx, LP, acol, yp, Z, n, false);                                // Z = A^T Q
        }
        fallbacks += orthonormalize_bfx(ctx, Z, n, l, 1);
        {
            BfxPlanes zp;
            bfx_planes(ctx, zp, Z, false, l, n, n, 1, bfx_tile_rows(LP, false), LP);
            bfx_gemm(ctx, LP, arow, zp, Y, m, false);                                // Y = A Z
        }
        // one split-bf16 CholeskyQR pass also before the projection: it brings
        // kappa(Y) to ~1, so the float-float R below does not amplify errors
        fallbacks += orthonormalize_bfx(ctx, Y, m, l, 1);
    }
    tm.mark();
    // Projection.  Y is orthonormal only to the split-bf16 level (its Grams
    // accumulate in FP32 over K = m); Q = Y R^-1 with R = chol(Y^T Y) formed
    // in float-float is orthonormal to ~1e-14, and B = Q^T A = R^-T (Y^T A)
    // needs no explicit Q: Y^T A on the tensor cores at level 3, R^-T applied
    // in float-float.
    DevBuf<double> G((size_t)l * l, ctx.stream), Ri((size_t)l * l, ctx.stream), Bt((size_t)l * n, ctx.stream),
        B((size_t)l * n, ctx.stream);
    gram_ff(ctx, Y, m, l, Y, m, l, m, G, l);
    if (!cholesky_upper_ff(ctx, G, l, l) || !upper_inverse(ctx, G, l, l, Ri, l)) {
        // Y lost rank: the FP64 Householder basis and the plain projection
        fallbacks += orthonormalize(ctx, Y, m, l, m, true);
        fill_identity(ctx, l, l, Ri, l);
    }
    // Y^T A (l x n) exactly on the tensor cores (integer digits, int64
    // windows): an FP32-accumulated product would leave B with errors of
    // ~1e-5 relative to sigma_k at K = 65536
    tc_exact_tn(ctx, Av, a_f32, m, n, lda, Y, l, m, Bt, l, true, 4);
    gram_ff(ctx, Ri, l, l, Bt, l, n, l, B, l);                                       // B = R^-T (Y^T A)
    tm.mark();
    // small SVD of B; U = Y (R^-1 U_B)
    const int64_t r = k < l ? k : l;
    DevBuf<double> UB((size_t)l * l, ctx.stream), sg(l, ctx.stream), VB((size_t)n * l, ctx.stream);
    if (!small_svd_gram(ctx, B, l, n, l, UB, l, sg, VB, n, &sweeps)) small_svd(ctx, B, l, n, l, UB, l, sg, VB, n);
    {
        DevBuf<double> RiT((size_t)l * l, ctx.stream), W2((size_t)l * r, ctx.stream);
        transpose(ctx, l, l, Ri, l, RiT, l);
        gram_ff(ctx, RiT, l, l, UB, l, r, l, W2, l);                                 // R^-1 U_B[:, :r]
        BfxPlanes yr, wp;
        bfx_planes(ctx, yr, Y, false, m, l, 1, m, bfx_tile_rows(3, true), 3);        // rows of Y
        bfx_planes(ctx, wp, W2, false, r, l, l, 1, bfx_tile_rows(3, false), 3);      // columns of W2
        bfx_gemm(ctx, 3, yr, wp, U, ldu, false);
    }
    RNLA_CUDA(cudaMemcpyAsync(sig, sg.get(), r * sizeof(double), cudaMemcpyDeviceToDevice, ctx.stream));
    transpose(ctx, n, r, VB, n, Vt, ldvt);
    return r;
}

static int64_t rand_svd_impl(Ctx& ctx, const void* Av, bool a_f32, int64_t m, int64_t n, int64_t lda,
                             int64_t k, double epsilon, int64_t s, const rnla_options& o, double* U,
                             int64_t ldu, double* sig, double* Vt, int64_t ldvt, rnla_stats* st) {
    if (k == 0) {
        char b[96];
        snprintf(b, sizeof b, "Rank k must be positive, current input is %lld", (long long)k);
        fail(RNLA_ERR_INVALID_PARAMETERS, b);
    }
    if (!(epsilon > 0.0)) {
        char b[96];
        snprintf(b, sizeof b, "Epsilon must be positive, current input is %g", epsilon);
        fail(RNLA_ERR_INVALID_PARAMETERS, b);
    }
    if (s == 0) {
        char b[112];
        snprintf(b, sizeof b, "Oversampling parameter s must be positive, current input is %lld",
                 (long long)s);
        fail(RNLA_ERR_INVALID_PARAMETERS, b);
    }
    if (k < 0 || s < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "k and s must be non-negative");
    if (m <= 0 || n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    StageTimer tm(ctx.stream);
    tm.mark();
    // A as double for the FP64 products (stored-FP32 inputs are widened once);
    // the tensor-core path reads FP32 or FP64 A directly
    DevBuf<double> Aw;
    const double* A = static_cast<const double*>(Av);
    int64_t ld = lda;
    if (a_f32 && o.precision == RNLA_PREC_FP64) {
        Aw.alloc((size_t)m * n, ctx.stream);
        copy_matrix_f32_to_f64(ctx, m, n, static_cast<const float*>(Av), lda, Aw, m);
        A = Aw.get();
        ld = m;
    }
    int64_t r = 0;
    int fallbacks = 0, sweeps = 0;
    if (o.mode == RNLA_MODE_RANDNLA && o.precision != RNLA_PREC_FP64) {
        if (!tc_available(ctx))
            fail(RNLA_ERR_UNSUPPORTED, "tensor-core precision requested but sm_103a kernels unavailable");
        int64_t l = k + s;
        const int64_t mn = m < n ? m : n;
        if (l > mn) l = mn;
        r = rand_svd_bfx(ctx, Av, a_f32, m, n, lda, k, l, o, U, ldu, sig, Vt, ldvt, fallbacks, sweeps, tm);
    } else if (o.mode == RNLA_MODE_REFERENCE) {
        if (o.precision != RNLA_PREC_FP64)
            fail(RNLA_ERR_UNSUPPORTED, "reference mode runs in FP64 only");
        const bool finite = all_finite(ctx, m, n, A, ld);
        DMat Q = rf1_ref(ctx, A, m, n, ld, k + s, finite);                 // QB1 line 20
        tm.mark();
        const int64_t cq = Q.cols;
        DevBuf<double> B((size_t)cq * n, ctx.stream);
        gemm_f64(ctx, 'T', 'N', cq, n, m, 1.0, Q.p(), m, A, ld, 0.0, B, cq);   // QB1 line 21
        tm.mark();
        r = svd_finish(ctx, o.precision, Q.p(), m, cq, B, n, k, U, ldu, sig, Vt, ldvt);
    } else {
        // Gaussian range finder, q power iterations, re-orthonormalised after
        // every product, on the FP64 CUDA cores.
        const int prec = o.precision;
        int64_t l = k + s;
        const int64_t mn = m < n ? m : n;
        if (l > mn) l = mn;
        const RngKey key = key_of(&o.rng);
        DevBuf<double> Y((size_t)m * l, ctx.stream), Z((size_t)n * l, ctx.stream);
        const bool force_hh = (o.orth == 1);
        {
            DevBuf<double> Om((size_t)n * l, ctx.stream);
            sketch_fill_f64(ctx, DIST_GAUSSIAN, key, n, l, Om, n);
            gemm_f64(ctx, 'N', 'N', m, l, n, 1.0, A, ld, Om, n, 0.0, Y, m);
        }
        fallbacks += orthonormalize(ctx, Y, m, l, m, force_hh);
        for (int it = 0; it < o.power_iters; ++it) {
            product_tn(ctx, prec, A, m, n, ld, Y, l, m, o.digits_a, o.digits_b, Z, n);   // Z = A^T Q
            fallbacks += orthonormalize(ctx, Z, n, l, n, force_hh);
            gemm_f64(ctx, 'N', 'N', m, l, n, 1.0, A, ld, Z, n, 0.0, Y, m);            // Y = A Z
            fallbacks += orthonormalize(ctx, Y, m, l, m, force_hh);
        }
        tm.mark();
        DevBuf<double> B((size_t)l * n, ctx.stream);
        product_tn(ctx, prec, Y, m, l, m, A, n, ld, o.digits_b, o.digits_a, B, l);   // B = Q^T A
        tm.mark();
        r = svd_finish(ctx, prec, Y, m, l, B, n, k, U, ldu, sig, Vt, ldvt);
    }
    tm.mark();
    if (st) {
        st->rank = r;
        st->orth_fallbacks = fallbacks;
        st->svd_sweeps = sweeps;
        st->precision_used = o.precision;
        st->ms_sketch = tm.ms(0, 1);
        st->ms_factor = tm.ms(1, 2);
        st->ms_solve = tm.ms(2, 3);
        st->ms_total = tm.ms(0, 3);
    }
    return r;
}

// ---------------------------------------------------------------------------
// blendenpik (sketch_and_precondition.rs:26-59)
// ---------------------------------------------------------------------------
static int64_t sketch_rows(int64_t m, int64_t n, double sf) {
    return (sf * (double)n > (double)m) ? m : (int64_t)std::floor(sf * (double)n);   // line 49
}

static void blendenpik_validate(int64_t m, int64_t n, double epsilon, int64_t l, double sf) {
    char b[160];
    if (m < n) {
        snprintf(b, sizeof b, "Need more columns than rows, found %lld rows and %lld columns",
                 (long long)m, (long long)n);
        fail(RNLA_ERR_NOT_OVERDETERMINED, b);
    }
    if (sf < 1.0) {
        snprintf(b, sizeof b, "Sampling factor must be greater than 1, current input is %g", sf);
        fail(RNLA_ERR_INVALID_PARAMETERS, b);
    }
    if (!(epsilon > 0.0)) {
        snprintf(b, sizeof b, "Epsilon must be positive, current input is %g", epsilon);
        fail(RNLA_ERR_INVALID_PARAMETERS, b);
    }
    if (l == 0) {
        snprintf(b, sizeof b, "Number of iterations must be positive, current input is %lld",
                 (long long)l);
        fail(RNLA_ERR_INVALID_PARAMETERS, b);
    }
    if (l < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "l must be positive");
    if (n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must have at least one column");
}

// max and min of the first n diagonal entries of R (ld), one CTA
__global__ void diag_range_kernel(const double* __restrict__ R, int64_t n, int64_t ld, double* __restrict__ out) {
    __shared__ double mx[256], mn[256];
    double a = 0.0, b = INFINITY;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = fabs(R[i + i * ld]);
        a = fmax(a, v);
        b = fmin(b, v);
    }
    mx[threadIdx.x] = a;
    mn[threadIdx.x] = b;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            mx[threadIdx.x] = fmax(mx[threadIdx.x], mx[threadIdx.x + s]);
            mn[threadIdx.x] = fmin(mn[threadIdx.x], mn[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = mx[0];
        out[1] = mn[0];
    }
}

// R of the sketch [S a, S b] (d x nc, ld d) without Householder reflections:
// the float-float Gram of [S a, S b] (gram_ff, ~2^-48 relative) and a blocked
// float-float Cholesky of it.  Its last column is R^-T (S a)^T S b = (Q^T S b)[:n],
// the reference's z_0 (sketch_and_precondition.rs:54), so R and z_0 land in
// the top n rows of SK exactly where the Householder QR leaves them.  The
// Gram's rounding perturbs the preconditioned sketch (S a) R^-1 by about
// 2^-48 kappa(S a)^2; R is kept only when that stays below 2^-5 (kappa
// estimated by the ratio of R's extreme diagonal entries, a lower bound),
// so the preconditioner's quality -- and the LSQR iteration count -- is that
// of the Householder R.  Otherwise SK is left untouched and false returned.
static bool cholqr_sketch(Ctx& ctx, double* SK, int64_t d, int64_t n, int64_t nc) {
    DevBuf<double> Gm((size_t)nc * nc, ctx.stream), ext(2, ctx.stream);
    gram_ff(ctx, SK, d, nc, SK, d, nc, d, Gm, nc);
    if (!cholesky_upper_ff(ctx, Gm, nc, nc, n)) return false;
    diag_range_kernel<<<1, 256, 0, ctx.stream>>>(Gm, n, nc, ext);
    RNLA_LAUNCH_CHECK();
    double h[2] = {0.0, 0.0};
    RNLA_CUDA(cudaMemcpyAsync(h, ext.get(), sizeof h, cudaMemcpyDeviceToHost, ctx.stream));
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    if (!(h[1] > 0.0)) return false;
    const double ratio = h[0] / h[1];
    if (!(ratio * ratio * 0x1p-48 <= 0x1p-5)) return false;
    copy_matrix(ctx, n, nc, Gm, nc, SK, d);
    return true;
}

// With a feed, A is still arriving from the host in column chunks: the
// tensor-core sketch consumes each column tile as it lands; every other
// path waits for the whole matrix first.
// lsrn (sketch_and_precondition.rs:82-119) is the same pipeline started
// from z0 = 0: its preconditioner V Sigma^-1 is R^-1 U_R, and the Krylov
// solvers are invariant under the orthogonal U_R.
static void blendenpik_impl(Ctx& ctx, const void* Av, bool a_f32, int64_t m, int64_t n, int64_t lda,
                            const double* b, double epsilon, int64_t l, double sf,
                            const rnla_options& o, double* x, rnla_stats* st,
                            const ColumnFeed* feed = nullptr, bool lsrn = false) {
    blendenpik_validate(m, n, epsilon, l, sf);
    const int64_t d = sketch_rows(m, n, sf);
    if (d < n) fail(RNLA_ERR_SINGULAR_MATRIX, "sketch has fewer rows than columns");
    StageTimer tm(ctx.stream);
    tm.mark();
    const RngKey key = key_of(&o.rng);
    const int64_t nc = n + 1;
    LsqrFFInput lsqr_in;
    DevBuf<double> SK((size_t)d * nc, ctx.stream);
    if (o.precision == RNLA_PREC_FP64) {
        if (feed) feed->wait_all(ctx.stream);
        // the reference's data flow: dense S (line 50), S a and S b (lines 51-52)
        DevBuf<double> S((size_t)d * m, ctx.stream);
        sketch_fill_f64(ctx, DIST_GAUSSIAN, key, d, m, S, d);
        DevBuf<double> Aw;
        const double* A = static_cast<const double*>(Av);
        int64_t ld = lda;
        if (a_f32) {
            Aw.alloc((size_t)m * n, ctx.stream);
            copy_matrix_f32_to_f64(ctx, m, n, static_cast<const float*>(Av), lda, Aw, m);
            A = Aw.get();
            ld = m;
        }
        gemm_f64(ctx, 'N', 'N', d, n, m, 1.0, S, d, A, ld, 0.0, SK, d);
        gemm_f64(ctx, 'N', 'N', d, 1, m, 1.0, S, d, b, m, 0.0, SK.get() + n * d, d);
    } else {
        if (!tc_available(ctx))
            fail(RNLA_ERR_UNSUPPORTED, "tensor-core precision requested but sm_103a kernels unavailable");
        // the whole BF16X solve is enqueued without intermediate host
        // synchronisation; the device status is checked once at the end
        ctx.deferred = true;
        // BF16X + LSQR: the solver's row-major (FP32 or float-float) copies of
        // A and b.  FP32 A: the sketch's digit-plane kernel writes the
        // row-major copy from the same reads of A (also column tile by column
        // tile as a feed lands).  FP64 A on the device: the float-float rows
        // are built on the main stream while the sketch generator (side
        // stream) is still running, ahead of the MMA that waits for it; with
        // a feed, on the side stream after the sketch.
        const bool ffp = o.inner_solver != RNLA_SOLVER_CGLS && lsqr_ff_supported(n);
        std::function<void(cudaStream_t)> before_mma;
        SketchRowMajor rm;
        if (ffp && (a_f32 || !feed)) lsqr_ff_alloc(ctx, Av, a_f32, m, n, lsqr_in);
        if (ffp && a_f32) {
            rm.dst = reinterpret_cast<float*>(lsqr_in.AF.get());
            rm.ld = lsqr_in.ldf;
        } else if (ffp && !feed) {
            before_mma = [&](cudaStream_t st) { lsqr_ff_build(ctx, lsqr_in, lda, b, st); };
        }
        // S [a b] in one pass: b rides along as column n of the digit planes
        tc_sketch_apply(ctx, key, Av, a_f32, m, n, lda, b, d, o.digits_a, SK, d, feed, DIST_GAUSSIAN, before_mma,
                        rm);
        if (feed) feed->wait_all(ctx.stream);
        if (ffp && a_f32) lsqr_ff_build(ctx, lsqr_in, lda, b, ctx.stream, true);
        else if (ffp && feed) lsqr_ff_prepare(ctx, Av, a_f32, m, n, lda, b, lsqr_in);
    }
    tm.mark();
    // QR of S a with S b carried as an extra column: R and z0 = (Q^T S b)[:n] (lines 53-54)
    DevBuf<double> tau(n, ctx.stream), Mi((size_t)n * n, ctx.stream);
    bool inv_ok;
    int qr_fallbacks = 0;
    if (o.precision != RNLA_PREC_FP64 && qr_ff_supported(ctx, d, n, nc)) {
        // float-float factorization on the FP32 pipe (qr_ff.cu)
        householder_qr_ff(ctx, SK, d, n, nc, d);
        inv_ok = upper_inverse_ff(ctx, SK, n, d, Mi, n);
    } else if (o.precision != RNLA_PREC_FP64 && qr_ff_tsqr_supported(ctx, d, n, nc)) {
        // wider sketches (d = 4096 at n = 1024): CholeskyQR where the sketch's
        // conditioning allows it, else two row halves, then their R blocks
        if (o.orth != 0 || !cholqr_sketch(ctx, SK, d, n, nc)) {
            if (o.orth == 0) ++qr_fallbacks;
            householder_qr_ff_tsqr(ctx, SK, d, n, nc, d);
        }
        inv_ok = upper_inverse_ff(ctx, SK, n, d, Mi, n);
    } else {
        householder_qr(ctx, SK, d, n, nc, d, tau);
        inv_ok = upper_inverse(ctx, SK, n, d, Mi, n);               // line 55
        // the float-float LSQR applies M rounded to ~48 bits; x = M z must use
        // that same M (with kappa(R) = 1e6 the difference would show in x)
        if (inv_ok && lsqr_in.ready) ff_round_upper(ctx, Mi, n, n);
    }
    if (!inv_ok) fail(RNLA_ERR_SINGULAR_MATRIX, "the R factor of the sketch is singular");
    tm.mark();
    const double* z0 = lsrn ? nullptr : SK.get() + n * d;
    DevBuf<double> z(n, ctx.stream);
    const double* a64 = a_f32 ? nullptr : static_cast<const double*>(Av);
    const float* a32 = a_f32 ? static_cast<const float*>(Av) : nullptr;
    int64_t iters = 0, istop = 0;
    LsqrResult lr;
    LsqrPending pend;
    if (o.inner_solver == RNLA_SOLVER_CGLS) {
        bool conv = false;
        iters = cgls_solve(ctx, a64, a32, m, n, lda, Mi, b, z0, epsilon, l, z, &conv);   // line 57
        istop = conv ? 1 : 0;
    } else {
        LsqrParams p;
        p.atol = o.atol;
        p.btol = o.btol;
        p.conlim = o.conlim > 0 ? o.conlim : 1e8;
        p.iter_lim = l;
        if (o.atol == 0.0 && o.btol == 0.0) p.abs_arnorm_tol = epsilon;
        lr = lsqr_solve(ctx, a64, a32, m, n, lda, Mi, b, z0, p, z, nullptr, nullptr,
                        o.precision != RNLA_PREC_FP64, lsqr_in.ready ? &lsqr_in : nullptr, &pend);
    }
    trmv_upper(ctx, Mi, n, n, z, x);                                // line 58
    tm.mark();
    if (ctx.deferred) ctx.finish("blendenpik (BF16X)");
    if (o.inner_solver != RNLA_SOLVER_CGLS) {
        pend.resolve(lr);              // after the synchronisation in finish()
        iters = lr.itn;
        istop = lr.istop;
    }
    if (st) {
        st->iterations = iters;
        st->istop = istop;
        st->r1norm = lr.r1norm;
        st->r2norm = lr.r2norm;
        st->anorm = lr.anorm;
        st->acond = lr.acond;
        st->arnorm = lr.arnorm;
        st->xnorm = lr.xnorm;
        st->sketch_rows = d;
        st->precision_used = o.precision;
        st->orth_fallbacks = qr_fallbacks;
        st->ms_sketch = tm.ms(0, 1);
        st->ms_factor = tm.ms(1, 2);
        st->ms_solve = tm.ms(2, 3);
        st->ms_total = tm.ms(0, 3);
        st->ms_kernel = lr.ms_kernel;
    }
}

// zero the strict lower triangle of an n x n matrix
__global__ void zero_lower_kernel(double* __restrict__ a, int64_t n, int64_t ld) {
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        if (i > j) a[i + j * ld] = 0.0;
    }
}

// y_i <- y_i / sigma_i, 0 where sigma_i == 0 (solvers.rs:56-70)
__global__ void divide_sigma_kernel(double* __restrict__ y, const double* __restrict__ sigma, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (sigma[i] != 0.0) ? y[i] / sigma[i] : 0.0;
}

// sketch_and_solve.rs:24-33 / 53-65.  [S a, S b] in one d x (n+1) block
// (d = m / 4); its Householder QR gives R and Q^T S b in column n.  The SVD
// variant factors R = U_R Sigma V^T: the SVD of S a is (Q U_R) Sigma V^T,
// so U^T S b = U_R^T (Q^T S b).
static void sketch_solve_impl(Ctx& ctx, const void* Av, bool a_f32, int64_t m, int64_t n, int64_t lda,
                              const double* b, bool use_svd, const rnla_options& o, double* x,
                              const ColumnFeed* feed) {
    if (m <= 0 || n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    const int64_t d = m / 4;
    if (d < n) fail(RNLA_ERR_INVALID_DIMENSIONS, "the sketch has m / 4 rows; it needs at least n");
    const RngKey key = key_of(&o.rng);
    const int64_t nc = n + 1;
    DevBuf<double> SK((size_t)d * nc, ctx.stream);
    if (o.precision == RNLA_PREC_FP64) {
        if (feed) feed->wait_all(ctx.stream);
        DevBuf<double> S((size_t)d * m, ctx.stream);
        sketch_fill_f64(ctx, DIST_GAUSSIAN, key, d, m, S, d);
        DevBuf<double> Aw;
        const double* A = static_cast<const double*>(Av);
        int64_t ld = lda;
        if (a_f32) {
            Aw.alloc((size_t)m * n, ctx.stream);
            copy_matrix_f32_to_f64(ctx, m, n, static_cast<const float*>(Av), lda, Aw, m);
            A = Aw.get();
            ld = m;
        }
        gemm_f64(ctx, 'N', 'N', d, n, m, 1.0, S, d, A, ld, 0.0, SK, d);
        gemm_f64(ctx, 'N', 'N', d, 1, m, 1.0, S, d, b, m, 0.0, SK.get() + n * d, d);
    } else {
        if (!tc_available(ctx))
            fail(RNLA_ERR_UNSUPPORTED, "tensor-core precision requested but sm_103a kernels unavailable");
        tc_sketch_apply(ctx, key, Av, a_f32, m, n, lda, b, d, o.digits_a, SK, d, feed);
        if (feed) feed->wait_all(ctx.stream);
    }
    if (o.precision != RNLA_PREC_FP64 && qr_ff_supported(ctx, d, n, nc)) {
        householder_qr_ff(ctx, SK, d, n, nc, d);
    } else if (o.precision != RNLA_PREC_FP64 && qr_ff_tsqr_supported(ctx, d, n, nc)) {
        householder_qr_ff_tsqr(ctx, SK, d, n, nc, d);
    } else {
        DevBuf<double> tau(n, ctx.stream);
        householder_qr(ctx, SK, d, n, nc, d, tau);
    }
    const double* z = SK.get() + n * d;          // (Q^T S b)[:n]
    if (!use_svd) {
        upper_solve_skip_zero(ctx, SK, n, d, z, x);
        return;
    }
    DevBuf<double> R((size_t)n * n, ctx.stream), U((size_t)n * n, ctx.stream), V((size_t)n * n, ctx.stream),
        sig(n, ctx.stream), y(n, ctx.stream);
    copy_matrix(ctx, n, n, SK, d, R, n);
    {
        int g = (int)div_up(n * n, 256);
        if (g > 8 * ctx.sm_count) g = 8 * ctx.sm_count;
        zero_lower_kernel<<<g, 256, 0, ctx.stream>>>(R, n, n);
        RNLA_LAUNCH_CHECK();
    }
    small_svd(ctx, R, n, n, n, U, n, sig, V, n);
    gemm_f64(ctx, 'T', 'N', n, 1, n, 1.0, U, n, z, d, 0.0, y, n);
    divide_sigma_kernel<<<(unsigned)div_up(n, 256), 256, 0, ctx.stream>>>(y, sig, n);
    RNLA_LAUNCH_CHECK();
    gemm_f64(ctx, 'N', 'N', n, 1, n, 1.0, V, n, y, n, 0.0, x, n);
}

}  // namespace rnla

using namespace rnla;

extern "C" {

// ---- solvers.rs ----
int rnla_solve_upper_triangular_system_dev(const double* u, int64_t n, int64_t ldu, const double* y,
                                           double* x, void* stream) {
    RNLA_API_BEGIN
    check_mat(n, n, ldu);
    Ctx ctx((cudaStream_t)stream);
    upper_solve_skip_zero(ctx, u, n, ldu, y, x);
    RNLA_API_END
}

int rnla_solve_upper_triangular_system(const double* u, int64_t n, int64_t ldu, const double* y,
                                       double* x) {
    RNLA_API_BEGIN
    check_mat(n, n, ldu);
    if (n == 0) return abi_ok();
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> U((size_t)n * n, s), Y(n, s), X(n, s);
    h2d_matrix(U, n, u, ldu, n, n, s);
    RNLA_CUDA(cudaMemcpyAsync(Y.get(), y, n * sizeof(double), cudaMemcpyHostToDevice, s));
    upper_solve_skip_zero(ctx, U, n, n, Y, X);
    RNLA_CUDA(cudaMemcpyAsync(x, X.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

int rnla_lsqr_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda, const double* b_dev,
                  double damp, double atol, double btol, double conlim, int64_t iter_lim,
                  int32_t calc_var, const double* x0_dev, double* x_dev, rnla_lsqr_result* result,
                  double* arnorms_host, double* var_dev, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m == 0 || n == 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    Ctx ctx((cudaStream_t)stream);
    LsqrParams p;
    p.damp = damp;
    p.atol = atol;
    p.btol = btol;
    p.conlim = conlim;
    p.iter_lim = iter_lim < 0 ? 2 * n : iter_lim;
    p.calc_var = calc_var != 0;
    DevBuf<double> arn(p.iter_lim > 0 ? p.iter_lim : 1, ctx.stream);
    LsqrResult r = lsqr_solve(ctx, a_dev, nullptr, m, n, lda, nullptr, b_dev, x0_dev, p, x_dev,
                              var_dev, arn, false);
    if (result) {
        result->istop = r.istop;
        result->itn = r.itn;
        result->r1norm = r.r1norm;
        result->r2norm = r.r2norm;
        result->anorm = r.anorm;
        result->acond = r.acond;
        result->xnorm = r.xnorm;
    }
    if (arnorms_host) {
        const int64_t cnt = r.itn > 0 ? r.itn : 1;
        RNLA_CUDA(cudaMemcpyAsync(arnorms_host, arn.get(), cnt * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx.stream));
        RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    }
    RNLA_API_END
}

int rnla_lsqr(const double* a, int64_t m, int64_t n, int64_t lda, const double* b, double damp,
              double atol, double btol, double conlim, int64_t iter_lim, int32_t calc_var,
              const double* x0, double* x, rnla_lsqr_result* result, double* arnorms, double* var) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m == 0 || n == 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    cudaStream_t s = host_stream();
    DevBuf<double> A((size_t)m * n, s), B(m, s), X0(n, s), X(n, s), V(n, s);
    h2d_matrix(A, m, a, lda, m, n, s);
    RNLA_CUDA(cudaMemcpyAsync(B.get(), b, m * sizeof(double), cudaMemcpyHostToDevice, s));
    if (x0) RNLA_CUDA(cudaMemcpyAsync(X0.get(), x0, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int rc = rnla_lsqr_dev(A, m, n, m, B, damp, atol, btol, conlim, iter_lim, calc_var,
                           x0 ? X0.get() : nullptr, X, result, arnorms, (calc_var && var) ? V.get() : nullptr, s);
    if (rc != RNLA_OK) return rc;
    RNLA_CUDA(cudaMemcpyAsync(x, X.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (calc_var && var) RNLA_CUDA(cudaMemcpyAsync(var, V.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

// ---- cg.rs ----
int rnla_cgls_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda, const double* b_dev,
                  double tolerance, int64_t num_iterations, const double* x0_dev, double* x_dev,
                  int64_t* iterations_out, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m == 0 || n == 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    if (num_iterations < 0) fail(RNLA_ERR_NEGATIVE_DIMENSIONS, "num_iterations must be >= 0");
    Ctx ctx((cudaStream_t)stream);
    bool conv = false;
    const int64_t it = cgls_solve(ctx, a_dev, nullptr, m, n, lda, nullptr, b_dev, x0_dev, tolerance,
                                  num_iterations, x_dev, &conv);
    if (iterations_out) *iterations_out = it;
    RNLA_API_END
}

int rnla_cgls(const double* a, int64_t m, int64_t n, int64_t lda, const double* b, double tolerance,
              int64_t num_iterations, const double* x0, double* x, int64_t* iterations_out) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m == 0 || n == 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    cudaStream_t s = host_stream();
    DevBuf<double> A((size_t)m * n, s), B(m, s), X0(n, s), X(n, s);
    h2d_matrix(A, m, a, lda, m, n, s);
    RNLA_CUDA(cudaMemcpyAsync(B.get(), b, m * sizeof(double), cudaMemcpyHostToDevice, s));
    if (x0) RNLA_CUDA(cudaMemcpyAsync(X0.get(), x0, n * sizeof(double), cudaMemcpyHostToDevice, s));
    int rc = rnla_cgls_dev(A, m, n, m, B, tolerance, num_iterations, x0 ? X0.get() : nullptr, X,
                           iterations_out, s);
    if (rc != RNLA_OK) return rc;
    RNLA_CUDA(cudaMemcpyAsync(x, X.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

// ---- lora_helpers.rs ----
int rnla_orth(const double* x, int64_t m, int64_t n, int64_t ldx, double* q, int64_t ldq) {
    RNLA_API_BEGIN
    check_mat(m, n, ldx);
    const int64_t c = m < n ? m : n;
    if (c == 0) return abi_ok();
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> X((size_t)m * n, s);
    h2d_matrix(X, m, x, ldx, m, n, s);
    DMat Q = orth_of(ctx, X, m, n, m);
    d2h_matrix(q, ldq, Q.p(), m, m, c, s);
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

int rnla_stabilizer(const double* x, int64_t m, int64_t n, int64_t ldx, double* l, int64_t ldl) {
    RNLA_API_BEGIN
    check_mat(m, n, ldx);
    const int64_t c = m < n ? m : n;
    if (c == 0) return abi_ok();
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> X((size_t)m * n, s), L((size_t)m * c, s);
    h2d_matrix(X, m, x, ldx, m, n, s);
    full_piv_lu_l(ctx, X, m, n, m, L, m);
    d2h_matrix(l, ldl, L, m, m, c, s);
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

int rnla_tsog1(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, int32_t num_passes,
               int32_t passes_per_stab, double* sk, int64_t lds, int64_t* cols_out) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m == 0 || n == 0 || k <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "empty input");
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> A((size_t)m * n, s);
    h2d_matrix(A, m, a, lda, m, n, s);
    const bool finite = all_finite(ctx, m, n, A, m);
    DMat S = tsog1_ref(ctx, A, m, n, m, k, num_passes, passes_per_stab, finite);
    d2h_matrix(sk, lds, S.p(), S.rows, S.rows, S.cols, s);
    RNLA_CUDA(cudaStreamSynchronize(s));
    if (cols_out) *cols_out = S.cols;
    RNLA_API_END
}

int rnla_rf1(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double* q, int64_t ldq,
             int64_t* cols_out) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m == 0 || n == 0 || k <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "empty input");
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> A((size_t)m * n, s);
    h2d_matrix(A, m, a, lda, m, n, s);
    const bool finite = all_finite(ctx, m, n, A, m);
    DMat Q = rf1_ref(ctx, A, m, n, m, k, finite);
    d2h_matrix(q, ldq, Q.p(), m, m, Q.cols, s);
    RNLA_CUDA(cudaStreamSynchronize(s));
    if (cols_out) *cols_out = Q.cols;
    RNLA_API_END
}

int rnla_qb1(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double epsilon, double* q,
             int64_t ldq, double* bq, int64_t ldb, int64_t* cols_out) {
    RNLA_API_BEGIN
    (void)epsilon;   // lora_helpers.rs:18
    check_mat(m, n, lda);
    if (m == 0 || n == 0 || k <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "empty input");
    cudaStream_t s = host_stream();
    Ctx ctx(s);
    DevBuf<double> A((size_t)m * n, s);
    h2d_matrix(A, m, a, lda, m, n, s);
    const bool finite = all_finite(ctx, m, n, A, m);
    DMat Q = rf1_ref(ctx, A, m, n, m, k, finite);
    const int64_t c = Q.cols;
    DevBuf<double> B((size_t)c * n, s);
    gemm_f64(ctx, 'T', 'N', c, n, m, 1.0, Q.p(), m, A, m, 0.0, B, c);
    d2h_matrix(q, ldq, Q.p(), m, m, c, s);
    d2h_matrix(bq, ldb, B, c, c, n, s);
    RNLA_CUDA(cudaStreamSynchronize(s));
    if (cols_out) *cols_out = c;
    RNLA_API_END
}

// ---- lora_drivers.rs ----
int rnla_rand_evd1(const double* a, int64_t n, int64_t lda, int64_t k, double epsilon, int64_t s, double* v,
                   int64_t ldv, double* lambda, int64_t* r_out) {
    RNLA_API_BEGIN
    check_mat(n, n, lda);
    if (n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "empty input");
    cudaStream_t st = host_stream();
    Ctx ctx(st);
    const int64_t kk = k > 0 ? k : 1;
    DevBuf<double> A((size_t)n * n, st), V((size_t)n * kk, st);
    h2d_matrix(A, n, a, lda, n, n, st);
    int64_t r = 0;
    rand_evd1_impl(ctx, A, n, n, k, epsilon, s, V, n, lambda, &r);
    d2h_matrix(v, ldv, V, n, n, r, st);
    RNLA_CUDA(cudaStreamSynchronize(st));
    if (r_out) *r_out = r;
    RNLA_API_END
}

int rnla_rand_evd2(const double* a, int64_t n, int64_t lda, int64_t k, int64_t s, double* v, int64_t ldv,
                   double* lambda, int64_t* r_out) {
    RNLA_API_BEGIN
    check_mat(n, n, lda);
    if (n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "empty input");
    cudaStream_t st = host_stream();
    Ctx ctx(st);
    const int64_t kk = k > 0 ? k : 1;
    DevBuf<double> A((size_t)n * n, st), V((size_t)n * kk, st);
    h2d_matrix(A, n, a, lda, n, n, st);
    int64_t r = 0;
    rand_evd2_impl(ctx, A, n, n, k, s, V, n, lambda, &r);
    d2h_matrix(v, ldv, V, n, n, r, st);
    RNLA_CUDA(cudaStreamSynchronize(st));
    if (r_out) *r_out = r;
    RNLA_API_END
}

int64_t rnla_rand_svd_rank(int64_t m, int64_t n, int64_t k, int64_t s, int32_t mode) {
    if (k <= 0 || s < 0 || m <= 0 || n <= 0) return 0;
    int64_t l = k + s;
    int64_t c = m < n ? m : n;
    if (l < c) c = l;
    (void)mode;
    return k < c ? k : c;
}

int rnla_rand_svd_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n, int64_t lda,
                      int64_t k, double epsilon, int64_t s, const rnla_options* opt, double* u_dev,
                      int64_t ldu, double* singular_values_dev, double* vt_dev, int64_t ldvt,
                      int64_t* r_out, rnla_stats* stats, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    Ctx ctx((cudaStream_t)stream);
    const rnla_options o = opts_or_default(opt);
    if (stats) memset(stats, 0, sizeof *stats);
    const int64_t r = rand_svd_impl(ctx, a_dev, a_is_f32 != 0, m, n, lda, k, epsilon, s, o, u_dev, ldu,
                                    singular_values_dev, vt_dev, ldvt, stats);
    if (r_out) *r_out = r;
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_API_END
}

int rnla_rand_svd_ex(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double epsilon,
                     int64_t s, const rnla_options* opt, double* u, int64_t ldu, double* sigma,
                     int64_t lds, double* vt, int64_t ldvt, int64_t* r_out, rnla_stats* stats) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    cudaStream_t st = host_stream();
    Ctx ctx(st);
    const rnla_options o = opts_or_default(opt);
    if (stats) memset(stats, 0, sizeof *stats);
    const int64_t rmax = rnla_rand_svd_rank(m, n, k, s, o.mode);
    DevBuf<double> A((size_t)m * n, st), U((size_t)m * (rmax ? rmax : 1), st),
        Sg(rmax ? rmax : 1, st), Vt((size_t)(rmax ? rmax : 1) * n, st);
    h2d_matrix(A, m, a, lda, m, n, st);
    const int64_t r = rand_svd_impl(ctx, A, false, m, n, m, k, epsilon, s, o, U, m, Sg, Vt,
                                    rmax ? rmax : 1, stats);
    std::vector<double> sg(r > 0 ? r : 1);
    d2h_matrix(u, ldu, U, m, m, r, st);
    d2h_matrix(vt, ldvt, Vt, rmax ? rmax : 1, r, n, st);
    if (r > 0) RNLA_CUDA(cudaMemcpyAsync(sg.data(), Sg.get(), r * sizeof(double), cudaMemcpyDeviceToHost, st));
    RNLA_CUDA(cudaStreamSynchronize(st));
    // S is the r x r diagonal matrix of lora_drivers.rs:64
    for (int64_t j = 0; j < r; ++j)
        for (int64_t i = 0; i < r; ++i) sigma[i + j * lds] = (i == j) ? sg[i] : 0.0;
    if (r_out) *r_out = r;
    RNLA_API_END
}

int rnla_rand_svd(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double epsilon,
                  int64_t s, double* u, int64_t ldu, double* sigma, int64_t lds, double* vt,
                  int64_t ldvt, int64_t* r_out) {
    return rnla_rand_svd_ex(a, m, n, lda, k, epsilon, s, nullptr, u, ldu, sigma, lds, vt, ldvt, r_out,
                            nullptr);
}

// ---- sketch_and_precondition.rs ----
int rnla_blendenpik_overdetermined_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n,
                                       int64_t lda, const double* b_dev, double epsilon, int64_t l,
                                       double sampling_factor, const rnla_options* opt,
                                       double* x_dev, rnla_stats* stats, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    Ctx ctx((cudaStream_t)stream);
    const rnla_options o = opts_or_default(opt);
    if (stats) memset(stats, 0, sizeof *stats);
    blendenpik_impl(ctx, a_dev, a_is_f32 != 0, m, n, lda, b_dev, epsilon, l, sampling_factor, o, x_dev,
                    stats);
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_API_END
}

// Host-pointer blendenpik / lsrn: A goes up in column tiles on the copy
// stream and the solve starts on the first tile while the rest is in flight.
static int blendenpik_host(const void* a, bool a_f32, int64_t m, int64_t n, int64_t lda, const double* b,
                           double epsilon, int64_t l, double sampling_factor, const rnla_options* opt, double* x,
                           rnla_stats* stats, bool lsrn) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    blendenpik_validate(m, n, epsilon, l, sampling_factor);
    cudaStream_t s = host_stream();
    const size_t es = a_f32 ? sizeof(float) : sizeof(double);
    DevBuf<unsigned char> A((size_t)m * n * es, s);
    DevBuf<double> B(m, s), X(n, s);
    RNLA_CUDA(cudaMemcpyAsync(B.get(), b, m * sizeof(double), cudaMemcpyHostToDevice, s));
    ColumnFeed feed;
    h2d_columns_async(A.get(), a, es, m, n, lda, TC_TILE_COLS, s, feed);
    Ctx ctx(s);
    const rnla_options o = opts_or_default(opt);
    if (stats) memset(stats, 0, sizeof *stats);
    blendenpik_impl(ctx, A.get(), a_f32, m, n, m, B, epsilon, l, sampling_factor, o, X, stats, &feed, lsrn);
    RNLA_CUDA(cudaMemcpyAsync(x, X.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

int rnla_blendenpik_overdetermined_ex(const double* a, int64_t m, int64_t n, int64_t lda,
                                      const double* b, double epsilon, int64_t l,
                                      double sampling_factor, const rnla_options* opt, double* x,
                                      rnla_stats* stats) {
    return blendenpik_host(a, false, m, n, lda, b, epsilon, l, sampling_factor, opt, x, stats, false);
}

int rnla_blendenpik_overdetermined_f32_ex(const float* a, int64_t m, int64_t n, int64_t lda,
                                          const double* b, double epsilon, int64_t l,
                                          double sampling_factor, const rnla_options* opt, double* x,
                                          rnla_stats* stats) {
    return blendenpik_host(a, true, m, n, lda, b, epsilon, l, sampling_factor, opt, x, stats, false);
}

int rnla_blendenpik_overdetermined(const double* a, int64_t m, int64_t n, int64_t lda, const double* b,
                                   double epsilon, int64_t l, double sampling_factor, double* x) {
    return rnla_blendenpik_overdetermined_ex(a, m, n, lda, b, epsilon, l, sampling_factor, nullptr, x,
                                             nullptr);
}

int rnla_lsrn_overdetermined_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n, int64_t lda,
                                 const double* b_dev, double epsilon, int64_t l, double sampling_factor,
                                 const rnla_options* opt, double* x_dev, rnla_stats* stats, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    Ctx ctx((cudaStream_t)stream);
    const rnla_options o = opts_or_default(opt);
    if (stats) memset(stats, 0, sizeof *stats);
    blendenpik_impl(ctx, a_dev, a_is_f32 != 0, m, n, lda, b_dev, epsilon, l, sampling_factor, o, x_dev,
                    stats, nullptr, true);
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_API_END
}

// Every problem goes through the single-problem pipeline on one of the
// workers' streams (grids sized for that worker's share of the SMs), so x
// matches its own _dev call to the solver's accuracy, not bit for bit.  A
// failing problem (bad shape, singular sketch, a device wait that gave up)
// is recorded and the batch goes on; a CUDA error ends it.
int rnla_solve_batched(const rnla_ls_problem* probs, int64_t count, double epsilon, int64_t l,
                       double sampling_factor, const rnla_options* opt, int32_t* status_out,
                       rnla_stats* stats_out, void* stream) {
    if (count < 0) return abi_error(RNLA_ERR_NEGATIVE_DIMENSIONS, "count must be non-negative");
    if (count > 0 && (!probs || !status_out))
        return abi_error(RNLA_ERR_INVALID_PARAMETERS, "probs and status_out are required");
    if (count == 0) return abi_ok();
    rnla_options o;
    int dev = 0, sms = 0;
    try {
        o = opts_or_default(opt);
        RNLA_CUDA(cudaGetDevice(&dev));
        RNLA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    } catch (const Error& e) {
        return abi_error(e.code, e.what());
    }
    // Small problems leave most of the GPU idle (their QR and LSQR are chains
    // of grid barriers and cross-SM hand-offs), so the batch runs as W
    // workers, each a host thread with its own main and side streams and grids
    // sized for sms / W SMs, taking the next problem from a shared counter.
    const int W = (int)std::min<int64_t>(count, batched_workers());
    std::vector<cudaStream_t> main_s(W), side_s(W);
    cudaEvent_t inputs = nullptr;
    try {
        for (int w = 0; w < W; ++w) {
            main_s[w] = worker_stream(dev, 2 * w);
            side_s[w] = worker_stream(dev, 2 * w + 1);
        }
        // the problems' data were written on the caller's stream
        RNLA_CUDA(cudaEventCreateWithFlags(&inputs, cudaEventDisableTiming));
        RNLA_CUDA(cudaEventRecord(inputs, (cudaStream_t)stream));
        for (int w = 0; w < W; ++w) RNLA_CUDA(cudaStreamWaitEvent(main_s[w], inputs, 0));
        RNLA_CUDA(cudaEventDestroy(inputs));
    } catch (const Error& e) {
        return abi_error(e.code, e.what());
    }
    std::atomic<int64_t> next{0};
    std::atomic<bool> dead{false};
    std::mutex mu;
    int first = RNLA_OK;
    int64_t first_p = -1;
    std::string first_msg;
    auto work = [&](int w) {
        cudaSetDevice(dev);
        for (;;) {
            const int64_t p = next.fetch_add(1);
            if (p >= count) break;
            if (dead.load()) {
                status_out[p] = RNLA_ERR_CUDA;
                continue;
            }
            const rnla_ls_problem& q = probs[p];
            rnla_stats* st = stats_out ? stats_out + p : nullptr;
            if (st) memset(st, 0, sizeof *st);
            int rc = RNLA_OK;
            std::string msg;
            try {
                check_mat(q.m, q.n, q.lda);
                if (!q.a || !q.b || !q.x) fail(RNLA_ERR_INVALID_PARAMETERS, "problem with a null pointer");
                Ctx ctx(main_s[w]);
                ctx.side = side_s[w];
                ctx.sm_count = std::max(1, sms / W);
                blendenpik_impl(ctx, q.a, q.a_is_f32 != 0, q.m, q.n, q.lda, q.b, epsilon, l, sampling_factor, o,
                                q.x, st);
            } catch (const Error& e) {
                rc = e.code;
                msg = e.what();
            } catch (const std::bad_alloc&) {
                rc = RNLA_ERR_COMPUTATION;
                msg = "host allocation failed";
            }
            status_out[p] = rc;
            if (rc != RNLA_OK) {
                std::lock_guard<std::mutex> g(mu);
                if (first_p < 0 || p < first_p) {
                    first = rc;
                    first_p = p;
                    first_msg = "problem " + std::to_string(p) + ": " + msg;
                }
                if (rc == RNLA_ERR_CUDA) dead.store(true);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < W; ++w) pool.emplace_back(work, w);
    work(0);
    for (auto& t : pool) t.join();
    for (int w = 0; w < W; ++w) {
        const cudaError_t e = cudaStreamSynchronize(main_s[w]);
        if (e != cudaSuccess) return abi_error(RNLA_ERR_CUDA, cudaGetErrorString(e));
    }
    const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return abi_error(RNLA_ERR_CUDA, cudaGetErrorString(e));
    return first == RNLA_OK ? abi_ok() : abi_error(first, first_msg.c_str());
}

int rnla_lsrn_overdetermined_ex(const double* a, int64_t m, int64_t n, int64_t lda, const double* b,
                                double epsilon, int64_t l, double sampling_factor, const rnla_options* opt,
                                double* x, rnla_stats* stats) {
    return blendenpik_host(a, false, m, n, lda, b, epsilon, l, sampling_factor, opt, x, stats, true);
}

int rnla_lsrn_overdetermined(const double* a, int64_t m, int64_t n, int64_t lda, const double* b,
                             double epsilon, int64_t l, double sampling_factor, double* x) {
    return rnla_lsrn_overdetermined_ex(a, m, n, lda, b, epsilon, l, sampling_factor, nullptr, x, nullptr);
}

int rnla_sketched_least_squares_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n, int64_t lda,
                                    const double* b_dev, int32_t use_svd, const rnla_options* opt,
                                    double* x_dev, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    Ctx ctx((cudaStream_t)stream);
    const rnla_options o = opts_or_default(opt);
    sketch_solve_impl(ctx, a_dev, a_is_f32 != 0, m, n, lda, b_dev, use_svd != 0, o, x_dev, nullptr);
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_API_END
}

int rnla_sap_chol_qrcp_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda, int64_t d,
                           const rnla_options* opt, double* q_dev, int64_t ldq, double* r_dev, int64_t ldr,
                           int64_t* jpvt_dev, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    check_mat(m, n, ldq);
    check_mat(n, n, ldr);
    Ctx ctx((cudaStream_t)stream);
    const rnla_options o = opts_or_default(opt);
    sap_chol_qrcp(ctx, key_of(&o.rng), o.precision, o.digits_a, a_dev, m, n, lda, d, q_dev, ldq, r_dev, ldr,
                  jpvt_dev);
    RNLA_CUDA(cudaStreamSynchronize(ctx.stream));
    RNLA_API_END
}

int rnla_sap_chol_qrcp(const double* a, int64_t m, int64_t n, int64_t lda, int64_t d, const rnla_options* opt,
                       double* q, int64_t ldq, double* r, int64_t ldr, int64_t* jpvt) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    check_mat(m, n, ldq);
    check_mat(n, n, ldr);
    cudaStream_t s = host_stream();
    DevBuf<double> A((size_t)m * n, s), Q((size_t)m * n, s), R((size_t)n * n, s);
    DevBuf<int64_t> J(n, s);
    h2d_matrix(A, m, a, lda, m, n, s);
    Ctx ctx(s);
    const rnla_options o = opts_or_default(opt);
    sap_chol_qrcp(ctx, key_of(&o.rng), o.precision, o.digits_a, A, m, n, m, d, Q, m, R, n, J);
    d2h_matrix(q, ldq, Q, m, m, n, s);
    d2h_matrix(r, ldr, R, n, n, n, s);
    RNLA_CUDA(cudaMemcpyAsync(jpvt, J.get(), n * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

static int sketched_ls_host(const double* a, int64_t m, int64_t n, int64_t lda, const double* b, bool use_svd,
                            const rnla_options* opt, double* x) {
    RNLA_API_BEGIN
    check_mat(m, n, lda);
    if (m <= 0 || n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "A must be non-empty");
    cudaStream_t s = host_stream();
    DevBuf<double> A((size_t)m * n, s), B(m, s), X(n, s);
    RNLA_CUDA(cudaMemcpyAsync(B.get(), b, m * sizeof(double), cudaMemcpyHostToDevice, s));
    ColumnFeed feed;
    h2d_columns_async(A.get(), a, sizeof(double), m, n, lda, TC_TILE_COLS, s, feed);
    Ctx ctx(s);
    const rnla_options o = opts_or_default(opt);
    sketch_solve_impl(ctx, A.get(), false, m, n, m, B, use_svd, o, X, &feed);
    RNLA_CUDA(cudaMemcpyAsync(x, X.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    RNLA_CUDA(cudaStreamSynchronize(s));
    RNLA_API_END
}

int rnla_sketched_least_squares_qr(const double* a, int64_t m, int64_t n, int64_t lda, const double* b,
                                   const rnla_options* opt, double* x) {
    return sketched_ls_host(a, m, n, lda, b, false, opt, x);
}

int rnla_sketched_least_squares_svd(const double* a, int64_t m, int64_t n, int64_t lda, const double* b,
                                    const rnla_options* opt, double* x) {
    return sketched_ls_host(a, m, n, lda, b, true, opt, x);
}

// ---- building blocks ----
int rnla_sketch_apply_ex_dev(const void* x_dev, int32_t x_is_f32, int64_t m, int64_t n, int64_t ldx,
                             int64_t d, int32_t dist, const rnla_rng* rng, int32_t precision, int32_t digits,
                             double* y_dev, int64_t ldy, void* stream) {
    RNLA_API_BEGIN
    check_mat(m, n, ldx);
    if (d <= 0 || m <= 0 || n <= 0) fail(RNLA_ERR_INVALID_DIMENSIONS, "empty sketch product");
    if (dist != RNLA_GAUSSIAN && dist != RNLA_UNIFORM && dist != RNLA_RADEMACHER)
        fail(RNLA_ERR_INVALID_PARAMETERS, "unknown distribution");
    int32_t unused = 0;
    resolve_precision(precision, digits, unused);
    Ctx ctx((cudaStream_t)stream);
    const RngKey key = key_of(rng);
    if (precision == RNLA_PREC_FP64) {
        DevBuf<double> S((size_t)d * m, ctx.stream);
        sketch_fill_f64(ctx, dist, key, d, m, S, d);
        DevBuf<double> Xw;
        const double* X = static_cast<const double*>(x_dev);
        int64_t ld = ldx;
        if (x_is_f32) {
            Xw.alloc((size_t)m * n, ctx.stream);
            copy_matrix_f32_to_f64(ctx, m, n, static_cast<const float*>(x_dev), ldx, Xw, m);
            X = Xw.get();
            ld = m;
        }
        gemm_f64(ctx, 'N', 'N', d, n, m, 1.0, S, d, X, ld, 0.0, y_dev, ldy);
    } else {
        if (!tc_available(ctx)) fail(RNLA_ERR_UNSUPPORTED, "sm_103a tensor-core kernels unavailable");
        tc_sketch_apply(ctx, key, x_dev, x_is_f32 != 0, m, n, ldx, nullptr, d, digits, y_dev, ldy, nullptr, dist);
    }
    RNLA_API_END
}

int rnla_sketch_apply_dev(const void* x_dev, int32_t x_is_f32, int64_t m, int64_t n, int64_t ldx,
                          int64_t d, const rnla_rng* rng, int32_t precision, int32_t digits,
                          double* y_dev, int64_t ldy, void* stream) {
    return rnla_sketch_apply_ex_dev(x_dev, x_is_f32, m, n, ldx, d, RNLA_GAUSSIAN, rng, precision, digits, y_dev,
                                    ldy, stream);
}

int rnla_gemm_tn_dev(const double* x_dev, int64_t k, int64_t mm, int64_t ldx, const double* y_dev,
                     int64_t nn, int64_t ldy, int32_t precision, int32_t digits_x, int32_t digits_y,
                     double* c_dev, int64_t ldc, void* stream) {
    RNLA_API_BEGIN
    check_mat(k, mm, ldx);
    check_mat(k, nn, ldy);
    resolve_precision(precision, digits_x, digits_y);
    Ctx ctx((cudaStream_t)stream);
    if (precision != RNLA_PREC_FP64 && !tc_available(ctx))
        fail(RNLA_ERR_UNSUPPORTED, "sm_103a tensor-core kernels unavailable");
    product_tn(ctx, precision, x_dev, k, mm, ldx, y_dev, nn, ldy, digits_x, digits_y, c_dev, ldc);
    RNLA_API_END
}

}  // extern "C"
