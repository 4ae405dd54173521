// Internal interfaces between the translation units of librandnla_gb300.
// Everything here works on device pointers, column-major storage, and is
// enqueued on ctx.stream.
#pragma once
#include <functional>
#include <vector>
#include "rnla_common.cuh"
#include "rnla_rng.cuh"

namespace rnla {

// ---- generators (rng.cu) ----
void rng_words(Ctx& ctx, const RngKey& key, uint64_t first_word, int64_t n, uint32_t* out);
void sketch_fill_f64(Ctx& ctx, int dist, const RngKey& key, int64_t rows, int64_t cols,
                     double* out, int64_t ld);
void sketch_fill_f32(Ctx& ctx, int dist, const RngKey& key, int64_t rows, int64_t cols,
                     bool quantized, float* out, int64_t ld);

// ---- dense FP64 kernels (dense.cu) ----
// C = alpha op(A) op(B) + beta C, op(X) = X ('N') or X^T ('T'); M x N result.
void gemm_f64(Ctx& ctx, char ta, char tb, int64_t M, int64_t N, int64_t K, double alpha,
              const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
              double* C, int64_t ldc);
void copy_matrix(Ctx& ctx, int64_t rows, int64_t cols, const double* src, int64_t lds,
                 double* dst, int64_t ldd);
void copy_matrix_f32_to_f64(Ctx& ctx, int64_t rows, int64_t cols, const float* src, int64_t lds,
                            double* dst, int64_t ldd);
// dst (cols x rows) = src^T
void transpose(Ctx& ctx, int64_t rows, int64_t cols, const double* src, int64_t lds, double* dst,
               int64_t ldd);
void fill_identity(Ctx& ctx, int64_t rows, int64_t cols, double* dst, int64_t ld);
void fill_zero(Ctx& ctx, int64_t rows, int64_t cols, double* dst, int64_t ld);
// returns false if any entry is NaN or infinite (synchronises)
bool all_finite(Ctx& ctx, int64_t rows, int64_t cols, const double* a, int64_t lda);

// ---- factorizations (factor.cu) ----
// Householder QR of the first n columns of X (m x nc, m >= n), LAPACK
// convention (tau = 0 when the sub-column is zero).  R in the upper
// triangle, reflectors below; columns n..nc-1 receive Q^T.  tau: n values.
void householder_qr(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld, double* tau);
// Thin Q (m x n) from the reflectors stored in V (m x n, ld) and tau.
void householder_form_q(Ctx& ctx, const double* V, int64_t m, int64_t n, int64_t ldv,
                        const double* tau, double* Q, int64_t ldq);
// Float-float Householder QR (qr_ff.cu): R in the upper triangle of X and
// Q^T applied to columns n..nc-1 (reflectors are not kept); the same
// contract as householder_qr without tau.  Supported when the column blocks
// fit in shared memory.
bool qr_ff_supported(const Ctx& ctx, int64_t m, int64_t n, int64_t nc);
void householder_qr_ff(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld);
// The same for sketches too tall for one factorization: two row halves, then
// their stacked R blocks (two-level TSQR); only the first n rows of X are
// meaningful afterwards.
bool qr_ff_tsqr_supported(const Ctx& ctx, int64_t m, int64_t n, int64_t nc);
void householder_qr_ff_tsqr(Ctx& ctx, double* X, int64_t m, int64_t n, int64_t nc, int64_t ld);
// Float-float R^-1 (qr_ff.cu); false on an exactly zero pivot (synchronises).
bool upper_inverse_ff(Ctx& ctx, const double* R, int64_t n, int64_t ldr, double* Rinv, int64_t ldi);
// Rinv (n x n, upper) = R^-1; returns false on an exactly zero pivot (synchronises).
bool upper_inverse(Ctx& ctx, const double* R, int64_t n, int64_t ldr, double* Rinv, int64_t ldi);
// back substitution with the reference's zero-pivot rule (solvers.rs:22-41)
void upper_solve_skip_zero(Ctx& ctx, const double* U, int64_t n, int64_t ldu, const double* y,
                           double* x);
// Cholesky G = R^T R (upper R written to the upper triangle of G, n x n);
// returns false if a pivot is not positive (synchronises).
bool cholesky_upper(Ctx& ctx, double* G, int64_t n, int64_t ld, int64_t npd = -1);
// The same factorization in float-float (chol_ff.cu) for the tensor-core
// paths, whose Grams carry ~2^-48 themselves.
bool cholesky_upper_ff(Ctx& ctx, double* G, int64_t n, int64_t ld, int64_t npd = -1);
// Thin orthonormal basis of Y (m x n, m >= n) in place: CholeskyQR2, with a
// Householder fallback when a Cholesky pivot fails.  Returns 1 if the
// fallback was taken.
int orthonormalize(Ctx& ctx, double* Y, int64_t m, int64_t n, int64_t ld, bool force_householder);
// Unit-lower L (m x min(m,n)) of complete-pivoting LU, without P.
void full_piv_lu_l(Ctx& ctx, const double* X, int64_t m, int64_t n, int64_t ldx, double* L,
                   int64_t ldl);
// Thin SVD of B (p x q): U (p x t), sigma (t), V (q x t), t = min(p, q),
// singular values descending; exactly-zero singular directions get the
// first unused coordinate vectors (so SVD(0) = (I, 0, I)).
// One-sided Jacobi of W (s x s), rotations accumulated into V (one CTA for
// s < 64, a cooperative grid above).
void jacobi_sweeps(Ctx& ctx, double* W, double* V, int64_t s, unsigned int* sweeps_dev = nullptr);
// SVD of a wide B (p <= q) through chol(B B^T) with a float-float Gram:
// U_B (p x p), sigma (p), V_B (q x p).  Returns false (caller uses
// small_svd) when the Cholesky fails or sigma_p / sigma_1 < 1e-5.
bool small_svd_gram(Ctx& ctx, const double* B, int64_t p, int64_t q, int64_t ldb, double* U, int64_t ldu,
                    double* sigma, double* V, int64_t ldv, int* sweeps = nullptr);
// Eigenvectors of the p x p SPD G (2 <= p <= 320) with R = chol(G): FP32
// cluster Jacobi on R^T, float-float Rayleigh-Ritz refinement (eig_refine.cu).
// UB (ld ldu) and sigma = sqrt(eigenvalues) in descending order; false when
// the refinement does not converge (nothing kept).
bool eig_gram_refined(Ctx& ctx, const double* G, const double* R, int64_t p, double* UB, int64_t ldu, double* sigma,
                      int* sweeps);
void small_svd(Ctx& ctx, const double* B, int64_t p, int64_t q, int64_t ldb, double* U,
               int64_t ldu, double* sigma, double* V, int64_t ldv);

// ---- pivoted QR and CQRRPT (cqrrpt.cu) ----
// Column-pivoted Householder QR of R (d x n, in place), the reference's
// greedy largest-remaining-norm rule; jpvt (device, n) receives the order.
void qrcp(Ctx& ctx, double* R, int64_t d, int64_t n, int64_t ld, int64_t* jpvt);
// cqrrpt.rs:27-58 on device data: Q (m x n), R (n x n), jpvt (device, n).
void sap_chol_qrcp(Ctx& ctx, const RngKey& key, int precision, int digits, const double* A, int64_t m,
                   int64_t n, int64_t lda, int64_t d, double* Q, int64_t ldq, double* R, int64_t ldr,
                   int64_t* jpvt_dev);

// ---- iterative solvers (iterative.cu) ----
struct LsqrParams {
    double damp = 0.0, atol = 1e-8, btol = 1e-8, conlim = 1e8;
    int64_t iter_lim = -1;
    bool calc_var = false;
    double abs_arnorm_tol = 0.0;   // > 0: also stop when the ||A^T r|| estimate < this (CGLS rule)
};
struct LsqrResult {
    int64_t istop = 0, itn = 0;
    double r1norm = 0, r2norm = 0, anorm = 0, acond = 0, xnorm = 0, arnorm = 0;
    double ms_kernel = 0;   // device time of the persistent kernel
};
// Result of a solve enqueued without a host synchronisation: the solver's
// scalars land in pinned host memory and are read by resolve() once the
// caller has synchronised the stream.
struct LsqrPending {
    double* host = nullptr;                 // 8 values (pinned, per thread)
    cudaEvent_t ev[2] = {nullptr, nullptr}; // around the kernel
    bool armed = false;
    LsqrPending() = default;
    LsqrPending(const LsqrPending&) = delete;
    LsqrPending& operator=(const LsqrPending&) = delete;
    ~LsqrPending() {
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
    void resolve(LsqrResult& r) const;
};
// LSQR on the operator A M (M upper-triangular n x n, or identity if
// Minv_rowmajor == nullptr).  A is double (a64) or float (a32), m x n, lda.
// x0 nullable; x receives z (the solution of the preconditioned problem,
// i.e. the caller applies M afterwards).  arnorms_dev nullable (iter_lim values).
struct LsqrFFInput;
LsqrResult lsqr_solve(Ctx& ctx, const double* a64, const float* a32, int64_t m, int64_t n,
                      int64_t lda, const double* M, const double* b, const double* x0,
                      const LsqrParams& prm, double* x, double* var, double* arnorms_dev,
                      bool ffp, const LsqrFFInput* pre = nullptr, LsqrPending* pend = nullptr);
// CGLS (cg.rs:18-61) on A M, same conventions; returns iterations used.
int64_t cgls_solve(Ctx& ctx, const double* a64, const float* a32, int64_t m, int64_t n,
                   int64_t lda, const double* M, const double* b, const double* x0,
                   double tolerance, int64_t num_iterations, double* x, bool* converged);
// Float-float LSQR (lsqr_ff.cu) on FP64 or FP32 data, 1 <= n <= 1024; same contract
// as lsqr_solve.  lsqr_ff_prepare builds the solver's copies of A and b on
// the side stream (so they overlap later work on ctx.stream); lsqr_ff_alloc
// + lsqr_ff_build do the same in two steps, the build on a stream of the
// caller's choosing; lsqr_ff_solve waits for them (or builds them itself
// when `pre` is null).
struct LsqrFFInput {
    DevBuf<float2> AF, bF;
    const void* A = nullptr;
    bool f32 = false;               // AF holds FP32 rows (A stored in FP32)
    int64_t m = 0, n = 0, ldf = 0;
    cudaEvent_t ready = nullptr;
    cudaStream_t owner = nullptr;   // stream the buffers are freed on
    LsqrFFInput() = default;
    LsqrFFInput(const LsqrFFInput&) = delete;
    LsqrFFInput& operator=(const LsqrFFInput&) = delete;
    // the buffers are released only after the side-stream copies (an early
    // error return must not free memory still being written)
    ~LsqrFFInput() {
        if (ready) {
            cudaStreamWaitEvent(owner, ready, 0);
            cudaEventDestroy(ready);
        }
    }
};
bool lsqr_ff_supported(int64_t n);
// M (n x n upper) <- the FP64 value of its float-float split, so that the
// float-float LSQR operator A M and a later FP64 product M z use the same M.
void ff_round_upper(Ctx& ctx, double* M, int64_t n, int64_t ldm);
void lsqr_ff_prepare(Ctx& ctx, const void* A, bool a_f32, int64_t m, int64_t n, int64_t lda, const double* b,
                     LsqrFFInput& in);
// Allocates the copies on ctx.stream (no kernels).
void lsqr_ff_alloc(Ctx& ctx, const void* A, bool a_f32, int64_t m, int64_t n, LsqrFFInput& in);
// Builds them on `st`, which the caller has ordered after the allocation and
// after A and b are written; a_done: the copy of A is already written
// (tc_sketch_apply's rm), only b's is built.
void lsqr_ff_build(Ctx& ctx, LsqrFFInput& in, int64_t lda, const double* b, cudaStream_t st,
                   bool a_done = false);
LsqrResult lsqr_ff_solve(Ctx& ctx, const void* A, bool a_f32, int64_t m, int64_t n, int64_t lda, const double* M,
                         const double* b, const double* x0, const LsqrParams& prm, double* x, double* var,
                         double* arnorms_dev, const LsqrFFInput* pre = nullptr, LsqrPending* pend = nullptr);
// Workspace-based LSQR used by the allocation-free entry point (noalloc.cu).
size_t lsqr_workspace_bytes(int64_t m, int64_t n, int sm_count, int* grid, size_t* smem,
                            const void** kernel);
LsqrResult lsqr_run_in_workspace(cudaStream_t stream, int sm_count, void* ws, size_t ws_bytes,
                                 const double* a64, int64_t m, int64_t n, int64_t lda, const double* b,
                                 const double* x0, const LsqrParams& prm, double* x);
// y = M x for upper-triangular M (n x n)
void trmv_upper(Ctx& ctx, const double* M, int64_t n, int64_t ldm, const double* x, double* y);

// ---- tensor-core digit-sliced products (sketch_tc.cu) ----
// Returns true if the sm_103a tensor-core kernels are usable on this device.
// A matrix arriving from the host in chunks of `cols` columns: chunk c is
// on the device once `ready[c]` (recorded on the copy stream) has fired.
struct ColumnFeed {
    int64_t cols = 0;
    std::vector<cudaEvent_t> ready;
    cudaStream_t owner = nullptr;   // stream that frees the destination buffer
    ColumnFeed() = default;
    ColumnFeed(const ColumnFeed&) = delete;
    ColumnFeed& operator=(const ColumnFeed&) = delete;
    // the owner stream waits for every copy before the destination can be
    // freed (an early error return must not free memory still being written)
    ~ColumnFeed() {
        for (cudaEvent_t e : ready) {
            if (owner) cudaStreamWaitEvent(owner, e, 0);
            cudaEventDestroy(e);
        }
    }
    // `s` waits for the chunks holding columns [j0, j1)
    void wait_cols(cudaStream_t s, int64_t j0, int64_t j1) const {
        if (j1 <= j0 || cols <= 0) return;
        const int64_t c1 = (j1 - 1) / cols;
        for (int64_t c = j0 / cols; c <= c1 && c < (int64_t)ready.size(); ++c)
            RNLA_CUDA(cudaStreamWaitEvent(s, ready[(size_t)c], 0));
    }
    void wait_all(cudaStream_t s) const {
        for (cudaEvent_t e : ready) RNLA_CUDA(cudaStreamWaitEvent(s, e, 0));
    }
};
// Copies the host matrix a (m x n, lda, elements of esize bytes) to dev (ld
// m) in column chunks on the device's copy stream, after the work already
// enqueued on `s`.
void h2d_columns_async(void* dev, const void* a, size_t esize, int64_t m, int64_t n, int64_t lda, int64_t chunk,
                       cudaStream_t s, ColumnFeed& feed);

bool tc_available(Ctx& ctx);
// C (M x N', ldc, FP64) = S [X extra] where S (M x K) is the quantised
// Gaussian sketch of `key` (entry (i,k) = word i + k*round_up(M,4)), X (K x N)
// and the optional double column `extra` (K values) appended as column N.
// With a feed, X arrives from the host in column chunks and each column tile
// of the product is started as soon as its columns are on the device.
// before_mma: the caller's work on the main stream ahead of the MMA (after
// the digit planes); rm: for FP32 X, a row-major FP32 copy of X (rows of
// rm.ld floats, zero from column N on) written by the digit-plane kernel
// from the same reads.
struct SketchRowMajor {
    float* dst = nullptr;
    int64_t ld = 0;
};
void tc_sketch_apply(Ctx& ctx, const RngKey& key, const void* X, bool x_f32, int64_t K, int64_t N,
                     int64_t ldx, const double* extra, int64_t M, int digits, double* C, int64_t ldc,
                     const ColumnFeed* feed = nullptr, int dist = DIST_GAUSSIAN,
                     const std::function<void(cudaStream_t)>& before_mma = {}, const SketchRowMajor& rm = {});
// Columns per host-to-device copy of the host-buffer entry points (the
// tensor-core sketch starts each column tile once its chunks have landed);
// also the width of the 64-column digit tiles.
constexpr int64_t TC_TILE_COLS = 64;
// ---- float-float tall-skinny products (gram_ff.cu) ----
// C (N1 x N2, FP64, ldc) = X^T Y for column-major FP64 X (K x N1, ldx) and
// Y (K x N2, ldy), accumulated in float-float (~48 bits) on the FP32 pipe.
void gram_ff(Ctx& ctx, const double* X, int64_t ldx, int64_t N1, const double* Y, int64_t ldy, int64_t N2,
             int64_t K, double* C, int64_t ldc);

// ---- split-bf16 tensor-core GEMM (gemm_bfx.cu) ----
// An operand as bf16 planes (X = X_0 + X_1 + ..., each the bf16 rounding of
// the remainder) in K-major SWIZZLE_128B tiles of TR rows x 64 K.
struct BfxPlanes {
    DevBuf<uint8_t> buf;
    int64_t R = 0, K = 0;
    int TR = 0, planes = 0, tiles = 0, Ks = 0;
};
// Tile height an operand image needs: 128 on the X (M) side; on the Y (N)
// side 96 for level 2 and 64 for level 3.
int bfx_tile_rows(int level, bool x_side);
// Element (r, k) of the operand (R x K) is src[r sr + k sk] (FP32 or FP64).
void bfx_planes(Ctx& ctx, BfxPlanes& P, const void* src, bool f32, int64_t R, int64_t K, int64_t sr, int64_t sk,
                int TR, int planes);
// C (X.R x Y.R, FP64, ldc) = X^T Y keeping the plane pairs p + q < level
// (2 or 3); trans stores C^T instead (C[j + i ldc]).
void bfx_gemm(Ctx& ctx, int level, const BfxPlanes& X, const BfxPlanes& Y, double* C, int64_t ldc, bool trans);

// C (MM x NN, FP64; C^T into ldc when trans) = X^T Y with exact tensor-core
// products: X (K x MM, FP32 or FP64) in xd signed 6-bit digits below each
// column's maximum, Y (K x NN, FP64) in four 8-bit digits (sketch_tc.cu).
void tc_exact_tn(Ctx& ctx, const void* X, bool x_f32, int64_t K, int64_t MM, int64_t ldx, const double* Y,
                 int64_t NN, int64_t ldy, double* C, int64_t ldc, bool trans, int xd = 4);
// C (MM x NN) = X^T Y, X (K x MM), Y (K x NN), all double.
void tc_gemm_tn(Ctx& ctx, const double* X, int64_t K, int64_t MM, int64_t ldx, const double* Y,
                int64_t NN, int64_t ldy, int dx, int dy, double* C, int64_t ldc);

}  // namespace rnla
