/*
 * librandnla_gb300 — C ABI of the GB300 (sm_103a) implementation of the
 * randomized linear-algebra hot path of the Rust crate `randblas`
 * (divijkhaitan/randnla): dense sketch operators, the rand_svd range finder
 * with its small-SVD finish, and the sketch-and-precondition overdetermined
 * least-squares solver with its CGLS / LSQR inner solvers.
 *
 * Conventions (the reference's nalgebra DMatrix layout):
 *   - matrices are column-major with an explicit leading dimension (ld >= rows);
 *   - functions without a suffix take HOST pointers, copy to the GPU, compute
 *     there and copy results back before returning (synchronous, like the
 *     reference's pure functions);
 *   - `_dev` functions take DEVICE pointers and a cudaStream_t (passed as
 *     void*); they are stream-ordered and return once the work is enqueued,
 *     except where a host-visible result (a rank, an iteration count) forces
 *     a synchronisation, which each declaration states;
 *   - the return value is an rnla_status; 0 is success and 1..10 are the
 *     variants of the reference's RandNLAError in declaration order
 *     (src/errors.rs:3-14).  rnla_last_error_message() returns the message
 *     payload of the last failure on the calling thread;
 *   - nothing is printed.  The reference prints progress lines
 *     (src/lora_drivers.rs:47, src/cg.rs:47,58); this library returns the same
 *     facts in rnla_stats instead.
 * Every computation runs on the GPU; there is no CPU fallback.  When no CUDA
 * device is usable every compute entry point returns RNLA_ERR_CUDA.
 */
#ifndef RANDNLA_GB300_H
#define RANDNLA_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define RNLA_API __attribute__((visibility("default")))
#else
#define RNLA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: src/errors.rs:3-14, then library-specific codes ---- */
typedef enum {
    RNLA_OK = 0,
    RNLA_ERR_INVALID_PARAMETERS = 1,        /* RandNLAError::InvalidParameters */
    RNLA_ERR_INVALID_DIMENSIONS = 2,        /* RandNLAError::InvalidDimensions */
    RNLA_ERR_NEGATIVE_DIMENSIONS = 3,       /* RandNLAError::NegativeDimensions */
    RNLA_ERR_NOT_OVERDETERMINED = 4,        /* RandNLAError::NotOverdetermined */
    RNLA_ERR_NOT_SQUARE = 5,                /* RandNLAError::NotSquare */
    RNLA_ERR_SINGULAR_MATRIX = 6,           /* RandNLAError::SingularMatrix */
    RNLA_ERR_MATRIX_DECOMPOSITION = 7,      /* RandNLAError::MatrixDecompositionError */
    RNLA_ERR_NOT_HERMITIAN = 8,             /* RandNLAError::NotHermitian */
    RNLA_ERR_NOT_POSITIVE_SEMIDEFINITE = 9, /* RandNLAError::NotPositiveSemiDefinite */
    RNLA_ERR_COMPUTATION = 10,              /* RandNLAError::ComputationError */
    RNLA_ERR_CUDA = 11,                     /* CUDA runtime / launch failure */
    RNLA_ERR_TIMEOUT = 12,                  /* a bounded device-side wait gave up */
    RNLA_ERR_UNSUPPORTED = 13               /* option combination not built */
} rnla_status;

/* Thread-local message of the last non-zero status (empty string if none). */
RNLA_API const char* rnla_last_error_message(void);
/* Library version string, e.g. "0.1.0 sm_103a". */
RNLA_API const char* rnla_version(void);
/* Number of usable CUDA devices (0 on a machine without a GPU; no error). */
RNLA_API int rnla_device_count(void);
/* Number of kernels this library has launched in the process so far (a
 * diagnostic counter; bench.py reports launches inside its timed region). */
RNLA_API uint64_t rnla_kernel_launches(void);
/* Scratch memory comes from one stream-ordered pool per device that keeps
 * freed blocks for the next call (no context handle to create or destroy).
 * This returns the blocks no call is using to the driver; call it when the
 * library is idle.  A no-op before the first GPU call. */
RNLA_API int rnla_release_cached_memory(void);
/* Bounded-wait self-check (no counterpart in the reference).  Every device
 * wait of the library (grid barriers of the persistent solvers, mbarrier
 * phases of the bulk-copy rings) gives up after a time limit and reports
 * RNLA_ERR_TIMEOUT instead of hanging.  This runs one such wait that cannot
 * complete -- which = 0: a grid barrier over every SM whose arrival count
 * never reaches the grid size; which = 1: an mbarrier phase that receives
 * one of two arrivals -- with a limit of limit_us (1 .. 2e6) microseconds,
 * and returns RNLA_ERR_TIMEOUT when the wait expired as designed.  The CUDA
 * context stays usable.  Synchronises. */
RNLA_API int rnla_check_bounded_wait(int32_t which, int64_t limit_us, void* stream);

/* ---- sketch distributions: src/sketch.rs:9-13 ---- */
typedef enum { RNLA_GAUSSIAN = 0, RNLA_UNIFORM = 1, RNLA_RADEMACHER = 2 } rnla_distribution;

/* ---- counter-based generators (rust-random123) ---- */
typedef enum {
    RNLA_GEN_PHILOX4X32 = 0,   /* rust-random123/src/philox.rs:81-105,211-223 */
    RNLA_GEN_THREEFRY2X64 = 1  /* rust-random123/src/threefry.rs:6-28,69-93 */
} rnla_generator;

typedef struct {
    int32_t generator;   /* rnla_generator */
    int32_t reserved;
    uint64_t key0;       /* Philox4x32: key = {low 32, high 32} of key0 (philox.rs:101-105) */
    uint64_t key1;       /* ThreeFry2x64: key = {key0, key1} (threefry.rs:23-27) */
} rnla_rng;

/* Word stream of a generator: word t is word (t mod 4) of block floor(t/4),
 * block g being the generator's output at counter value g (128-bit /
 * two-word little-endian counter, philox.rs:87-99, threefry.rs:13-21); a
 * ThreeFry2x64 block contributes low then high halves of its two outputs.
 * Writes n words starting at word index first_word into host memory.
 * Replaces the block streams of Philox4x32Rng / ThreeFry2x64Rng
 * (rust-random123/src/rng.rs:85-96). */
RNLA_API int rnla_rng_words(const rnla_rng* rng, uint64_t first_word, int64_t n, uint32_t* out);
RNLA_API int rnla_rng_words_dev(const rnla_rng* rng, uint64_t first_word, int64_t n, uint32_t* out_dev,
                       void* stream);

/* sketch::sketching_operator (src/sketch.rs:102-130): a dense rows x cols
 * operator with iid entries, written column-major into out (ld >= rows).
 * The reference seeds ThreeFry2x64 with seed_from_u64(0) on every call
 * (sketch.rs:112) and has no seed argument; this entry point does the same
 * with the library's generator (Philox4x32, key 0).  Entry (i, j) uses
 * word i + j*round_up(rows, 4) of the stream; Gaussian entries are
 * Box-Muller pairs, Uniform is U(-1, 1), Rademacher is +-1.
 * Errors: rows == 0 or cols == 0 -> RNLA_ERR_INVALID_DIMENSIONS (sketch.rs:107-111). */
RNLA_API int rnla_sketching_operator(int32_t dist, int64_t rows, int64_t cols, double* out, int64_t ld);
RNLA_API int rnla_sketching_operator_ex(int32_t dist, int64_t rows, int64_t cols, const rnla_rng* rng,
                               double* out, int64_t ld);
RNLA_API int rnla_sketching_operator_dev(int32_t dist, int64_t rows, int64_t cols, const rnla_rng* rng,
                                double* out_dev, int64_t ld, void* stream);
/* float32 entries; `quantized` != 0 gives the operator the tensor-core
 * sketch applies (exactly representable in bf16): the Gaussian as t / 8,
 * t = round(8 g) clamped to +-63 (drawn through an alias table), the uniform
 * as the bin midpoints (2 floor(u / 2^26) - 63) / 64, Rademacher unchanged. */
RNLA_API int rnla_sketching_operator_f32_dev(int32_t dist, int64_t rows, int64_t cols, const rnla_rng* rng,
                                    int32_t quantized, float* out_dev, int64_t ld, void* stream);

/* ---- solver options and statistics ---- */
typedef enum {
    RNLA_PREC_FP64 = 0,      /* every product in FP64 on CUDA cores: the plain FP64 GPU path */
    RNLA_PREC_BF16X = 1,     /* tensor-core bf16 digit-sliced products with exact chunk sums */
    RNLA_PREC_BF16 = 2       /* RNLA_PREC_BF16X with one 8-bit digit per operand (fast, low accuracy);
                                other values: RNLA_ERR_INVALID_PARAMETERS */
} rnla_precision;

typedef enum {
    RNLA_MODE_REFERENCE = 0, /* rand_svd: the reference data flow (lora_helpers.rs:37-105) */
    RNLA_MODE_RANDNLA = 1    /* rand_svd: Gaussian range finder with q power iterations */
} rnla_mode;

typedef enum { RNLA_SOLVER_CGLS = 0, RNLA_SOLVER_LSQR = 1 } rnla_inner_solver;

typedef struct {
    int32_t precision;        /* rnla_precision */
    int32_t mode;             /* rnla_mode (rand_svd) */
    int32_t inner_solver;     /* rnla_inner_solver (blendenpik) */
    int32_t power_iters;      /* q for RNLA_MODE_RANDNLA */
    rnla_rng rng;             /* sketch generator and key */
    double atol;              /* LSQR atol/btol for blendenpik with RNLA_SOLVER_LSQR; */
    double btol;              /*   0 means: stop when ||(A M)^T r|| < epsilon, as CGLS does */
    double conlim;            /* LSQR conlim (0 -> 1e8) */
    int32_t digits_a;         /* 8-bit bf16 digits of the data matrix for RNLA_PREC_BF16X, 1..4 (0 = auto: 4) */
    int32_t digits_b;         /* bf16 digits of the second operand when it is a matrix (0 = auto) */
    int32_t orth;             /* 0 = CholeskyQR2 with Householder fallback, 1 = Householder */
    int32_t reserved;
} rnla_options;

typedef struct {
    int64_t iterations;       /* inner solver iterations */
    int64_t istop;            /* LSQR stop reason 0..7 (solvers.rs:264-270); CGLS: 1 = converged, 0 = not */
    double r1norm, r2norm, anorm, acond, arnorm, xnorm;
    int64_t sketch_rows;      /* d */
    int64_t rank;             /* r of rand_svd */
    int32_t orth_fallbacks;   /* CholeskyQR2 -> Householder fallbacks taken */
    int32_t precision_used;
    double ms_sketch, ms_factor, ms_solve, ms_total;  /* device-timed stages */
    double ms_kernel;         /* the inner solver's persistent kernel alone (device-timed; LSQR) */
    int64_t svd_sweeps;       /* rand_svd (tensor-core RandNLA mode): one-sided Jacobi sweeps of the small SVD */
} rnla_stats;

/* Defaults: FP64, reference mode, CGLS, power_iters 2, Philox4x32 key 0,
 * atol = btol = 0, conlim 1e8, automatic digits, CholeskyQR2. */
RNLA_API void rnla_options_default(rnla_options* opt);

/* ---- solvers.rs ---- */

/* solvers::solve_upper_triangular_system (src/solvers.rs:22-41): back
 * substitution for U x = y with U n x n upper triangular; a zero diagonal
 * entry leaves x_i = 0 (the reference skips it). */
RNLA_API int rnla_solve_upper_triangular_system(const double* u, int64_t n, int64_t ldu, const double* y,
                                       double* x);
RNLA_API int rnla_solve_upper_triangular_system_dev(const double* u, int64_t n, int64_t ldu,
                                           const double* y, double* x, void* stream);

/* Result record of rnla_lsqr: the scalar members of the reference's
 * 10-tuple (src/solvers.rs:125-136). */
typedef struct {
    int64_t istop, itn;
    double r1norm, r2norm, anorm, acond, xnorm;
} rnla_lsqr_result;

/* solvers::lsqr (src/solvers.rs:115-278): Paige-Saunders LSQR for
 * min ||A x - b||^2 + damp^2 ||x||^2.  iter_lim < 0 means the reference's
 * default 2n (solvers.rs:139).  x0 may be NULL (solvers.rs:142-152).
 * var (n values) is filled when calc_var != 0 and var != NULL.  arnorms,
 * if not NULL, receives the history of ||A^T r|| estimates (at most
 * iter_lim values, count = result->itn, or 1 for the early exit of
 * solvers.rs:180-182).  The persistent kernel holds the n-vectors across
 * its threads: n <= 4096 (RNLA_ERR_UNSUPPORTED above; the reference has no
 * limit), which also bounds the drivers built on it. */
RNLA_API int rnla_lsqr(const double* a, int64_t m, int64_t n, int64_t lda, const double* b, double damp,
              double atol, double btol, double conlim, int64_t iter_lim, int32_t calc_var,
              const double* x0, double* x, rnla_lsqr_result* result, double* arnorms, double* var);
RNLA_API int rnla_lsqr_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda, const double* b_dev,
                  double damp, double atol, double btol, double conlim, int64_t iter_lim,
                  int32_t calc_var, const double* x0_dev, double* x_dev, rnla_lsqr_result* result,
                  double* arnorms_host, double* var_dev, void* stream);  /* synchronises */

/* Allocation-free LSQR (no counterpart in the reference).  For callers that
 * cannot let a library allocate device memory: applications running under a
 * fixed memory budget managed by their own allocator, where a cudaMalloc can
 * fail or synchronise the device at an uncontrolled moment, and tight loops
 * that must not pay cudaMalloc/cudaFree per call.  Same algorithm as
 * rnla_lsqr_dev without the variance and history outputs; FP64 arithmetic.
 * All scratch lives in a fixed 32 MiB device array inside the library (held
 * by every GPU that loads it until the process exits); a problem needs
 * 8 * (10 + 4G + m + 5n + G n) bytes, G <= 4 x (number of SMs), and larger
 * problems return RNLA_ERR_INVALID_DIMENSIONS; n > 4096 returns
 * RNLA_ERR_UNSUPPORTED.  Calls share that array, so calls on one device are
 * serialised (a per-device lock held until the call has synchronised).
 * Every call clears its words with cudaMemsetAsync and synchronises the
 * given stream on its result before it returns: it must not be called on a
 * stream that is being captured into a graph. */
RNLA_API int rnla_lsqr_noalloc_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda,
                                   const double* b_dev, double damp, double atol, double btol,
                                   double conlim, int64_t iter_lim, const double* x0_dev,
                                   double* x_dev, rnla_lsqr_result* result, void* stream);

/* ---- cg.rs ---- */

/* cg::cgls (src/cg.rs:18-61): CGLS from x0 (NULL -> zeros); stops when
 * ||A^T r||_2 < tolerance (absolute) or after num_iterations.  The
 * reference's alpha = ||s||^2 / ||A p||^2 is kept as written, so a zero
 * right-hand side yields NaN as it does there.  iterations_out (nullable)
 * receives the iteration count.  n <= 4096, as for rnla_lsqr. */
RNLA_API int rnla_cgls(const double* a, int64_t m, int64_t n, int64_t lda, const double* b, double tolerance,
              int64_t num_iterations, const double* x0, double* x, int64_t* iterations_out);
RNLA_API int rnla_cgls_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda, const double* b_dev,
                  double tolerance, int64_t num_iterations, const double* x0_dev, double* x_dev,
                  int64_t* iterations_out, void* stream);  /* synchronises */

/* ---- lora_helpers.rs ---- */

/* lora_helpers::Orth (src/lora_helpers.rs:131-133): thin Q of a Householder
 * QR of X (m x n) into q (m x min(m,n), ldq). */
RNLA_API int rnla_orth(const double* x, int64_t m, int64_t n, int64_t ldx, double* q, int64_t ldq);
/* lora_helpers::Stabilizer (src/lora_helpers.rs:144-146): the unit-lower L
 * (m x min(m,n)) of a complete-pivoting LU P X Q = L U, without P.
 * Ties in the pivot search go to the first maximum in column-major order. */
RNLA_API int rnla_stabilizer(const double* x, int64_t m, int64_t n, int64_t ldx, double* l, int64_t ldl);
/* lora_helpers::tsog1 (src/lora_helpers.rs:58-105) with the reference's
 * data flow.  For even num_passes the Gaussian draw of line 71 is discarded
 * by the reference (the loop starts from the zero S1 of line 63), so the
 * result is a function of A alone.  Output s: n x cols_out, cols_out
 * returned through cols_out (nullable).  Odd num_passes use the library's
 * Philox4x32 Gaussian (key 0). */
RNLA_API int rnla_tsog1(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, int32_t num_passes,
               int32_t passes_per_stab, double* s, int64_t lds, int64_t* cols_out);
/* lora_helpers::RF1 (src/lora_helpers.rs:37-44): Q = Orth(A tsog1(A,k,2,1)),
 * m x cols_out. */
RNLA_API int rnla_rf1(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double* q,
             int64_t ldq, int64_t* cols_out);
/* lora_helpers::QB1 (src/lora_helpers.rs:17-23): Q = RF1(A,k), B = Q^T A
 * (cols_out x n).  epsilon is ignored, as in the reference (line 18). */
RNLA_API int rnla_qb1(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double epsilon,
             double* q, int64_t ldq, double* b, int64_t ldb, int64_t* cols_out);

/* ---- lora_drivers.rs ---- */

/* Rank r of rand_svd's outputs: min(k, min(m, n, k + s)) in reference
 * mode (lora_drivers.rs:51 with the shapes of lora_helpers.rs:58-105). */
RNLA_API int64_t rnla_rand_svd_rank(int64_t m, int64_t n, int64_t k, int64_t s, int32_t mode);

/* lora_drivers.rs:84-140 (rand_evd1): a (n x n, symmetric) ~ V diag(lambda)
 * V^T from QB1(a, k + s) and the eigenpairs of C = B Q, ordered by
 * decreasing |lambda|; r = min(k, columns of Q) pairs.  v: n x k (ldv),
 * lambda: k.  Errors: InvalidParameters (k, epsilon, s), NotHermitian (a
 * differs from its transpose). */
RNLA_API int rnla_rand_evd1(const double* a, int64_t n, int64_t lda, int64_t k, double epsilon, int64_t s,
                            double* v, int64_t ldv, double* lambda, int64_t* r_out);
/* lora_drivers.rs:153-213 (rand_evd2): Nystrom approximation of a PSD a
 * with the shift nu = sqrt(n) eps ||a S||_F, S = tsog1(a, k + s, 3, 1);
 * lambda = sigma^2 - nu of the singular values of (a S + nu S) R^-1 above the
 * shift, r <= k of them.  Errors: InvalidParameters (k),
 * NotPositiveSemiDefinite (an eigenvalue of a below 0),
 * MatrixDecompositionError (the Cholesky factorization fails). */
RNLA_API int rnla_rand_evd2(const double* a, int64_t n, int64_t lda, int64_t k, int64_t s, double* v,
                            int64_t ldv, double* lambda, int64_t* r_out);

/* lora_drivers::rand_svd (src/lora_drivers.rs:30-69): U (m x r), S (r x r,
 * diagonal, singular values descending), Vt (r x n).  Errors (checked in
 * this order, lora_drivers.rs:31-45): k == 0, epsilon <= 0, s == 0 ->
 * RNLA_ERR_INVALID_PARAMETERS. */
RNLA_API int rnla_rand_svd(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double epsilon,
                  int64_t s, double* u, int64_t ldu, double* sigma, int64_t lds, double* vt,
                  int64_t ldvt, int64_t* r_out);
/* Extended form: options select reference / RandNLA mode, precision, q and
 * the generator; `singular_values` (nullable, r values) receives the
 * diagonal of S; stats (nullable).  Reference mode runs in FP64 (a
 * tensor-core precision returns RNLA_ERR_UNSUPPORTED).  RandNLA mode under
 * RNLA_PREC_BF16X runs the range finder (A Omega, A^T Q, A Z) and the
 * projection B = Q^T A as split-bf16 tcgen05 GEMMs with FP32 accumulation
 * (digits_a = planes of the power-iteration products, default 2; the
 * projection and the CholeskyQR2 Grams and triangular products use 3), the
 * Cholesky, R^-1 and small SVD in FP64; Omega is the FP64 path's Gaussian,
 * so the two precisions can be compared on the same Omega. */
RNLA_API int rnla_rand_svd_ex(const double* a, int64_t m, int64_t n, int64_t lda, int64_t k, double epsilon,
                     int64_t s, const rnla_options* opt, double* u, int64_t ldu, double* sigma,
                     int64_t lds, double* vt, int64_t ldvt, int64_t* r_out, rnla_stats* stats);
/* Device-pointer form.  a_dev may be float (a_is_f32 != 0, the stored-FP32
 * configurations) or double.  Synchronises (r is returned). */
RNLA_API int rnla_rand_svd_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n, int64_t lda,
                      int64_t k, double epsilon, int64_t s, const rnla_options* opt, double* u_dev,
                      int64_t ldu, double* singular_values_dev, double* vt_dev, int64_t ldvt,
                      int64_t* r_out, rnla_stats* stats, void* stream);

/* ---- sketch_and_precondition.rs ---- */

/* sketch_and_precondition::blendenpik_overdetermined
 * (src/sketch_and_precondition.rs:26-59): d = min(m, floor(sf n)) Gaussian
 * sketch, QR of S A, z0 = Q^T S b, preconditioner R^-1, inner solver on
 * A R^-1 from z0, x = R^-1 z (n values).  The reference forms A R^-1
 * explicitly (line 56); here R^-1 is applied inside the solver's kernels.
 * Errors (in the reference's order, lines 29-48): m < n ->
 * RNLA_ERR_NOT_OVERDETERMINED; sampling_factor < 1, epsilon <= 0, l == 0 ->
 * RNLA_ERR_INVALID_PARAMETERS; a singular R (the reference's unwrap at
 * line 55 panics) -> RNLA_ERR_SINGULAR_MATRIX. */
RNLA_API int rnla_blendenpik_overdetermined(const double* a, int64_t m, int64_t n, int64_t lda,
                                   const double* b, double epsilon, int64_t l,
                                   double sampling_factor, double* x);
RNLA_API int rnla_blendenpik_overdetermined_ex(const double* a, int64_t m, int64_t n, int64_t lda,
                                      const double* b, double epsilon, int64_t l,
                                      double sampling_factor, const rnla_options* opt, double* x,
                                      rnla_stats* stats);
/* The same with A stored in FP32 on the host (b and x stay FP64): the
 * reference takes &DMatrix<f64> only; FP32 storage halves the bytes of A
 * moved and streamed for large problems.  A goes up in 64-column chunks and
 * the sketch starts on each of its column tiles as the tile's chunks land. */
RNLA_API int rnla_blendenpik_overdetermined_f32_ex(const float* a, int64_t m, int64_t n, int64_t lda,
                                          const double* b, double epsilon, int64_t l,
                                          double sampling_factor, const rnla_options* opt, double* x,
                                          rnla_stats* stats);
/* Device-pointer form; a_dev is double or float (a_is_f32). Synchronises. */
RNLA_API int rnla_blendenpik_overdetermined_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n,
                                       int64_t lda, const double* b_dev, double epsilon,
                                       int64_t l, double sampling_factor, const rnla_options* opt,
                                       double* x_dev, rnla_stats* stats, void* stream);

/* sketch_and_precondition.rs:82-119 (lsrn): the same sketch as blendenpik,
 * preconditioner N = V Sigma^-1 from the SVD of S a, CGLS on A N from 0,
 * x = N y.  Built on the QR of S a: with R = U_R Sigma V^T, N = R^-1 U_R, and
 * CGLS on A R^-1 U_R from 0 is CGLS on A R^-1 from 0 rotated by U_R^T, so
 * x = R^-1 z with z from CGLS (or LSQR, opt->inner_solver) on A R^-1
 * started at 0.  An exactly singular sketch returns RNLA_ERR_SINGULAR_MATRIX
 * (the reference would drop the zero singular directions). */
RNLA_API int rnla_lsrn_overdetermined(const double* a, int64_t m, int64_t n, int64_t lda, const double* b,
                                      double epsilon, int64_t l, double sampling_factor, double* x);
RNLA_API int rnla_lsrn_overdetermined_ex(const double* a, int64_t m, int64_t n, int64_t lda,
                                         const double* b, double epsilon, int64_t l,
                                         double sampling_factor, const rnla_options* opt, double* x,
                                         rnla_stats* stats);
RNLA_API int rnla_lsrn_overdetermined_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n,
                                          int64_t lda, const double* b_dev, double epsilon, int64_t l,
                                          double sampling_factor, const rnla_options* opt, double* x_dev,
                                          rnla_stats* stats, void* stream);

/* One least-squares problem of a batch: device pointers to column-major A
 * (m x n, leading dimension lda; float when a_is_f32), b (m values) and
 * the output x (n values). */
typedef struct {
    const void* a;
    int32_t a_is_f32;
    int32_t reserved;
    int64_t m, n, lda;
    const double* b;
    double* x;
} rnla_ls_problem;

/* Many independent blendenpik_overdetermined solves
 * (sketch_and_precondition.rs:26-59 per problem; the reference has no
 * batched entry, callers loop) with shared epsilon, l, sampling_factor and
 * options.  The problems' data must be in place in `stream` order; the
 * batch runs on four workers (host threads, each with its own streams and
 * grids sized for a quarter of the SMs) that take problems in index order,
 * so small problems run side by side.  Each x matches what
 * rnla_blendenpik_overdetermined_dev gives for the problem alone to the
 * solver's accuracy (same sketch seed and kernels; the smaller grids group
 * partial sums differently).  status_out (count entries, required) receives
 * each problem's status, stats_out (nullable, count entries) its facts.
 * Returns RNLA_OK when every problem succeeded, else the lowest-index
 * failing problem's status (its message in rnla_last_error_message); a
 * CUDA error stops the batch and marks the problems not yet run
 * RNLA_ERR_CUDA.  Synchronises. */
RNLA_API int rnla_solve_batched(const rnla_ls_problem* probs, int64_t count, double epsilon, int64_t l,
                                double sampling_factor, const rnla_options* opt, int32_t* status_out,
                                rnla_stats* stats_out, void* stream);

/* cqrrpt.rs:27-58 (sap_chol_qrcp): Gaussian sketch S (d x m, n <= d <= m) of
 * a, column-pivoted Householder QR of S a (pivot_decompositions.rs:106-174:
 * largest remaining column norm, first index on ties), then CholeskyQR of
 * a[:, jpvt] R_sk^-1:  a[:, jpvt] = Q R with Q m x n (orthonormal columns),
 * R n x n upper triangular, jpvt the column order (n entries).  Errors:
 * RNLA_ERR_INVALID_PARAMETERS unless n <= d <= m; RNLA_ERR_SINGULAR_MATRIX
 * when the sketch's numerical rank (|R_ii| > 1e-10) is below n;
 * RNLA_ERR_MATRIX_DECOMPOSITION when the Cholesky factorization fails. */
RNLA_API int rnla_sap_chol_qrcp(const double* a, int64_t m, int64_t n, int64_t lda, int64_t d,
                                const rnla_options* opt, double* q, int64_t ldq, double* r, int64_t ldr,
                                int64_t* jpvt);
RNLA_API int rnla_sap_chol_qrcp_dev(const double* a_dev, int64_t m, int64_t n, int64_t lda, int64_t d,
                                    const rnla_options* opt, double* q_dev, int64_t ldq, double* r_dev,
                                    int64_t ldr, int64_t* jpvt_dev, void* stream);

/* sketch_and_solve.rs:24-33 (qr) and :53-65 (svd): x (n) from the
 * Gaussian sketch S (m/4 x m; generator and key of opt, Philox key 0 by
 * default) of [a b]: thin QR of S a and x = R^-1 (Q^T S b), or the SVD
 * S a = U Sigma V^T and x = V Sigma^+ U^T S b; an exactly zero pivot or
 * singular value gives a zero component (solvers.rs:22-41, 56-70).
 * opt->precision selects the FP64 data flow or the tensor-core sketch.
 * RNLA_ERR_INVALID_DIMENSIONS when m/4 < n. */
RNLA_API int rnla_sketched_least_squares_qr(const double* a, int64_t m, int64_t n, int64_t lda,
                                            const double* b, const rnla_options* opt, double* x);
RNLA_API int rnla_sketched_least_squares_svd(const double* a, int64_t m, int64_t n, int64_t lda,
                                             const double* b, const rnla_options* opt, double* x);
RNLA_API int rnla_sketched_least_squares_dev(const void* a_dev, int32_t a_is_f32, int64_t m, int64_t n,
                                             int64_t lda, const double* b_dev, int32_t use_svd,
                                             const rnla_options* opt, double* x_dev, void* stream);

/* ---- building blocks exposed for parity tests (device pointers) ---- */

/* Y (ldy) = S X: the sketch S (d x m, Gaussian, generator rng) applied to
 * X (m x n, ldx) without materialising S.  precision RNLA_PREC_BF16X uses
 * the tensor-core digit-sliced kernel with the quantised Gaussian
 * (rnla_sketching_operator_f32_dev with quantized = 1); digits = 8-bit
 * bf16 digits of X, 1..4 (0 = auto: 4).  x_is_f32 selects float or double X. */
RNLA_API int rnla_sketch_apply_dev(const void* x_dev, int32_t x_is_f32, int64_t m, int64_t n, int64_t ldx,
                          int64_t d, const rnla_rng* rng, int32_t precision, int32_t digits,
                          double* y_dev, int64_t ldy, void* stream);
/* The same with the distribution of S (dist: RNLA_GAUSSIAN, RNLA_UNIFORM,
 * RNLA_RADEMACHER).  Under RNLA_PREC_BF16X S is the quantised form of the
 * distribution (rnla_sketching_operator_f32_dev with quantized = 1): t / 8
 * with t the alias-table Gaussian, (2 floor(u / 2^26) - 63) / 64 for the
 * uniform, the exact +-1 for Rademacher. */
RNLA_API int rnla_sketch_apply_ex_dev(const void* x_dev, int32_t x_is_f32, int64_t m, int64_t n, int64_t ldx,
                                      int64_t d, int32_t dist, const rnla_rng* rng, int32_t precision,
                                      int32_t digits, double* y_dev, int64_t ldy, void* stream);

/* C (ldc) = X^T Y for X (k x mm, ldx) and Y (k x nn, ldy), both double:
 * RNLA_PREC_FP64 on the FP64 CUDA cores; RNLA_PREC_BF16X on the split-bf16
 * tcgen05 GEMM, each operand cut into max(digits_x, digits_y) bf16 planes
 * (1..3, default 3) and the plane pairs p + q < planes accumulated in FP32
 * (3 planes: ~24 significant bits per operand); RNLA_PREC_BF16 = one plane;
 * 4 or more digits select exact integer digit products (X in five 6-bit
 * digits and Y in four 8-bit digits below each column's maximum, 1024-term
 * windows exact in FP32 and folded into int64). */
RNLA_API int rnla_gemm_tn_dev(const double* x_dev, int64_t k, int64_t mm, int64_t ldx, const double* y_dev,
                     int64_t nn, int64_t ldy, int32_t precision, int32_t digits_x,
                     int32_t digits_y, double* c_dev, int64_t ldc, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RANDNLA_GB300_H */
