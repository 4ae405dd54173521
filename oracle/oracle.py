"""ORACLE — test infrastructure only.

CPU restatement of the reference crate's hot path (divijkhaitan/randnla,
crate `randblas`) in numpy, plus this project's intended RandNLA variants in
plain FP64, used as the checker for the CUDA library.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import this
module; the product library never calls it.

Every function cites the reference lines it restates.  The dense kernels the
reference delegates to nalgebra 0.33.0 (GEMM, Householder QR, SVD,
full-pivot LU, triangular solve; absent from the checkout) are restated as
textbook algorithms or LAPACK calls through numpy:

* Householder QR  -> numpy.linalg.qr (LAPACK geqrf/orgqr; a column whose
  sub-diagonal part is zero gets the identity reflector, which reproduces the
  reference tests Orth(0) = I and Orth(I) = I, lora_helpers.rs:325-341);
* full-pivot LU   -> complete pivoting (Golub & Van Loan, alg. 3.4.3); ties
  go to the first maximum in column-major order; a zero pivot ends the
  elimination, which reproduces Stabilizer(0) = I (lora_helpers.rs:359-366);
* SVD             -> numpy.linalg.svd (LAPACK gesdd).

Parity status: the reference's generator values
(rand_distr's normal sampler behind sketch.rs:114-117) are unpinned; results
that are independent of the sketch (the reference rand_svd, which never uses
its Gaussian — lora_helpers.rs:70-99 — and converged least-squares
solutions) are compared directly.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

DIST_GAUSSIAN, DIST_UNIFORM, DIST_RADEMACHER = 0, 1, 2
GEN_PHILOX4X32, GEN_THREEFRY2X64 = 0, 1


def lib():
    """The oracle's C checker (rng_oracle.c), built by oracle/build_oracle.sh."""
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "liboracle_rng.so")
        if not os.path.exists(path):
            import subprocess
            subprocess.check_call(["sh", os.path.join(_HERE, "build_oracle.sh")])
        L = ctypes.CDLL(path)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        L.oracle_philox4x32.argtypes = [u32p, u32p, u32p]
        L.oracle_philox2x32.argtypes = [u32p, u32p, u32p]
        L.oracle_philox2x64.argtypes = [u64p, u64p, u64p]
        L.oracle_philox4x64.argtypes = [u64p, u64p, u64p]
        L.oracle_threefry2x64.argtypes = [u64p, u64p, u64p]
        L.oracle_word_stream.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                         ctypes.c_uint64, ctypes.c_int64, ctypes.c_void_p]
        L.oracle_word_checksums.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                            ctypes.c_uint64, ctypes.c_int64, u64p, u64p]
        L.oracle_sketch_fill.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                         ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_int64]
        L.oracle_sketch_fill_cols.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                              ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64]
        L.oracle_qgauss_t.argtypes = [ctypes.c_uint32]
        L.oracle_qgauss_t.restype = ctypes.c_int
        L.oracle_sketch_fill_quantized.argtypes = [ctypes.c_int, ctypes.c_uint64,
                                                   ctypes.c_uint64, ctypes.c_int64,
                                                   ctypes.c_int64, ctypes.c_void_p,
                                                   ctypes.c_int64]
        L.oracle_sketch_fill_quantized_dist.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                                         ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                                         ctypes.c_void_p, ctypes.c_int64]
        _LIB = L
    return _LIB


def _arr(ctype, vals):
    return (ctype * len(vals))(*vals)


def philox4x32(ctr, key):
    out = (ctypes.c_uint32 * 4)()
    lib().oracle_philox4x32(_arr(ctypes.c_uint32, ctr), _arr(ctypes.c_uint32, key), out)
    return list(out)


def philox2x32(ctr, key):
    out = (ctypes.c_uint32 * 2)()
    lib().oracle_philox2x32(_arr(ctypes.c_uint32, ctr), _arr(ctypes.c_uint32, key), out)
    return list(out)


def philox2x64(ctr, key):
    out = (ctypes.c_uint64 * 2)()
    lib().oracle_philox2x64(_arr(ctypes.c_uint64, ctr), _arr(ctypes.c_uint64, key), out)
    return list(out)


def philox4x64(ctr, key):
    out = (ctypes.c_uint64 * 4)()
    lib().oracle_philox4x64(_arr(ctypes.c_uint64, ctr), _arr(ctypes.c_uint64, key), out)
    return list(out)


def threefry2x64(ctr, key):
    out = (ctypes.c_uint64 * 2)()
    lib().oracle_threefry2x64(_arr(ctypes.c_uint64, ctr), _arr(ctypes.c_uint64, key), out)
    return list(out)


def word_stream(gen, key0, key1, first_word, n):
    out = np.empty(n, dtype=np.uint32)
    lib().oracle_word_stream(gen, key0, key1, first_word, n, out.ctypes.data)
    return out


def word_checksums(gen, key0, key1, first_word, n):
    """(sum of the words, sum of word xor offset) of n stream words, mod 2^64."""
    s1, s2 = ctypes.c_uint64(0), ctypes.c_uint64(0)
    lib().oracle_word_checksums(gen, key0, key1, first_word, n, ctypes.byref(s1), ctypes.byref(s2))
    return s1.value, s2.value


def sketch(dist, rows, cols, gen=GEN_PHILOX4X32, key0=0, key1=0, quantized=False):
    """Dense rows x cols sketching operator (float64, column-major).

    Shape checks follow sketch.rs:107-111; the entry values follow this
    project's transform (rng_oracle.c), not rand_distr (unpinned)."""
    if rows <= 0 or cols <= 0:
        raise ValueError("Rows and columns must be greater than 0")
    out = np.empty((rows, cols), dtype=np.float32, order="F")
    if quantized:
        lib().oracle_sketch_fill_quantized_dist(dist, gen, key0, key1, rows, cols, out.ctypes.data, rows)
    else:
        lib().oracle_sketch_fill(dist, gen, key0, key1, rows, cols, out.ctypes.data, rows)
    return out.astype(np.float64)


def sketch_cols(dist, rows, j0, j1, gen=GEN_PHILOX4X32, key0=0, key1=0, threads=None):
    """Columns [j0, j1) of sketch(dist, rows, cols) (float64, column-major),
    generated by `threads` host threads in column blocks (the C fill releases
    the GIL).  Entry values are those of sketch()."""
    import concurrent.futures as cf
    cols = j1 - j0
    out = np.empty((rows, cols), dtype=np.float32, order="F")
    threads = threads or os.cpu_count() or 1
    step = max(1, -(-cols // threads))
    L = lib()

    def fill(c0):
        c1 = min(cols, c0 + step)
        L.oracle_sketch_fill_cols(dist, gen, key0, key1, rows, j0 + c0, j0 + c1,
                                  out.ctypes.data + 4 * rows * c0, rows)

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(fill, range(0, cols, step)))
    return out.astype(np.float64)


# ---------------------------------------------------------------------------
# solvers.rs
# ---------------------------------------------------------------------------

def solve_upper_triangular_system(u, y):
    """solvers.rs:22-41: back substitution; a zero pivot leaves x_i = 0."""
    u = np.asarray(u, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64).reshape(-1)
    n = u.shape[0]
    x = np.zeros(n)
    for i in range(n - 1, -1, -1):
        if u[i, i] != 0.0:
            s = 0.0
            for j in range(i + 1, n):
                s += u[i, j] * x[j]
            x[i] = (y[i] - s) / u[i, i]
    return x


def _sign(x):
    """solvers.rs:77-81 (sign(0) = 0)."""
    return 1.0 if x > 0 else (-1.0 if x < 0 else 0.0)


def sym_ortho(a, b):
    """solvers.rs:84-102."""
    if b == 0.0:
        return _sign(a), 0.0, abs(a)
    if a == 0.0:
        return 0.0, _sign(b), abs(b)
    if abs(b) > abs(a):
        tau = a / b
        s = _sign(b) / np.sqrt(1.0 + tau * tau)
        c = s * tau
        return c, s, b / s
    tau = b / a
    c = _sign(a) / np.sqrt(1.0 + tau * tau)
    s = c * tau
    return c, s, a / c


def lsqr(a, b, damp=0.0, atol=1e-8, btol=1e-8, conlim=1e8, iter_lim=None,
         calc_var=False, x0=None, matvec=None, rmatvec=None):
    """solvers.rs:115-278 (Paige-Saunders LSQR as translated from scipy).

    Returns the reference's 10-tuple
    (x, istop, itn, r1norm, r2norm, anorm, acond, arnorms, xnorm, var).
    matvec/rmatvec optionally replace a @ v and a.T @ u (used for the
    implicitly preconditioned operator)."""
    if matvec is None:
        matvec = lambda v: a @ v
        rmatvec = lambda u: a.T @ u
        m, n = a.shape
    else:
        m, n = a
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    eps = np.finfo(np.float64).eps
    if iter_lim is None:
        iter_lim = 2 * n
    var = np.zeros(n)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64).reshape(-1)
    u = b.copy()
    bnorm = np.linalg.norm(b)
    if x0 is not None:
        u = u - matvec(x)
        beta = np.linalg.norm(u)
    else:
        beta = bnorm
    u = u * (1.0 / beta if beta > 0 else 0.0)
    v = rmatvec(u)
    alfa = np.linalg.norm(v)
    v = v * (1.0 / alfa if alfa > 0 else 0.0)
    w = v.copy()
    rhobar, phibar = alfa, beta
    rnorm = r1norm = r2norm = beta
    anorm = acond = 0.0
    dampsq = damp * damp
    ddnorm = res2 = xnorm = xxnorm = z = 0.0
    cs2, sn2 = -1.0, 0.0
    arnorm = alfa * beta
    if arnorm == 0.0:
        return x, 0, 0, beta, beta, 0.0, 0.0, [0.0], 0.0, var
    ctol = 1.0 / conlim if conlim > 0 else 0.0
    arnorms = [-1.0] * iter_lim
    itn = 0
    istop = 0
    while itn < iter_lim:
        arnorms[itn] = arnorm
        itn += 1
        u = matvec(v) - alfa * u
        beta = np.linalg.norm(u)
        if beta > 0:
            u = u * (1.0 / beta)
            anorm = np.sqrt(anorm ** 2 + alfa ** 2 + beta ** 2 + dampsq)
            v = rmatvec(u) - beta * v
            alfa = np.linalg.norm(v)
            v = v * (1.0 / alfa if alfa > 0 else 0.0)
        rhobar1 = np.sqrt(rhobar ** 2 + dampsq)
        cs1 = rhobar / rhobar1
        sn1 = damp / rhobar1
        psi = sn1 * phibar
        phibar = phibar * cs1
        cs, sn, rho = sym_ortho(rhobar1, beta)
        theta = sn * alfa
        rhobar = -cs * alfa
        phi = cs * phibar
        phibar = phibar * sn
        tau = sn * phi
        t1 = phi / rho
        t2 = -theta / rho
        dk = w * (1.0 / rho)
        x = x + t1 * w
        w = v + t2 * w
        ddnorm += float(dk @ dk)
        if calc_var:
            var = var + dk * dk
        delta = sn2 * rho
        gambar = -cs2 * rho
        rhs = phi - delta * z
        zbar = rhs / gambar
        xnorm = np.sqrt(xxnorm + zbar ** 2)
        gamma = np.sqrt(gambar ** 2 + theta ** 2)
        cs2 = gambar / gamma
        sn2 = theta / gamma
        z = rhs / gamma
        xxnorm += z ** 2
        acond = anorm * np.sqrt(ddnorm)
        res1 = phibar ** 2
        res2 += psi ** 2
        rnorm = np.sqrt(res1 + res2)
        arnorm = alfa * abs(tau)
        r1sq = rnorm ** 2 - dampsq * xxnorm
        r1norm = np.sqrt(abs(r1sq))
        r2norm = rnorm
        test1 = rnorm / bnorm
        test2 = arnorm / (anorm * rnorm + eps)
        test3 = 1.0 / (acond + eps)
        t1 = test1 / (1.0 + anorm * xnorm / bnorm)
        rtol = atol + btol * (anorm * xnorm / bnorm)
        if itn >= iter_lim:
            istop = 7
        if 1.0 + test3 <= 1.0:
            istop = 6
        if 1.0 + test2 <= 1.0:
            istop = 5
        if 1.0 + t1 <= 1.0:
            istop = 4
        if test3 <= ctol:
            istop = 3
        if test2 <= atol:
            istop = 2
        if test1 <= rtol:
            istop = 1
        if istop != 0:
            break
    arnorms = [v_ for v_ in arnorms if v_ > -1.0]
    return x, istop, itn, r1norm, r2norm, anorm, acond, arnorms, xnorm, var


# ---------------------------------------------------------------------------
# cg.rs
# ---------------------------------------------------------------------------

def cgls(a, b, tolerance, num_iterations, x=None, return_iters=False):
    """cg.rs:18-61: CGLS; stops when ||A^T r||_2 < tolerance (absolute) or
    after num_iterations.  0/0 in alpha propagates NaN exactly as the
    reference does."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    n = a.shape[1]
    x = np.zeros(n) if x is None else np.array(x, dtype=np.float64).reshape(-1)
    r = b - a @ x
    s = a.T @ r
    p = s.copy()
    norm_s = float(s @ s)
    iters = 0
    with np.errstate(divide="ignore", invalid="ignore"):
        for i in range(num_iterations):
            ap = a @ p
            alpha = np.float64(norm_s) / np.float64(ap @ ap)
            x = x + alpha * p
            r = r - alpha * ap
            s_new = a.T @ r
            norm_s_new = float(s_new @ s_new)
            iters = i + 1
            if np.sqrt(norm_s_new) < tolerance:
                break
            beta = np.float64(norm_s_new) / np.float64(norm_s)
            norm_s = norm_s_new
            p = s_new + beta * p
    return (x, iters) if return_iters else x


# ---------------------------------------------------------------------------
# lora_helpers.rs / lora_drivers.rs
# ---------------------------------------------------------------------------

def orth(X):
    """lora_helpers.rs:131-133: thin Q of a Householder QR, m x min(m, n)."""
    q, _ = np.linalg.qr(np.asarray(X, dtype=np.float64), mode="reduced")
    return q


def full_piv_lu_l(X):
    """lora_helpers.rs:144-146: the unit-lower L of a complete-pivoting LU
    P X Q = L U, returned WITHOUT the row permutation P (m x min(m, n))."""
    A = np.array(X, dtype=np.float64, copy=True)
    m, n = A.shape
    p = min(m, n)
    for k in range(p):
        sub = np.abs(A[k:, k:])
        idx = int(np.argmax(sub.T))           # first maximum, column-major order
        jj, ii = divmod(idx, m - k)
        if sub[ii, jj] == 0.0:
            break
        r, c = k + ii, k + jj
        if r != k:
            A[[k, r], :] = A[[r, k], :]
        if c != k:
            A[:, [k, c]] = A[:, [c, k]]
        A[k + 1:, k] /= A[k, k]
        A[k + 1:, k + 1:] -= np.outer(A[k + 1:, k], A[k, k + 1:])
    return np.tril(A[:, :p], -1) + np.eye(m, p)


stabilizer = full_piv_lu_l


def tsog1(A, k, num_passes=2, passes_per_stab=1, gaussian=None):
    """lora_helpers.rs:58-105, data flow reproduced literally.

    With an even num_passes the Gaussian is drawn into S and then overwritten
    (lines 70-72, 89): the loop starts from S1, which is still the zero n x k
    matrix of line 63.  `gaussian(rows, cols)` supplies the odd-pass draw
    (unpinned values)."""
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    passes_done = 0
    S1 = np.zeros((n, k))
    S = np.zeros((n, k))
    if num_passes % 2 == 0:
        S = gaussian(n, k) if gaussian is not None else S   # discarded below
    else:
        S1 = gaussian(m, k)
        S1 = A.T @ S1
        passes_done += 1
        if passes_done % passes_per_stab == 0:
            _ = stabilizer(S1)                                  # result unused (_S2)
    diff = num_passes - passes_done
    while diff >= 2:
        S = A @ S1
        passes_done += 1
        if passes_done % passes_per_stab == 0:
            S = stabilizer(S)
        S = A.T @ S
        passes_done += 1
        if passes_done % passes_per_stab == 0:
            S = stabilizer(S)
        diff -= 2
    return S


def rf1(A, k):
    """lora_helpers.rs:37-44."""
    S = tsog1(A, k, 2, 1)
    return orth(np.asarray(A) @ S)


def qb1(A, k, epsilon=None):
    """lora_helpers.rs:17-23 (epsilon ignored, line 18)."""
    Q = rf1(A, k)
    return Q, Q.T @ np.asarray(A)


class InvalidParameters(ValueError):
    pass


# the other RandNLAError variants (errors.rs:3-14) the restatements raise
class InvalidDimensions(ValueError):
    pass


class NotOverdetermined(ValueError):
    pass


class SingularMatrix(ValueError):
    pass


class MatrixDecompositionError(ValueError):
    pass


class NotHermitian(ValueError):
    pass


class NotPositiveSemiDefinite(ValueError):
    pass


def rand_svd(A, k, epsilon, s):
    """lora_drivers.rs:30-69: validation, QB1(A, k+s), SVD of B, truncation
    to r = min(k, Q.ncols()), U = Q U_B.  Returns (U m x r, S r x r, Vt r x n)."""
    if k == 0:
        raise InvalidParameters("Rank k must be positive, current input is %d" % k)
    if not epsilon > 0.0:
        raise InvalidParameters("Epsilon must be positive, current input is %r" % epsilon)
    if s == 0:
        raise InvalidParameters("Oversampling parameter s must be positive, current input is %d" % s)
    Q, B = qb1(A, k + s, epsilon)
    r = min(k, Q.shape[1])
    U, sig, Vt = np.linalg.svd(B, full_matrices=False)
    return Q @ U[:, :r], np.diag(sig[:r]), Vt[:r, :]


def rand_evd1(A, k, epsilon, s):
    """lora_drivers.rs:84-140 restated: QB1(A, k + s), the eigenpairs of
    C = B Q by decreasing |lambda|, V = Q U for the first min(k, cols) pairs."""
    A = np.asarray(A, dtype=np.float64)
    if k == 0 or not epsilon > 0.0 or s == 0:
        raise InvalidParameters("invalid rand_evd1 parameters")
    if not np.array_equal(A, A.T):
        raise NotHermitian("NotHermitian")
    Q, B = qb1(A, k + s, epsilon)
    w, U = np.linalg.eigh(B @ Q)
    order = np.argsort(-np.abs(w), kind="stable")
    r = min(k, len(w))
    return Q @ U[:, order[:r]], [float(w[i]) for i in order[:r]]


def rand_evd2(A, k, s):
    """lora_drivers.rs:153-213 restated: PSD check on every eigenvalue,
    S = tsog1(A, k + s, 3, 1), the shifted Nystrom factor (A S + nu S) R^-1,
    R^T R = S^T (A S + nu S), and lambda = sigma^2 - nu above the shift."""
    A = np.asarray(A, dtype=np.float64)
    if k == 0:
        raise InvalidParameters("Rank k must be positive")
    if np.any(np.linalg.eigvalsh(A) < 0.0):
        raise NotPositiveSemiDefinite("NotPositiveSemiDefinite")
    n = A.shape[0]
    # the odd-pass Gaussian: this library's Philox stream, key 0 (as the GPU draws it)
    S = tsog1(A, k + s, 3, 1, gaussian=lambda r, c: sketch(DIST_GAUSSIAN, r, c))
    Y = A @ S
    nu = np.sqrt(n) * np.finfo(np.float64).eps * np.linalg.norm(Y)
    Yn = Y + nu * S
    try:
        R = np.linalg.cholesky(S.T @ Yn).T
    except np.linalg.LinAlgError:
        raise MatrixDecompositionError("Cholesky Decomposition Failed") from None
    B = Yn @ np.linalg.inv(R)
    U, sig, _ = np.linalg.svd(B, full_matrices=False)
    lam = [x * x for x in sig if x > 0.0]
    r = min(k, sum(1 for x in lam if x > nu))
    return U[:, :r], [x - nu for x in lam[:r]]


def sketch_rows(m, n, sampling_factor):
    """sketch_and_precondition.rs:49: d = m if sf*n > m else floor(sf*n)."""
    return m if sampling_factor * n > m else int(np.floor(sampling_factor * n))


def blendenpik_overdetermined(a, b, epsilon, l, sampling_factor, S=None, return_iters=False):
    """sketch_and_precondition.rs:26-59: Gaussian sketch, QR of S a,
    z0 = Q^T S b, explicit R^-1, explicit a R^-1, CGLS, x = R^-1 z.
    S (d x m) may be supplied; by default the oracle's Philox sketch, seed 0."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    m, n = a.shape
    if m < n:
        raise NotOverdetermined("NotOverdetermined")
    if sampling_factor < 1.0 or not epsilon > 0.0 or l == 0:
        raise InvalidParameters("invalid blendenpik parameters")
    d = sketch_rows(m, n, sampling_factor)
    if S is None:
        S = sketch(DIST_GAUSSIAN, d, m)
    a_sk = S @ a
    b_sk = S @ b
    q, r = np.linalg.qr(a_sk, mode="reduced")
    z0 = q.T @ b_sk
    rinv = _upper_inverse(r)
    a_pre = a @ rinv
    z, iters = cgls(a_pre, b, epsilon, l, z0, return_iters=True)
    x = rinv @ z
    return (x, iters) if return_iters else x


def blendenpik_overdetermined_blocked(a, b, epsilon, l, sampling_factor, block=65536, threads=None,
                                      return_iters=False):
    """blendenpik_overdetermined with the same S formed in column blocks:
    S a and S b accumulate block by block (block columns of S generated by
    `threads` host threads), so the d x m operator is never held whole.  The
    rest of the data flow (QR, z0 = Q^T S b, explicit R^-1 and a R^-1, CGLS,
    x = R^-1 z) is that of sketch_and_precondition.rs:26-59."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    m, n = a.shape
    if m < n:
        raise NotOverdetermined("NotOverdetermined")
    if sampling_factor < 1.0 or not epsilon > 0.0 or l == 0:
        raise InvalidParameters("invalid blendenpik parameters")
    d = sketch_rows(m, n, sampling_factor)
    a_sk = np.zeros((d, n))
    b_sk = np.zeros(d)
    for k0 in range(0, m, block):
        k1 = min(m, k0 + block)
        S = sketch_cols(DIST_GAUSSIAN, d, k0, k1, threads=threads)
        a_sk += S @ a[k0:k1]
        b_sk += S @ b[k0:k1]
        del S
    q, r = np.linalg.qr(a_sk, mode="reduced")
    z0 = q.T @ b_sk
    rinv = _upper_inverse(r)
    a_pre = a @ rinv
    z, iters = cgls(a_pre, b, epsilon, l, z0, return_iters=True)
    x = rinv @ z
    return (x, iters) if return_iters else x


def lsrn_overdetermined(a, b, epsilon, l, sampling_factor, S=None, return_iters=False):
    """sketch_and_precondition.rs:82-119: the blendenpik sketch, N = V Sigma^+
    from the SVD of S a (zero singular values give zero), CGLS on the
    explicit A N from y = 0, x = N y."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    m, n = a.shape
    if m < n:
        raise NotOverdetermined("NotOverdetermined")
    if sampling_factor < 1.0 or not epsilon > 0.0 or l == 0:
        raise InvalidParameters("invalid lsrn parameters")
    d = sketch_rows(m, n, sampling_factor)
    if S is None:
        S = sketch(DIST_GAUSSIAN, d, m)
    _, sig, vt = np.linalg.svd(S @ a, full_matrices=False)
    sinv = np.where(sig != 0.0, 1.0 / np.where(sig != 0.0, sig, 1.0), 0.0)
    N = vt.T * sinv
    y, iters = cgls(a @ N, b, epsilon, l, np.zeros(N.shape[1]), return_iters=True)
    x = N @ y
    return (x, iters) if return_iters else x


def qrcp(a):
    """pivot_decompositions.rs:106-174 restated: greedy column pivoting by the
    largest remaining norm (strictly larger moves; the first index keeps ties),
    Householder v = x + sign(x_0) ||x|| e_0 normalised, c -= 2 v (v^T c) on the
    columns from k on, norms of the later columns recomputed below row k.
    Returns (r, p): r the reflected matrix (R in its upper triangle), p the
    column order."""
    r = np.array(a, dtype=np.float64, copy=True)
    m, n = r.shape
    p = list(range(n))
    norms = [float(np.linalg.norm(r[:, j])) for j in range(n)]
    for k in range(min(m, n)):
        best, bi = norms[k], k
        for j in range(k + 1, n):
            if norms[j] > best:
                best, bi = norms[j], j
        if bi != k:
            r[:, [k, bi]] = r[:, [bi, k]]
            p[k], p[bi] = p[bi], p[k]
            norms[k], norms[bi] = norms[bi], norms[k]
        x = r[k:, k].copy()
        nx = float(np.linalg.norm(x))
        if nx != 0.0:
            v = x
            v[0] += nx if v[0] >= 0.0 else -nx
            v /= np.linalg.norm(v)
            r[k:, k:] -= 2.0 * np.outer(v, v @ r[k:, k:])
            for j in range(k + 1, n):
                norms[j] = float(np.linalg.norm(r[k + 1:, j]))
    return r, p


def sap_chol_qrcp(a, d, S=None):
    """cqrrpt.rs:27-58 restated: QRCP of the d x m Gaussian sketch of a, then
    CholeskyQR of a[:, p] R_sk^-1.  Returns (q, r, p) with a[:, p] = q r
    (r upper triangular, the sketch's R taken from its upper triangle)."""
    a = np.asarray(a, dtype=np.float64)
    m, n = a.shape
    if not (n <= d <= m):
        raise InvalidParameters("d must satisfy n <= d << m")
    if S is None:
        S = sketch(DIST_GAUSSIAN, d, m)
    r_sk, p = qrcp(S @ a)
    k = sum(1 for i in range(min(d, n)) if abs(r_sk[i, i]) > 1e-10)
    if k < n:
        raise SingularMatrix("SingularMatrix")
    rk = np.triu(r_sk[:n, :n])
    a_pre = a[:, p] @ _upper_inverse(rk)
    r_pre = np.linalg.cholesky(a_pre.T @ a_pre).T
    q = a_pre @ _upper_inverse(r_pre)
    return q, r_pre @ rk, p


def sketched_least_squares_qr(a, b, S=None):
    """sketch_and_solve.rs:24-33: Gaussian sketch S (m/4 x m, Philox key 0
    by default), thin QR of S a, x = R^-1 Q^T S b with the zero-pivot rule
    of solvers.rs:22-41.  Returns x (n)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    m, n = a.shape
    d = m // 4
    if d < n:
        raise InvalidDimensions("InvalidDimensions")
    if S is None:
        S = sketch(DIST_GAUSSIAN, d, m)
    q, r = np.linalg.qr(S @ a, mode="reduced")
    return solve_upper_triangular_system(r, q.T @ (S @ b))


def sketched_least_squares_svd(a, b, S=None):
    """sketch_and_solve.rs:53-65: SVD of S a, x = V Sigma^+ U^T S b, a zero
    singular value giving a zero component (solvers.rs:56-70).  Returns x (n)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    m, n = a.shape
    d = m // 4
    if d < n:
        raise InvalidDimensions("InvalidDimensions")
    if S is None:
        S = sketch(DIST_GAUSSIAN, d, m)
    u, sig, vt = np.linalg.svd(S @ a, full_matrices=False)
    y = u.T @ (S @ b)
    y = np.where(sig != 0.0, y / np.where(sig != 0.0, sig, 1.0), 0.0)
    return vt.T @ y


def _upper_inverse(r):
    """R^-1 of an upper-triangular R column by column (solve R X = I),
    as sketch_and_precondition.rs:55 does with solve_upper_triangular."""
    import scipy.linalg
    return scipy.linalg.solve_triangular(r, np.eye(r.shape[0]), lower=False)


# ---------------------------------------------------------------------------
# This project's intended RandNLA algorithms in plain FP64 (the FP64 oracle
# of the GPU fast paths).  Same seed, same (optionally quantised) sketch.
# ---------------------------------------------------------------------------

def blendenpik_lsqr(a, b, sampling_factor=4.0, atol=1e-12, btol=1e-12, iter_lim=None,
                    seed=0, quantized=False, conlim=1e8):
    """Sketch [a b] with the Philox Gaussian (d x m), Householder QR,
    M = R^-1, LSQR on the implicitly preconditioned operator a M from
    z0 = (Q^T S b)[:n], x = M z.  Returns (x, lsqr_tuple)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    m, n = a.shape
    d = sketch_rows(m, n, sampling_factor)
    S = sketch(DIST_GAUSSIAN, d, m, key0=seed, quantized=quantized)
    sk = S @ np.column_stack([a, b])
    q, r = np.linalg.qr(sk[:, :n], mode="reduced")
    z0 = q.T @ sk[:, n]
    M = _upper_inverse(r)
    res = lsqr((m, n), b, 0.0, atol, btol, conlim, iter_lim, False, z0,
               matvec=lambda v: a @ (M @ v), rmatvec=lambda u: M.T @ (a.T @ u))
    return M @ res[0], res


def rand_svd_randnla(A, k, p, q, seed=42, quantized=False):
    """Gaussian range finder with q power iterations and re-orthonormalisation
    after every product, QB, small SVD, truncation to k.  Omega is the
    n x (k+p) Philox Gaussian with the given seed."""
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    l = k + p
    Om = sketch(DIST_GAUSSIAN, n, l, key0=seed, quantized=quantized)
    Q = orth(A @ Om)
    for _ in range(q):
        Z = orth(A.T @ Q)
        Q = orth(A @ Z)
    B = Q.T @ A
    U, sig, Vt = np.linalg.svd(B, full_matrices=False)
    r = min(k, Q.shape[1])
    return Q @ U[:, :r], sig[:r], Vt[:r, :]


def make_lowrank_test_matrix(m, n, sigma, seed_u, seed_v):
    """A = U diag(sigma) V^T with U, V the Q factors of seeded standard
    Gaussian matrices (numpy PCG64 generators)."""
    r = len(sigma)
    U = np.linalg.qr(np.random.default_rng(seed_u).standard_normal((m, r)))[0]
    V = np.linalg.qr(np.random.default_rng(seed_v).standard_normal((n, r)))[0]
    return (U * sigma) @ V.T
