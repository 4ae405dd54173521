"""randnla_gb300 — GB300 (sm_103a) implementation of the randomized
linear-algebra hot path of the Rust crate `randblas` (divijkhaitan/randnla).

The functions below mirror the reference's public functions (same names,
argument meaning and error behaviour) over the C ABI of
librandnla_gb300.so; every computation runs on the GPU:

    sketching_operator        src/sketch.rs:102-130
    tsog1, RF1, QB1, Orth,    src/lora_helpers.rs:17-146
    Stabilizer
    rand_svd                  src/lora_drivers.rs:30-69
    blendenpik_overdetermined src/sketch_and_precondition.rs:26-59
    cgls                      src/cg.rs:18-61
    lsqr                      src/solvers.rs:115-278
    solve_upper_triangular_system  src/solvers.rs:22-41

Matrices are numpy arrays (converted to column-major float64, the layout of
nalgebra's DMatrix).  Errors raise RandNLAError subclasses named after the
reference's enum variants (src/errors.rs:3-14).  The `*_dev` functions take
torch CUDA tensors and work on the current torch stream.
"""
import ctypes
import enum

import numpy as np

from . import _lib
from ._lib import Options, Rng, Stats, LsqrResult, LsProblem

__all__ = [
    "DistributionType", "Precision", "Mode", "InnerSolver", "Generator", "RandNLAError",
    "sketching_operator", "tsog1", "RF1", "QB1", "Orth", "Stabilizer", "rand_svd", "rand_evd1", "rand_evd2",
    "blendenpik_overdetermined", "lsrn_overdetermined", "solve_batched_dev", "sap_chol_qrcp", "sketched_least_squares_qr",
    "sketched_least_squares_svd", "cgls",
    "lsqr", "solve_upper_triangular_system", "options", "lib",
]


class DistributionType(enum.IntEnum):
    """src/sketch.rs:9-13"""
    Gaussian = 0
    Uniform = 1
    Rademacher = 2


class Precision(enum.IntEnum):
    FP64 = 0
    BF16X = 1
    BF16 = 2


class Mode(enum.IntEnum):
    Reference = 0
    RandNLA = 1


class InnerSolver(enum.IntEnum):
    CGLS = 0
    LSQR = 1


class Generator(enum.IntEnum):
    Philox4x32 = 0
    ThreeFry2x64 = 1


class RandNLAError(Exception):
    """Base of the reference's RandNLAError variants (src/errors.rs:3-14)."""
    code = -1


def _variant(name, code):
    return type(name, (RandNLAError,), {"code": code})


InvalidParameters = _variant("InvalidParameters", 1)
InvalidDimensions = _variant("InvalidDimensions", 2)
NegativeDimensions = _variant("NegativeDimensions", 3)
NotOverdetermined = _variant("NotOverdetermined", 4)
NotSquare = _variant("NotSquare", 5)
SingularMatrix = _variant("SingularMatrix", 6)
MatrixDecompositionError = _variant("MatrixDecompositionError", 7)
NotHermitian = _variant("NotHermitian", 8)
NotPositiveSemiDefinite = _variant("NotPositiveSemiDefinite", 9)
ComputationError = _variant("ComputationError", 10)
CudaError = _variant("CudaError", 11)
DeviceTimeout = _variant("DeviceTimeout", 12)
Unsupported = _variant("Unsupported", 13)
_BY_CODE = {c.code: c for c in (InvalidParameters, InvalidDimensions, NegativeDimensions,
                                 NotOverdetermined, NotSquare, SingularMatrix,
                                 MatrixDecompositionError, NotHermitian, NotPositiveSemiDefinite,
                                 ComputationError, CudaError, DeviceTimeout, Unsupported)}
__all__ += [c.__name__ for c in _BY_CODE.values()]


def lib():
    return _lib.load()


def _check(rc):
    if rc != 0:
        msg = lib().rnla_last_error_message().decode(errors="replace")
        raise _BY_CODE.get(rc, RandNLAError)(msg)


def _f64(a, ndim=2):
    a = np.asarray(a, dtype=np.float64)
    if ndim == 2 and a.ndim == 1:
        a = a.reshape(-1, 1)
    return np.asfortranarray(a)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def options(precision=Precision.FP64, mode=Mode.Reference, inner_solver=InnerSolver.CGLS,
            power_iters=2, generator=Generator.Philox4x32, seed=0, key1=0, atol=0.0, btol=0.0,
            conlim=1e8, digits_a=0, digits_b=0, orth=0):
    o = Options()
    lib().rnla_options_default(ctypes.byref(o))
    o.precision, o.mode, o.inner_solver, o.power_iters = int(precision), int(mode), int(inner_solver), power_iters
    o.rng.generator, o.rng.key0, o.rng.key1 = int(generator), seed, key1
    o.atol, o.btol, o.conlim = atol, btol, conlim
    o.digits_a, o.digits_b, o.orth = digits_a, digits_b, orth
    return o


def _rng(generator=Generator.Philox4x32, key0=0, key1=0):
    r = Rng()
    r.generator, r.key0, r.key1 = int(generator), key0, key1
    return r


# ---------------------------------------------------------------------------
# sketch.rs
# ---------------------------------------------------------------------------
def sketching_operator(dist_type, rows, cols, generator=Generator.Philox4x32, seed=0, key1=0):
    """src/sketch.rs:102-130.  Dense rows x cols operator (column-major)."""
    out = np.empty((max(rows, 1), max(cols, 1)), dtype=np.float64, order="F")
    r = _rng(generator, seed, key1)
    _check(lib().rnla_sketching_operator_ex(int(dist_type), rows, cols, ctypes.byref(r),
                                            _ptr(out), max(rows, 1)))
    return out


def rng_words(first_word, n, generator=Generator.Philox4x32, key0=0, key1=0):
    """Word stream of Philox4x32 / ThreeFry2x64 (rust-random123), computed on the GPU."""
    out = np.empty(n, dtype=np.uint32)
    r = _rng(generator, key0, key1)
    _check(lib().rnla_rng_words(ctypes.byref(r), first_word, n, _ptr(out)))
    return out


# ---------------------------------------------------------------------------
# solvers.rs / cg.rs
# ---------------------------------------------------------------------------
def solve_upper_triangular_system(u, y):
    """src/solvers.rs:22-41.  Returns an n x 1 matrix."""
    u = _f64(u)
    y = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
    n = u.shape[0]
    x = np.zeros(n)
    _check(lib().rnla_solve_upper_triangular_system(_ptr(u), n, max(n, 1), _ptr(y), _ptr(x)))
    return x.reshape(-1, 1)


def lsqr(a, b, damp=0.0, atol=1e-8, btol=1e-8, conlim=1e8, iter_lim=None, calc_var=False, x0=None):
    """src/solvers.rs:115-278.  Returns the reference's 10-tuple
    (x, istop, itn, r1norm, r2norm, anorm, acond, arnorms, xnorm, var)."""
    a = _f64(a)
    m, n = a.shape
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(-1))
    il = 2 * n if iter_lim is None else int(iter_lim)
    x = np.zeros(n)
    var = np.zeros(n)
    arn = np.zeros(max(il, 1))
    x0a = None if x0 is None else np.ascontiguousarray(np.asarray(x0, dtype=np.float64).reshape(-1))
    res = LsqrResult()
    _check(lib().rnla_lsqr(_ptr(a), m, n, max(m, 1), _ptr(b), damp, atol, btol, conlim, il,
                           int(bool(calc_var)), _ptr(x0a), _ptr(x), ctypes.byref(res), _ptr(arn),
                           _ptr(var)))
    cnt = res.itn if res.itn > 0 else 1
    return (x, int(res.istop), int(res.itn), res.r1norm, res.r2norm, res.anorm, res.acond,
            list(arn[:cnt]), res.xnorm, var)


def cgls(a, b, tolerance, num_iterations, x=None, return_iterations=False):
    """src/cg.rs:18-61.  Returns x (n x 1)."""
    a = _f64(a)
    m, n = a.shape
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(-1))
    x0 = None if x is None else np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
    out = np.zeros(n)
    it = ctypes.c_int64(0)
    _check(lib().rnla_cgls(_ptr(a), m, n, max(m, 1), _ptr(b), tolerance, num_iterations, _ptr(x0),
                           _ptr(out), ctypes.byref(it)))
    return (out.reshape(-1, 1), it.value) if return_iterations else out.reshape(-1, 1)


# ---------------------------------------------------------------------------
# lora_helpers.rs / lora_drivers.rs
# ---------------------------------------------------------------------------
def Orth(X):
    """src/lora_helpers.rs:131-133."""
    X = _f64(X)
    m, n = X.shape
    q = np.zeros((m, min(m, n)), order="F")
    _check(lib().rnla_orth(_ptr(X), m, n, max(m, 1), _ptr(q), max(m, 1)))
    return q


def Stabilizer(X):
    """src/lora_helpers.rs:144-146."""
    X = _f64(X)
    m, n = X.shape
    L = np.zeros((m, min(m, n)), order="F")
    _check(lib().rnla_stabilizer(_ptr(X), m, n, max(m, 1), _ptr(L), max(m, 1)))
    return L


def tsog1(A, k, num_passes, passes_per_stab):
    """src/lora_helpers.rs:58-105."""
    A = _f64(A)
    m, n = A.shape
    S = np.zeros((n, max(k, 1) + m), order="F")
    cols = ctypes.c_int64(0)
    _check(lib().rnla_tsog1(_ptr(A), m, n, max(m, 1), k, num_passes, passes_per_stab, _ptr(S),
                            max(n, 1), ctypes.byref(cols)))
    return np.asfortranarray(S[:, :cols.value])


def RF1(A, k):
    """src/lora_helpers.rs:37-44."""
    A = _f64(A)
    m, n = A.shape
    Q = np.zeros((m, max(k, 1)), order="F")
    cols = ctypes.c_int64(0)
    _check(lib().rnla_rf1(_ptr(A), m, n, max(m, 1), k, _ptr(Q), max(m, 1), ctypes.byref(cols)))
    return np.asfortranarray(Q[:, :cols.value])


def QB1(A, k, epsilon):
    """src/lora_helpers.rs:17-23 (epsilon ignored as in the reference)."""
    A = _f64(A)
    m, n = A.shape
    Q = np.zeros((m, max(k, 1)), order="F")
    B = np.zeros((max(k, 1), n), order="F")
    cols = ctypes.c_int64(0)
    _check(lib().rnla_qb1(_ptr(A), m, n, max(m, 1), k, epsilon, _ptr(Q), max(m, 1), _ptr(B),
                          max(k, 1), ctypes.byref(cols)))
    c = cols.value
    return np.asfortranarray(Q[:, :c]), np.asfortranarray(B[:c, :])


def rand_svd(A, k, epsilon, s, opts=None, return_stats=False):
    """src/lora_drivers.rs:30-69.  Returns (U m x r, S r x r, Vt r x n)."""
    A = _f64(A)
    m, n = A.shape
    o = opts if opts is not None else options()
    rmax = max(int(lib().rnla_rand_svd_rank(m, n, k, s, o.mode)), 1)
    U = np.zeros((m, rmax), order="F")
    S = np.zeros((rmax, rmax), order="F")
    Vt = np.zeros((rmax, n), order="F")
    r = ctypes.c_int64(0)
    st = Stats()
    _check(lib().rnla_rand_svd_ex(_ptr(A), m, n, max(m, 1), k, epsilon, s, ctypes.byref(o), _ptr(U),
                                  max(m, 1), _ptr(S), rmax, _ptr(Vt), rmax, ctypes.byref(r),
                                  ctypes.byref(st)))
    rr = r.value
    out = (np.asfortranarray(U[:, :rr]), np.asfortranarray(S[:rr, :rr]), np.asfortranarray(Vt[:rr, :]))
    return out + (st.as_dict(),) if return_stats else out


def rand_evd1(A, k, epsilon, s):
    """src/lora_drivers.rs:84-140.  Returns (V n x r, lambda list of r)."""
    A = _f64(A)
    n = A.shape[0]
    if A.shape[1] != n:
        raise InvalidDimensions("A must be square")
    kk = max(int(k), 1)
    V = np.zeros((n, kk), order="F")
    lam = np.zeros(kk)
    r = ctypes.c_int64(0)
    _check(lib().rnla_rand_evd1(_ptr(A), n, max(n, 1), k, epsilon, s, _ptr(V), max(n, 1), _ptr(lam),
                                ctypes.byref(r)))
    return np.asfortranarray(V[:, :r.value]), [float(x) for x in lam[:r.value]]


def rand_evd2(A, k, s):
    """src/lora_drivers.rs:153-213.  Returns (V n x r, lambda list of r)."""
    A = _f64(A)
    n = A.shape[0]
    if A.shape[1] != n:
        raise InvalidDimensions("A must be square")
    kk = max(int(k), 1)
    V = np.zeros((n, kk), order="F")
    lam = np.zeros(kk)
    r = ctypes.c_int64(0)
    _check(lib().rnla_rand_evd2(_ptr(A), n, max(n, 1), k, s, _ptr(V), max(n, 1), _ptr(lam), ctypes.byref(r)))
    return np.asfortranarray(V[:, :r.value]), [float(x) for x in lam[:r.value]]


# ---------------------------------------------------------------------------
# sketch_and_precondition.rs
# ---------------------------------------------------------------------------
def blendenpik_overdetermined(a, b, epsilon, l, sampling_factor, opts=None, return_stats=False):
    """src/sketch_and_precondition.rs:26-59.  Returns x (n x 1)."""
    a = _f64(a)
    m, n = a.shape
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(-1))
    x = np.zeros(n)
    o = opts if opts is not None else options()
    st = Stats()
    _check(lib().rnla_blendenpik_overdetermined_ex(_ptr(a), m, n, max(m, 1), _ptr(b), epsilon, l,
                                                   sampling_factor, ctypes.byref(o), _ptr(x),
                                                   ctypes.byref(st)))
    return (x.reshape(-1, 1), st.as_dict()) if return_stats else x.reshape(-1, 1)


def lsrn_overdetermined(a, b, epsilon, l, sampling_factor, opts=None, return_stats=False):
    """src/sketch_and_precondition.rs:82-119.  Returns x (n x 1)."""
    a = _f64(a)
    m, n = a.shape
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(-1))
    x = np.zeros(n)
    o = opts if opts is not None else options()
    st = Stats()
    _check(lib().rnla_lsrn_overdetermined_ex(_ptr(a), m, n, max(m, 1), _ptr(b), epsilon, l,
                                             sampling_factor, ctypes.byref(o), _ptr(x), ctypes.byref(st)))
    return (x.reshape(-1, 1), st.as_dict()) if return_stats else x.reshape(-1, 1)


# ---------------------------------------------------------------------------
# cqrrpt.rs
# ---------------------------------------------------------------------------
def sap_chol_qrcp(a, d, opts=None):
    """src/cqrrpt.rs:27-58.  Returns (q m x n, r n x n, j) with a[:, j] = q r."""
    a = _f64(a)
    m, n = a.shape
    q = np.zeros((m, n), order="F")
    r = np.zeros((n, n), order="F")
    j = np.zeros(n, dtype=np.int64)
    o = opts if opts is not None else options()
    _check(lib().rnla_sap_chol_qrcp(_ptr(a), m, n, max(m, 1), d, ctypes.byref(o), _ptr(q), max(m, 1),
                                    _ptr(r), max(n, 1), _ptr(j)))
    return q, r, [int(v) for v in j]


# ---------------------------------------------------------------------------
# sketch_and_solve.rs
# ---------------------------------------------------------------------------
def _sketched_ls(entry, a, b, opts):
    a = _f64(a)
    m, n = a.shape
    b = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(-1))
    x = np.zeros(n)
    o = opts if opts is not None else options()
    _check(entry(_ptr(a), m, n, max(m, 1), _ptr(b), ctypes.byref(o), _ptr(x)))
    return x.reshape(-1, 1)


def sketched_least_squares_qr(a, b, opts=None):
    """src/sketch_and_solve.rs:24-33: QR of the m/4-row Gaussian sketch.  Returns x (n x 1)."""
    return _sketched_ls(lib().rnla_sketched_least_squares_qr, a, b, opts)


def sketched_least_squares_svd(a, b, opts=None):
    """src/sketch_and_solve.rs:53-65: SVD of the m/4-row Gaussian sketch.  Returns x (n x 1)."""
    return _sketched_ls(lib().rnla_sketched_least_squares_svd, a, b, opts)


# ---------------------------------------------------------------------------
# Device-pointer forms (torch CUDA tensors, current torch stream)
# ---------------------------------------------------------------------------
def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dptr(t):
    """Device pointer of a torch CUDA tensor on the current device (None
    passes through).  Any other tensor is refused here, before the library
    could use its address as device memory."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor, got one on %s" % t.device)
    import torch
    if t.device.index != torch.cuda.current_device():
        raise ValueError("tensor on %s, but the current device is cuda:%d"
                         % (t.device, torch.cuda.current_device()))
    return ctypes.c_void_p(t.data_ptr())


def _ld(t):
    """Leading dimension of a column-major (Fortran-strided) 2-D torch tensor."""
    if t.dim() == 1:
        return max(t.shape[0], 1)
    assert t.stride(0) == 1, "expected a column-major tensor (stride(0) == 1)"
    return max(t.stride(1), t.shape[0], 1)


def blendenpik_dev(a, b, x, epsilon, l, sampling_factor, opts=None):
    """rnla_blendenpik_overdetermined_dev on torch CUDA tensors (a: m x n
    float64/float32 column-major, b: m float64, x: n float64 output)."""
    import torch
    o = opts if opts is not None else options()
    st = Stats()
    m, n = a.shape
    _check(lib().rnla_blendenpik_overdetermined_dev(
        _dptr(a), int(a.dtype == torch.float32), m, n, _ld(a), _dptr(b), epsilon, l, sampling_factor,
        ctypes.byref(o), _dptr(x), ctypes.byref(st), _stream()))
    return st.as_dict()


def lsrn_dev(a, b, x, epsilon, l, sampling_factor, opts=None):
    """rnla_lsrn_overdetermined_dev on torch CUDA tensors (same conventions
    as blendenpik_dev)."""
    import torch
    o = opts if opts is not None else options()
    st = Stats()
    m, n = a.shape
    _check(lib().rnla_lsrn_overdetermined_dev(
        _dptr(a), int(a.dtype == torch.float32), m, n, _ld(a), _dptr(b), epsilon, l, sampling_factor,
        ctypes.byref(o), _dptr(x), ctypes.byref(st), _stream()))
    return st.as_dict()


def solve_batched_dev(problems, epsilon, l, sampling_factor, opts=None):
    """rnla_solve_batched: problems is a sequence of (a, b, x) torch CUDA
    tensors as for blendenpik_dev.  Returns (statuses, stats): one status
    code and one stats dict per problem; a failing problem does not stop
    the others, and nothing is raised for it (a CUDA error is raised)."""
    import torch
    o = opts if opts is not None else options()
    count = len(problems)
    arr = (LsProblem * max(count, 1))()
    for i, (a, b, x) in enumerate(problems):
        m, n = a.shape
        arr[i] = LsProblem(_dptr(a), int(a.dtype == torch.float32), 0, m, n, _ld(a), _dptr(b), _dptr(x))
    status = (ctypes.c_int32 * max(count, 1))()
    st = (Stats * max(count, 1))()
    rc = lib().rnla_solve_batched(arr, count, epsilon, l, sampling_factor, ctypes.byref(o), status, st,
                                  _stream())
    if rc == CudaError.code:
        _check(rc)
    return [int(status[i]) for i in range(count)], [st[i].as_dict() for i in range(count)]


def sketched_least_squares_dev(a, b, x, use_svd=False, opts=None):
    """rnla_sketched_least_squares_dev on torch CUDA tensors (a: m x n
    float64/float32 column-major, b: m float64, x: n float64 output)."""
    import torch
    o = opts if opts is not None else options()
    m, n = a.shape
    _check(lib().rnla_sketched_least_squares_dev(_dptr(a), int(a.dtype == torch.float32), m, n, _ld(a),
                                                 _dptr(b), int(bool(use_svd)), ctypes.byref(o), _dptr(x),
                                                 _stream()))


def rand_svd_dev(a, k, epsilon, s, U, sigma, Vt, opts=None):
    import torch
    o = opts if opts is not None else options()
    st = Stats()
    r = ctypes.c_int64(0)
    m, n = a.shape
    _check(lib().rnla_rand_svd_dev(_dptr(a), int(a.dtype == torch.float32), m, n, _ld(a), k, epsilon,
                                   s, ctypes.byref(o), _dptr(U), _ld(U), _dptr(sigma), _dptr(Vt),
                                   _ld(Vt), ctypes.byref(r), ctypes.byref(st), _stream()))
    return r.value, st.as_dict()


def sketch_apply_dev(x, d, y, precision=Precision.FP64, digits=0, generator=Generator.Philox4x32,
                     seed=0, dist_type=DistributionType.Gaussian):
    """y (d x n, column-major float64) = S x for the sketch S (d x m) of
    `dist_type` (quantised under Precision.BF16X)."""
    import torch
    r = _rng(generator, seed)
    m, n = x.shape
    _check(lib().rnla_sketch_apply_ex_dev(_dptr(x), int(x.dtype == torch.float32), m, n, _ld(x), d,
                                          int(dist_type), ctypes.byref(r), int(precision), digits, _dptr(y),
                                          _ld(y), _stream()))


def sketching_operator_dev(out, dist_type=DistributionType.Gaussian, quantized=False,
                           generator=Generator.Philox4x32, seed=0):
    import torch
    r = _rng(generator, seed)
    rows, cols = out.shape
    if out.dtype == torch.float32:
        _check(lib().rnla_sketching_operator_f32_dev(int(dist_type), rows, cols, ctypes.byref(r),
                                                     int(quantized), _dptr(out), _ld(out), _stream()))
    else:
        _check(lib().rnla_sketching_operator_dev(int(dist_type), rows, cols, ctypes.byref(r),
                                                 _dptr(out), _ld(out), _stream()))


def gemm_tn_dev(x, y, c, precision=Precision.FP64, digits_x=0, digits_y=0):
    """c (mm x nn) = x^T y for column-major float64 tensors x (k x mm), y (k x nn)."""
    k, mm = x.shape
    _, nn = y.shape
    _check(lib().rnla_gemm_tn_dev(_dptr(x), k, mm, _ld(x), _dptr(y), nn, _ld(y), int(precision),
                                  digits_x, digits_y, _dptr(c), _ld(c), _stream()))
