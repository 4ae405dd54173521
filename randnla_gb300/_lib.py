"""ctypes binding of librandnla_gb300.so (include/randnla_gb300.h).

Loading fails loudly when the shared library has not been built: there is
no Python or CPU fallback for any compute entry point.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librandnla_gb300.so")

c_i32, c_i64, c_u32, c_u64, c_dbl, c_vp = (ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32,
                                           ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p)
P_dbl = ctypes.POINTER(ctypes.c_double)
P_i64 = ctypes.POINTER(ctypes.c_int64)


class Rng(ctypes.Structure):
    _fields_ = [("generator", c_i32), ("reserved", c_i32), ("key0", c_u64), ("key1", c_u64)]


class Options(ctypes.Structure):
    _fields_ = [("precision", c_i32), ("mode", c_i32), ("inner_solver", c_i32),
                ("power_iters", c_i32), ("rng", Rng), ("atol", c_dbl), ("btol", c_dbl),
                ("conlim", c_dbl), ("digits_a", c_i32), ("digits_b", c_i32), ("orth", c_i32),
                ("reserved", c_i32)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", c_i64), ("istop", c_i64), ("r1norm", c_dbl), ("r2norm", c_dbl),
                ("anorm", c_dbl), ("acond", c_dbl), ("arnorm", c_dbl), ("xnorm", c_dbl),
                ("sketch_rows", c_i64), ("rank", c_i64), ("orth_fallbacks", c_i32),
                ("precision_used", c_i32), ("ms_sketch", c_dbl), ("ms_factor", c_dbl),
                ("ms_solve", c_dbl), ("ms_total", c_dbl), ("ms_kernel", c_dbl), ("svd_sweeps", c_i64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class LsProblem(ctypes.Structure):
    _fields_ = [("a", c_vp), ("a_is_f32", c_i32), ("reserved", c_i32), ("m", c_i64), ("n", c_i64),
                ("lda", c_i64), ("b", c_vp), ("x", c_vp)]


class LsqrResult(ctypes.Structure):
    _fields_ = [("istop", c_i64), ("itn", c_i64), ("r1norm", c_dbl), ("r2norm", c_dbl),
                ("anorm", c_dbl), ("acond", c_dbl), ("xnorm", c_dbl)]


# (name, restype, argtypes) for every symbol declared in include/randnla_gb300.h
SIGNATURES = [
    ("rnla_last_error_message", ctypes.c_char_p, []),
    ("rnla_version", ctypes.c_char_p, []),
    ("rnla_device_count", ctypes.c_int, []),
    ("rnla_kernel_launches", c_u64, []),
    ("rnla_rng_words", ctypes.c_int, [ctypes.POINTER(Rng), c_u64, c_i64, c_vp]),
    ("rnla_rng_words_dev", ctypes.c_int, [ctypes.POINTER(Rng), c_u64, c_i64, c_vp, c_vp]),
    ("rnla_sketching_operator", ctypes.c_int, [c_i32, c_i64, c_i64, c_vp, c_i64]),
    ("rnla_sketching_operator_ex", ctypes.c_int, [c_i32, c_i64, c_i64, ctypes.POINTER(Rng), c_vp, c_i64]),
    ("rnla_sketching_operator_dev", ctypes.c_int,
     [c_i32, c_i64, c_i64, ctypes.POINTER(Rng), c_vp, c_i64, c_vp]),
    ("rnla_sketching_operator_f32_dev", ctypes.c_int,
     [c_i32, c_i64, c_i64, ctypes.POINTER(Rng), c_i32, c_vp, c_i64, c_vp]),
    ("rnla_options_default", None, [ctypes.POINTER(Options)]),
    ("rnla_solve_upper_triangular_system", ctypes.c_int, [c_vp, c_i64, c_i64, c_vp, c_vp]),
    ("rnla_solve_upper_triangular_system_dev", ctypes.c_int, [c_vp, c_i64, c_i64, c_vp, c_vp, c_vp]),
    ("rnla_lsqr", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_dbl, c_dbl, c_dbl, c_i64, c_i32, c_vp, c_vp,
      ctypes.POINTER(LsqrResult), c_vp, c_vp]),
    ("rnla_lsqr_dev", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_dbl, c_dbl, c_dbl, c_i64, c_i32, c_vp, c_vp,
      ctypes.POINTER(LsqrResult), c_vp, c_vp, c_vp]),
    ("rnla_lsqr_noalloc_dev", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_dbl, c_dbl, c_dbl, c_i64, c_vp, c_vp,
      ctypes.POINTER(LsqrResult), c_vp]),
    ("rnla_cgls", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_vp, c_vp, P_i64]),
    ("rnla_cgls_dev", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_vp, c_vp, P_i64, c_vp]),
    ("rnla_orth", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    ("rnla_stabilizer", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64]),
    ("rnla_tsog1", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_i64, c_i32, c_i32, c_vp, c_i64, P_i64]),
    ("rnla_rf1", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_i64, P_i64]),
    ("rnla_qb1", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_i64, c_dbl, c_vp, c_i64, c_vp, c_i64, P_i64]),
    ("rnla_rand_svd_rank", c_i64, [c_i64, c_i64, c_i64, c_i64, c_i32]),
    ("rnla_rand_evd1", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_dbl, c_i64, c_vp, c_i64, c_vp, P_i64]),
    ("rnla_rand_evd2", ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_i64, c_vp, P_i64]),
    ("rnla_rand_svd", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_i64, c_dbl, c_i64, c_vp, c_i64, c_vp, c_i64, c_vp, c_i64, P_i64]),
    ("rnla_rand_svd_ex", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_i64, c_dbl, c_i64, ctypes.POINTER(Options), c_vp, c_i64, c_vp,
      c_i64, c_vp, c_i64, P_i64, ctypes.POINTER(Stats)]),
    ("rnla_rand_svd_dev", ctypes.c_int,
     [c_vp, c_i32, c_i64, c_i64, c_i64, c_i64, c_dbl, c_i64, ctypes.POINTER(Options), c_vp, c_i64,
      c_vp, c_vp, c_i64, P_i64, ctypes.POINTER(Stats), c_vp]),
    ("rnla_blendenpik_overdetermined", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, c_vp]),
    ("rnla_blendenpik_overdetermined_ex", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, ctypes.POINTER(Options), c_vp,
      ctypes.POINTER(Stats)]),
    ("rnla_blendenpik_overdetermined_f32_ex", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, ctypes.POINTER(Options), c_vp,
      ctypes.POINTER(Stats)]),
    ("rnla_blendenpik_overdetermined_dev", ctypes.c_int,
     [c_vp, c_i32, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, ctypes.POINTER(Options), c_vp,
      ctypes.POINTER(Stats), c_vp]),
    ("rnla_lsrn_overdetermined", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, c_vp]),
    ("rnla_lsrn_overdetermined_ex", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, ctypes.POINTER(Options), c_vp,
      ctypes.POINTER(Stats)]),
    ("rnla_lsrn_overdetermined_dev", ctypes.c_int,
     [c_vp, c_i32, c_i64, c_i64, c_i64, c_vp, c_dbl, c_i64, c_dbl, ctypes.POINTER(Options), c_vp,
      ctypes.POINTER(Stats), c_vp]),
    ("rnla_release_cached_memory", ctypes.c_int, []),
    ("rnla_check_bounded_wait", ctypes.c_int, [c_i32, c_i64, c_vp]),
    ("rnla_solve_batched", ctypes.c_int,
     [ctypes.POINTER(LsProblem), c_i64, c_dbl, c_i64, c_dbl, ctypes.POINTER(Options),
      ctypes.POINTER(c_i32), ctypes.POINTER(Stats), c_vp]),
    ("rnla_sap_chol_qrcp", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_i64, ctypes.POINTER(Options), c_vp, c_i64, c_vp, c_i64, c_vp]),
    ("rnla_sap_chol_qrcp_dev", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_i64, ctypes.POINTER(Options), c_vp, c_i64, c_vp, c_i64, c_vp, c_vp]),
    ("rnla_sketched_least_squares_qr", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, ctypes.POINTER(Options), c_vp]),
    ("rnla_sketched_least_squares_svd", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, ctypes.POINTER(Options), c_vp]),
    ("rnla_sketched_least_squares_dev", ctypes.c_int,
     [c_vp, c_i32, c_i64, c_i64, c_i64, c_vp, c_i32, ctypes.POINTER(Options), c_vp, c_vp]),
    ("rnla_sketch_apply_ex_dev", ctypes.c_int,
     [c_vp, c_i32, c_i64, c_i64, c_i64, c_i64, c_i32, ctypes.POINTER(Rng), c_i32, c_i32, c_vp, c_i64, c_vp]),
    ("rnla_sketch_apply_dev", ctypes.c_int,
     [c_vp, c_i32, c_i64, c_i64, c_i64, c_i64, ctypes.POINTER(Rng), c_i32, c_i32, c_vp, c_i64, c_vp]),
    ("rnla_gemm_tn_dev", ctypes.c_int,
     [c_vp, c_i64, c_i64, c_i64, c_vp, c_i64, c_i64, c_i32, c_i32, c_i32, c_vp, c_i64, c_vp]),
]

_LIB = None


def load():
    """Load and bind the library; raises if it was not built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError("librandnla_gb300.so is not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib
