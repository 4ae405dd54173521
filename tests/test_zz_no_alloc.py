"""The allocation-free LSQR entry point (rnla_lsqr_noalloc_dev) against the
regular one (rnla_lsqr_dev), through the C ABI, on two calls in a row.

It exists for callers that cannot let a library allocate device memory
(a fixed budget owned by their own allocator, or loops that must not pay
cudaMalloc/cudaFree per call); its scratch is a fixed array inside the
library.  This file is collected last so a failure here leaves every other
test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, fn, A, b, x, extra_dev):
    import torch
    from randnla_gb300 import _lib
    res = _lib.LsqrResult()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    m, n = A.shape
    args = [ctypes.c_void_p(A.data_ptr()), m, n, A.stride(1), ctypes.c_void_p(b.data_ptr()), 0.0, 1e-12,
            1e-12, 1e8, 4 * n]
    if extra_dev:     # rnla_lsqr_dev: calc_var, x0, x, result, arnorms, var, stream
        rc = fn(*args, 0, None, ctypes.c_void_p(x.data_ptr()), ctypes.byref(res), None, None, s)
    else:             # rnla_lsqr_noalloc_dev: x0, x, result, stream
        rc = fn(*args, None, ctypes.c_void_p(x.data_ptr()), ctypes.byref(res), s)
    assert rc == 0, lib.rnla_last_error_message().decode()
    torch.cuda.synchronize()
    return res


# (3000, 40) and (20000, 300) take the streaming kernel (n <= 1024); (4001,
# 1500) the staged kernel with an odd m, so the vectors carved after u start
# on an 8-byte (not 16-byte) boundary; (6000, 4096) the largest n.
@pytest.mark.parametrize("m,n", [(3000, 40), (20000, 300), (4001, 1500), (6000, 4096)])
def test_noalloc_matches_regular_entry_point_twice(rnla, m, n):
    import torch
    lib = rnla.lib()
    g = torch.Generator(device="cuda").manual_seed(m + n)
    A = torch.randn((n, m), generator=g, device="cuda", dtype=torch.float64).t()
    b = torch.randn(m, generator=g, device="cuda", dtype=torch.float64)
    x_ref = torch.empty(n, dtype=torch.float64, device="cuda")
    r_ref = _call(lib, lib.rnla_lsqr_dev, A, b, x_ref, True)
    for _ in range(2):
        x = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        r = _call(lib, lib.rnla_lsqr_noalloc_dev, A, b, x, False)
        assert r.istop == r_ref.istop and r.itn == r_ref.itn
        np.testing.assert_allclose(x.cpu().numpy(), x_ref.cpu().numpy(), rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose([r.r1norm, r.anorm, r.acond, r.xnorm],
                                   [r_ref.r1norm, r_ref.anorm, r_ref.acond, r_ref.xnorm], rtol=1e-12)


def test_noalloc_rejects_oversized_problem(rnla):
    import torch
    lib = rnla.lib()
    from randnla_gb300 import _lib
    m, n = 5_000_000, 2
    A = torch.zeros((1, 1), dtype=torch.float64, device="cuda")   # never read: rejected first
    res = _lib.LsqrResult()
    rc = lib.rnla_lsqr_noalloc_dev(ctypes.c_void_p(A.data_ptr()), m, n, m, ctypes.c_void_p(A.data_ptr()),
                                   0.0, 1e-8, 1e-8, 1e8, 10, None, ctypes.c_void_p(A.data_ptr()),
                                   ctypes.byref(res), None)
    assert rc == rnla.InvalidDimensions.code
    assert "needs" in lib.rnla_last_error_message().decode()


def test_noalloc_rejects_n_above_4096(rnla):
    import torch
    lib = rnla.lib()
    from randnla_gb300 import _lib
    m, n = 5000, 4097
    A = torch.zeros((1, 1), dtype=torch.float64, device="cuda")   # never read: rejected first
    res = _lib.LsqrResult()
    rc = lib.rnla_lsqr_noalloc_dev(ctypes.c_void_p(A.data_ptr()), m, n, m, ctypes.c_void_p(A.data_ptr()),
                                   0.0, 1e-8, 1e-8, 1e8, 10, None, ctypes.c_void_p(A.data_ptr()),
                                   ctypes.byref(res), None)
    assert rc == rnla.Unsupported.code
    assert "4096" in lib.rnla_last_error_message().decode()


def test_noalloc_rejects_sizes_that_would_overflow(rnla):
    import torch
    lib = rnla.lib()
    from randnla_gb300 import _lib
    A = torch.zeros((1, 1), dtype=torch.float64, device="cuda")   # never read: rejected first
    res = _lib.LsqrResult()
    m = 1 << 61
    rc = lib.rnla_lsqr_noalloc_dev(ctypes.c_void_p(A.data_ptr()), m, 2, m, ctypes.c_void_p(A.data_ptr()),
                                   0.0, 1e-8, 1e-8, 1e8, 10, None, ctypes.c_void_p(A.data_ptr()),
                                   ctypes.byref(res), None)
    assert rc == rnla.InvalidDimensions.code
