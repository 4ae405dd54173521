"""The bounded device waits: a wait that cannot complete gives up after its
limit and comes back as RNLA_ERR_TIMEOUT, and the CUDA context keeps
working (a solve afterwards matches LAPACK)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1])
def test_expired_wait_reports_timeout_and_context_survives(rnla, which):
    lib = rnla.lib()
    t0 = time.perf_counter()
    rc = lib.rnla_check_bounded_wait(which, 100000, None)     # 0.1 s limit
    dt = time.perf_counter() - t0
    assert rc == rnla.DeviceTimeout.code, (rc, lib.rnla_last_error_message())
    assert "exceeded its limit" in lib.rnla_last_error_message().decode()
    assert 0.09 < dt < 10.0
    rng = np.random.default_rng(which)
    a = rng.standard_normal((3000, 20))
    b = rng.standard_normal(3000)
    x = rnla.blendenpik_overdetermined(a, b, 1e-12, 500, 4.0,
                                       rnla.options(inner_solver=rnla.InnerSolver.LSQR, atol=1e-14, btol=1e-14))
    xl = np.linalg.lstsq(a, b, rcond=None)[0]
    np.testing.assert_allclose(x.ravel(), xl, rtol=1e-9, atol=1e-12)


def test_bounded_wait_rejects_bad_arguments(rnla):
    lib = rnla.lib()
    assert lib.rnla_check_bounded_wait(2, 1000, None) == rnla.InvalidParameters.code
    assert lib.rnla_check_bounded_wait(0, 0, None) == rnla.InvalidParameters.code
