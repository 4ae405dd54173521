"""The C-ABI library loads and exports every symbol include/*.h declares.
No compute entry point is called here (this suite also runs without a GPU)."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            txt = f.read()
        names |= set(re.findall(r"^RNLA_API\s+[\w\s\*]+?\b(rnla_\w+)\s*\(", txt, re.M))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("rnla_sketching_operator", "rnla_rand_svd", "rnla_blendenpik_overdetermined",
                 "rnla_cgls", "rnla_lsqr", "rnla_solve_upper_triangular_system", "rnla_qb1",
                 "rnla_rf1", "rnla_tsog1", "rnla_orth", "rnla_stabilizer"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from randnla_gb300 import _lib
    assert os.path.exists(_lib.LIB_PATH), "library not built"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s+(rnla_\w+)", out))
    missing = declared_symbols() - exported
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert bound == declared_symbols()


def test_library_loads_and_answers_host_queries():
    import randnla_gb300 as R
    lib = R.lib()
    assert lib.rnla_version().decode().endswith("sm_103a")
    assert lib.rnla_device_count() >= 0
    o = R.options()
    assert o.precision == 0 and o.conlim == 1e8 and o.power_iters == 2
    # rank rule of lora_drivers.rs:51 with the reference shapes
    assert lib.rnla_rand_svd_rank(100, 50, 45, 2, 0) == 45
    assert lib.rnla_rand_svd_rank(5, 20, 3, 2, 0) == 3
    assert lib.rnla_rand_svd_rank(10, 2, 3, 2, 0) == 2


def test_python_mirror_declares_every_entry_point():
    """Every C entry point has a ctypes declaration in the Python mirror."""
    from randnla_gb300 import _lib
    with open(_lib.__file__) as f:
        declared = set(re.findall(r'\("(rnla_\w+)"', f.read()))
    assert declared == declared_symbols()


def test_struct_layouts_match_header():
    from randnla_gb300 import _lib
    assert ctypes.sizeof(_lib.Rng) == 24
    assert ctypes.sizeof(_lib.Options) == 16 + 24 + 24 + 16
    assert ctypes.sizeof(_lib.LsqrResult) == 16 + 5 * 8
    assert ctypes.sizeof(_lib.LsProblem) == 8 + 8 + 24 + 16


def test_release_cached_memory_before_any_gpu_call():
    import randnla_gb300 as R
    assert R.lib().rnla_release_cached_memory() == 0


def test_batched_argument_errors_need_no_device():
    """rnla_solve_batched rejects a negative count or missing arrays before
    touching the GPU; an empty batch is fine."""
    import randnla_gb300 as R
    lib = R.lib()
    st = (ctypes.c_int32 * 1)()
    assert lib.rnla_solve_batched(None, -1, 1e-8, 10, 4.0, None, st, None, None) == R.NegativeDimensions.code
    assert lib.rnla_solve_batched(None, 2, 1e-8, 10, 4.0, None, st, None, None) == R.InvalidParameters.code
    assert lib.rnla_solve_batched((R.LsProblem * 1)(), 1, 1e-8, 10, 4.0, None, None, None, None) \
        == R.InvalidParameters.code
    assert lib.rnla_solve_batched(None, 0, 1e-8, 10, 4.0, None, None, None, None) == 0
    # option enumerations are checked before any device work
    one = (R.LsProblem * 1)()
    for field, bad in (("precision", 7), ("mode", 3), ("inner_solver", 2)):
        o = R.options()
        setattr(o, field, bad)
        assert lib.rnla_solve_batched(one, 1, 1e-8, 10, 4.0, ctypes.byref(o), st, None, None) \
            == R.InvalidParameters.code, field


def test_no_oracle_in_product():
    """The product package never imports or loads the oracle."""
    for path in glob.glob(os.path.join(ROOT, "randnla_gb300", "**", "*"), recursive=True):
        if path.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
            with open(path) as f:
                txt = f.read()
            assert "oracle" not in txt.lower(), path


def test_device_wrappers_refuse_host_tensors():
    """The _dev wrappers check every tensor before the library sees its
    address: a CPU tensor is a ValueError, not a device access."""
    import torch
    import randnla_gb300 as R
    a = torch.zeros((100, 10), dtype=torch.float64).t().contiguous().t()
    b = torch.zeros(100, dtype=torch.float64)
    x = torch.zeros(10, dtype=torch.float64)
    with pytest.raises(ValueError):
        R.blendenpik_dev(a, b, x, 1e-8, 10, 4.0)
    with pytest.raises(ValueError):
        R.solve_batched_dev([(a, b, x)], 1e-8, 10, 4.0)
    assert R._dptr(None) is None
