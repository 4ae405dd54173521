import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    import json
    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "rng_kat.json")) as f:
        rng = json.load(f)
    with open(os.path.join(d, "solver_kat.json")) as f:
        solv = json.load(f)
    return {"rng": rng, "solvers": solv}


@pytest.fixture(scope="session")
def rnla():
    """The product library; GPU tests fail (not skip) when it is missing."""
    import randnla_gb300 as R
    R.lib()
    return R
