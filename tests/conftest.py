import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 host)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "golden_arrays.npz")))
    return meta, arrays


@pytest.fixture(scope="session")
def lib():
    """The C-ABI library, built in-tree if needed."""
    from suitesparse_gb300 import build, cholmod
    if not os.path.exists(cholmod.LIB_PATH):
        build.build()
    return cholmod.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    oracle.lib()
    return oracle


def make_case(meta, name):
    from suitesparse_gb300 import matrices as M
    rec = meta[name]
    if rec["kind"] == "batch":
        return M.batch_system(rec["kwargs"]["index"], rec["kwargs"]["side"])
    return getattr(M, rec["kind"])(**rec["kwargs"])
