import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libvfmm.so")


@pytest.fixture(scope="session")
def vfmm_lib():
    """libvfmm.so, built for sm_103a if missing; loading failures are errors."""
    from uvlm_gb300 import _build, _lib
    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.lib()


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def golden_bodies(d):
    from uvlm_gb300._lib import BODY_DTYPE
    b = np.zeros(len(d["X"]), BODY_DTYPE)
    b["X"] = d["X"]
    b["alpha"] = d["alpha"]
    b["radius"] = d["radius"]
    return b


def rel(a, b):
    """max |a - b| / max |b| (0 when both are zero)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.abs(b).max() if b.size else 0.0
    num = np.abs(a - b).max() if b.size else 0.0
    return 0.0 if den == 0 and num == 0 else num / den
