"""vfmm_advance loads only the fields a step reads from the caller's records
and sets the others to NaN on the device (uvlm_gb300/csrc/api.cu
`advance_input_fields`).  A field left out that the step reads, or that it
should pass through, would come back as NaN: every field of the records after
two steps must be finite, for every scheme, formulation and viscous model, in
FP64 and mixed precision.  The registered (mapped) host path, where the
transposing kernel reads the records over the host link, must give the same
records, bit for bit, as the pageable path."""
import numpy as np
import pytest

from uvlm_gb300 import BODY_DTYPE, FMMCalculator, workloads
from uvlm_gb300._lib import lib

pytestmark = pytest.mark.gpu


def start(n: int, seed: int = 13) -> np.ndarray:
    b = workloads.cloud(n, seed=seed)
    rng = np.random.default_rng(seed)
    for f in BODY_DTYPE.names:
        if f not in ("X", "alpha", "radius"):
            b[f] = rng.standard_normal(b[f].shape)
    return b


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("integration", ["Euler", "RK2", "RK3", "RK4"])
@pytest.mark.parametrize("formulation,viscous,relax", [("cVPM", "Inviscid", 0.0), ("rVPM", "Inviscid", 0.0),
                                                       ("cVPM", "PSE", 0.0), ("cVPM", "CSM", 0.3)])
def test_advance_fields_finite(vfmm_lib, precision, integration, formulation, viscous, relax):
    b = start(3000)
    with FMMCalculator(p=6, ncrit=32, theta=0.5, integration=integration, formulation=formulation, viscous=viscous,
                       nu=1e-3 if viscous != "Inviscid" else 0.0, relax=relax, precision=precision) as c:
        for _ in range(2):
            c.advance(b, 0.01)
    for f in BODY_DTYPE.names:
        assert np.isfinite(b[f]).all(), f


@pytest.mark.parametrize("integration", ["RK2", "RK3"])
def test_registered_records_match_pageable(vfmm_lib, integration):
    a = start(40000, seed=3)
    b = a.copy()
    L = lib()
    assert L.vfmm_host_register(b.ctypes.data, b.nbytes) == 0
    try:
        with FMMCalculator(p=8, ncrit=64, theta=0.5, integration=integration, precision="mixed") as c:
            c.advance(b, 0.01)
    finally:
        L.vfmm_host_unregister(b.ctypes.data)
    with FMMCalculator(p=8, ncrit=64, theta=0.5, integration=integration, precision="mixed") as c:
        c.advance(a, 0.01)
    for f in BODY_DTYPE.names:
        assert (a[f] == b[f]).all(), f
        assert np.isfinite(b[f]).all(), f
