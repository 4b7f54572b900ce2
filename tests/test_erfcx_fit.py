"""The mixed P2P kernel's erf-free form of g(rho) = erf(rho) - (2/sqrt(pi)) rho
e^(-rho^2): g = 1 - e^(-rho^2) (erfcx(rho) + (2/sqrt(pi)) rho) with a fitted
erfcx (constants in uvlm_gb300/csrc/mixed.cu).  Checked on the CPU in FP32
arithmetic against FP64 erf: the relative error of g stays within a few times
that of the FP32 erf form it replaced, band by band."""
import os
import re

import numpy as np
import pytest

scipy_special = pytest.importorskip("scipy.special")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def constants():
    src = open(os.path.join(ROOT, "uvlm_gb300", "csrc", "mixed.cu")).read()
    c = {k: float(v) for k, v in re.findall(r"constexpr float kErfcx(\w+)\s*=\s*([-0-9.e]+)f;", src)}
    return c["A"], [c[str(k)] for k in range(1, 6)]


def g_fp32(rho):
    """The kernel's operation sequence in FP32 (e^(-rho^2) correctly rounded)."""
    f32 = np.float32
    a, c = constants()
    r = rho.astype(f32)
    t = (f32(1) / (f32(a) * r + f32(1))).astype(f32)
    q = f32(c[4])
    for k in (3, 2, 1, 0):
        q = (q * t + f32(c[k])).astype(f32)
    kx = (r * f32(2 / np.sqrt(np.pi))).astype(f32)
    ex = np.exp(-(r.astype(np.float64)) ** 2).astype(f32)
    H = (q * t + kx).astype(f32)
    return (f32(1) - (ex * H).astype(f32)).astype(f32)


def test_fit_in_fp64():
    a, c = constants()
    rho = np.linspace(0.5, 14, 200001)
    t = 1 / (1 + a * rho)
    fit = t * (c[0] + t * (c[1] + t * (c[2] + t * (c[3] + t * c[4]))))
    ex = np.exp(-rho ** 2)
    g = scipy_special.erf(rho) - 2 / np.sqrt(np.pi) * rho * ex
    assert np.max(np.abs(ex * (fit - scipy_special.erfcx(rho))) / g) < 5e-8


@pytest.mark.parametrize("lo,hi,bound", [(0.5, 0.7, 3e-6), (0.7, 1.0, 1e-6), (1.0, 2.0, 4e-7), (2.0, 4.0, 1.5e-7), (4.0, 30.0, 6e-8)])
def test_fp32_error_band(lo, hi, bound):
    rho = np.linspace(lo, hi, 100001)
    g = scipy_special.erf(rho) - 2 / np.sqrt(np.pi) * rho * np.exp(-rho ** 2)
    rel = np.abs(g_fp32(rho).astype(np.float64) - g) / g
    assert rel.max() < bound and rel.mean() < bound / 4
