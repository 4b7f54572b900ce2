"""The oracle's whole-step complex-step checker (oracle/complex_step.hpp):
with T = double it is the same FMM step as the restatement of the reference
(vo_advance), and its complex-step derivatives agree with central
differences taken where no tree or list decision changes.  CPU only."""
import ctypes

import numpy as np

from oracle.oracle import oracle
from uvlm_gb300 import workloads


def advance_plain(L, b, scheme):
    bb = b.copy()
    assert L.vo_cs_advance(bb.ctypes.data, bb.size, 8, 32, 0.5, scheme, 0, 0.02, 2, 0.0, 0, 0, 0.0) == 0
    return bb


def test_templated_step_equals_the_reference_restatement():
    L = oracle()
    b = workloads.ring(16, seed=3)
    n = b.size
    b1, b2 = b.copy(), b.copy()
    assert L.vo_advance(b1.ctypes.data, n, 8, 32, 0.5, 0.02, 2, 2, 0, 0, 0.0, 0, 0, 0.0) == 0
    assert L.vo_cs_advance(b2.ctypes.data, n, 8, 32, 0.5, 2, 0, 0.02, 2, 0.0, 0, 0, 0.0) == 0
    for f, tol in (("X", 1e-14), ("alpha", 1e-14), ("velocity", 1e-12), ("J", 1e-11), ("dadt", 1e-11)):
        a, r = b2[f].reshape(n, -1), b1[f].reshape(n, -1)
        assert np.linalg.norm(a - r) <= tol * np.linalg.norm(r), f


def test_templated_rk4_equals_the_reference_restatement():
    """RK4 with the reference's half-step third stage (oracle scheme 3) and
    with a full-step one (scheme 4, rk4_fixed of the restatement)."""
    L = oracle()
    b = workloads.ring(16, seed=4)
    n = b.size
    for fixed in (0, 1):
        b1, b2 = b.copy(), b.copy()
        assert L.vo_advance(b1.ctypes.data, n, 8, 32, 0.5, 0.02, 2, 3, 0, 0, 0.0, fixed, 0, 0.0) == 0
        assert L.vo_cs_advance(b2.ctypes.data, n, 8, 32, 0.5, 3 + fixed, 0, 0.02, 2, 0.0, 0, 0, 0.0) == 0
        for f, tol in (("X", 1e-14), ("alpha", 1e-14), ("velocity", 1e-12), ("J", 1e-11), ("dadt", 1e-11)):
            a, r = b2[f].reshape(n, -1), b1[f].reshape(n, -1)
            assert np.linalg.norm(a - r) <= tol * np.linalg.norm(r), (fixed, f)


def test_templated_step_with_relaxation_equals_the_reference_restatement():
    """Relaxation after each step's last stage (relaxation.hpp:8-19) in the
    templated step against vo_advance's."""
    L = oracle()
    b = workloads.ring(16, seed=5)
    n = b.size
    for scheme in (0, 2):
        b1, b2 = b.copy(), b.copy()
        assert L.vo_advance(b1.ctypes.data, n, 8, 32, 0.5, 0.02, 2, scheme, 0, 0, 0.3, 0, 0, 0.0) == 0
        assert L.vo_cs_advance(b2.ctypes.data, n, 8, 32, 0.5, scheme, 0, 0.02, 2, 0.3, 0, 0, 0.0) == 0
        for f, tol in (("X", 1e-14), ("alpha", 1e-13), ("velocity", 1e-12), ("J", 1e-11), ("dadt", 1e-11)):
            a, r = b2[f].reshape(n, -1), b1[f].reshape(n, -1)
            assert np.linalg.norm(a - r) <= tol * np.linalg.norm(r), (scheme, f)
        assert not np.allclose(b2["alpha"], advance_plain(L, b, scheme)["alpha"], rtol=1e-6), "relaxation changed nothing"


def test_templated_rvpm_step_equals_the_reference_restatement():
    """The rVPM terms (fmmCalculator.hpp:407-418) and the radius updates of
    the templated step against vo_advance's, RK2 and RK3."""
    L = oracle()
    b = workloads.ring(16, seed=6)
    n = b.size
    for scheme in (1, 2):
        b1, b2 = b.copy(), b.copy()
        assert L.vo_advance(b1.ctypes.data, n, 8, 32, 0.5, 0.02, 2, scheme, 0, 1, 0.0, 0, 0, 0.0) == 0
        assert L.vo_cs_advance(b2.ctypes.data, n, 8, 32, 0.5, scheme, 0, 0.02, 2, 0.0, 1, 0, 0.0) == 0
        for f, tol in (("X", 1e-14), ("alpha", 1e-13), ("radius", 1e-14), ("drdt", 1e-11), ("velocity", 1e-12), ("J", 1e-11),
                       ("dadt", 1e-11)):
            a, r = b2[f].reshape(n, -1), b1[f].reshape(n, -1)
            assert np.linalg.norm(a - r) <= tol * np.linalg.norm(r), (scheme, f)
        assert not np.array_equal(b2["radius"], b["radius"]), "rVPM left the radii unchanged"


def test_templated_viscous_step_equals_the_reference_restatement():
    """PSE (multipoleKernels.hpp:415-450) and CSM (fmmCalculator.hpp:334-337)
    in the templated step against vo_advance's, RK2."""
    L = oracle()
    b = workloads.cloud(3000, seed=7)
    n = b.size
    for viscous in (1, 2):
        b1, b2 = b.copy(), b.copy()
        assert L.vo_advance(b1.ctypes.data, n, 8, 32, 0.5, 0.02, 2, 1, 0, 0, 0.0, 0, viscous, 0.01) == 0
        assert L.vo_cs_advance(b2.ctypes.data, n, 8, 32, 0.5, 1, 0, 0.02, 2, 0.0, 0, viscous, 0.01) == 0
        for f, tol in (("X", 1e-14), ("alpha", 1e-13), ("radius", 1e-14), ("velocity", 1e-12), ("J", 1e-11), ("dadt", 1e-11)):
            a, r = b2[f].reshape(n, -1), b1[f].reshape(n, -1)
            assert np.linalg.norm(a - r) <= tol * np.linalg.norm(r), (viscous, f)
        plain = b.copy()
        assert L.vo_cs_advance(plain.ctypes.data, n, 8, 32, 0.5, 1, 0, 0.02, 2, 0.0, 0, 0, 0.0) == 0
        changed = "alpha" if viscous == 1 else "radius"
        assert not np.allclose(b2[changed], plain[changed], rtol=1e-9, atol=0), (viscous, "viscosity changed nothing")


def test_complex_step_against_central_differences():
    L = oracle()
    b = workloads.ring(16, seed=3)
    n = b.size
    rng = np.random.default_rng(0)
    dx = rng.normal(size=(1, n, 3))
    da = rng.normal(size=(1, n, 3)) * np.abs(b["alpha"]).max()
    wI = np.array([0.0, 0.0, 1.0])

    def value(bb, dirs=None):
        v, der = ctypes.c_double(), np.zeros(1)
        args = (dx.ctypes.data, da.ctypes.data, 1) if dirs else (None, None, 0)
        assert L.vo_cs_objective(bb.ctypes.data, n, 8, 32, 0.47, 2, 0, 0.02, 1, 1.0, wI.ctypes.data, *args, ctypes.byref(v),
                                 der.ctypes.data, 0.0, 0, 0, 0.0) == 0
        return v.value, der[0]

    _, cs = value(b, True)
    h = 1e-8  # small enough that no body crosses a cell boundary between the two runs
    bp, bm = b.copy(), b.copy()
    bp["X"] += h * dx[0]
    bp["alpha"] += h * da[0]
    bm["X"] -= h * dx[0]
    bm["alpha"] -= h * da[0]
    fd = (value(bp)[0] - value(bm)[0]) / (2 * h)
    assert abs(fd - cs) <= 1e-5 * abs(cs)
