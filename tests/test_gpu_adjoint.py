"""Reverse-mode gradients (vfmm_adjoint) against central finite differences of
the same FP64 forward: directional derivatives of the objective along random
directions of the initial positions and strengths, one evaluation alone and
through Euler, RK2, RK3 and RK4 steps with checkpointing.

The FMM is piecewise smooth: at theta = 0.5 cells two apart on the octree
lattice sit exactly on the MAC boundary |dX| theta = R_i + R_j
(traverse.hpp:52-57), so rounding decides them and any change of the
bounding box can flip them, a jump that a finite difference sees.  The
checks use theta = 0.47, where no exact ties exist, or at theta = 0.5 only
directions that leave the bounding box (and so every cell centre) fixed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-6  # relative, directional derivative against central differences


def fd_check(c, b, dt, steps, every=1, nd=3, h=1e-7, seed=0, parts=("x", "alpha"), interior=False, **obj):
    val, gx, ga = c.adjoint(b, dt, steps, every, **obj)
    rng = np.random.default_rng(seed)
    amax = np.abs(b["alpha"]).max()
    errs = []
    for part in parts:
        for _ in range(nd):
            vx = rng.normal(size=gx.shape) if part == "x" else np.zeros(gx.shape)
            va = rng.normal(size=ga.shape) * amax if part == "alpha" else np.zeros(ga.shape)
            if interior:  # leave the bodies that set the bounding box in place
                for d in range(3):
                    vx[np.argmin(b["X"][:, d])] = vx[np.argmax(b["X"][:, d])] = 0
            bp, bm = b.copy(), b.copy()
            bp["X"] += h * vx
            bp["alpha"] += h * va
            bm["X"] -= h * vx
            bm["alpha"] -= h * va
            fp = c.adjoint(bp, dt, steps, every, gradient=False, **obj)
            fm = c.adjoint(bm, dt, steps, every, gradient=False, **obj)
            fd = (fp - fm) / (2 * h)
            an = float((gx * vx).sum() + (ga * va).sum())
            errs.append((part, abs(fd - an) / abs(an), fd, an))
    return val, gx, ga, errs


def worst(errs):
    return max(e[1] for e in errs)


def test_evaluation_gradient_single_leaf(vfmm_lib):
    """All bodies in one leaf: the objective's evaluation is the P2P near field only."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(200, seed=1)
    with FMMCalculator(p=6, ncrit=256, theta=0.5, integration="Euler") as c:
        _, _, _, errs = fd_check(c, b, 0.01, 0)
    assert worst(errs) < TOL, errs


def test_evaluation_gradient_full_tree(vfmm_lib):
    """A deep tree: P2M, M2M, M2L, L2L, L2P transposed, plus the bounding-box terms."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(4000, seed=2)
    with FMMCalculator(p=8, ncrit=32, theta=0.47, integration="Euler") as c:
        _, _, _, errs = fd_check(c, b, 0.01, 0)
    assert worst(errs) < TOL, errs
    with FMMCalculator(p=8, ncrit=32, theta=0.5, integration="Euler") as c:
        _, _, _, errs = fd_check(c, b, 0.01, 0, interior=True, seed=1)
    assert worst(errs) < TOL, errs


@pytest.mark.parametrize("integration,stretching,rk4_fixed", [("Euler", "Transposed", False), ("RK2", "Transposed", False),
                                                              ("RK3", "Transposed", False), ("RK2", "Classic", False),
                                                              ("RK4", "Transposed", False), ("RK4", "Transposed", True),
                                                              ("RK4", "Classic", False)])
def test_step_gradients(vfmm_lib, integration, stretching, rk4_fixed):
    """Under RK4 with the full-step third stage the ring of seed 3 sits on a
    branch boundary of the map (the oracle's one-sided differences along the
    first direction disagree by 100%), so that case takes the ring of seed 5,
    on which both RK4 forms are smooth."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(24, seed=5 if rk4_fixed else 3)
    with FMMCalculator(p=8, ncrit=32, theta=0.47, integration=integration, stretching=stretching, rk4_fixed=rk4_fixed) as c:
        _, _, _, errs = fd_check(c, b, 0.02, 2, every=1, nd=2, h=1e-8)
    assert worst(errs) < 1e-5, errs  # h = 1e-8: rounding of the differences ~1e-7


def test_checkpoint_spacing_does_not_change_the_gradient(vfmm_lib):
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.leapfrog(16, seed=4)
    out = []
    with FMMCalculator(p=8, ncrit=32, theta=0.5, integration="RK3") as c:
        for every in (1, 2, 4):
            out.append(c.adjoint(b, 0.01, 4, every))
    for v, gx, ga in out[1:]:
        assert v == out[0][0] and np.array_equal(gx, out[0][1]) and np.array_equal(ga, out[0][2])


def test_seeds_follow_the_bodies(vfmm_lib):
    """With only seeds on the final state and no steps, the gradient is the seed
    itself, in the caller's order although the trees reorder the bodies."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(3000, seed=5)
    rng = np.random.default_rng(6)
    sx, sa = rng.normal(size=(b.size, 3)), rng.normal(size=(b.size, 3))
    with FMMCalculator(p=6, ncrit=32, theta=0.47, integration="RK2") as c:
        v, gx, ga = c.adjoint(b, 0.01, 0, energy=0.0, impulse=(0, 0, 0), seed_x=sx, seed_alpha=sa)
        assert np.array_equal(gx, sx) and np.array_equal(ga, sa)
        assert v == pytest.approx(float((sx * b["X"]).sum() + (sa * b["alpha"]).sum()), rel=1e-12)
        _, _, _, errs = fd_check(c, b, 0.02, 1, energy=0.0, impulse=(0, 0, 0), seed_x=sx, seed_alpha=sa, nd=2)
    assert worst(errs) < TOL, errs


@pytest.mark.parametrize("kw,tol", [(dict(integration="RK3"), 1e-5), (dict(integration="RK4"), 1e-5),
                                    (dict(integration="RK2", relax=0.3), 3e-5),
                                    (dict(integration="RK3", m2l_kernel="tensor"), 2e-5)])
def test_mixed_gradient_close_to_fp64(vfmm_lib, kw, tol):
    """Mixed precision (FP32 forward kernels, FP32 P2P^T and M2L^T in the
    reverse sweep): the gradient differs from the all-FP64 one by FP32
    rounding of the trajectory and of the transposed passes (RK3, RK4, and
    RK2 with relaxation).  Relaxation rescales alpha by |alpha| / |w| with w
    a difference of J entries, which amplifies J's rounding (measured 1.1e-5
    on this case; the FP64 relaxation adjoint matches the complex step to
    1e-8).  With the forward M2L on the tensor cores (three TF32 products,
    operands held to about 2^-22 against FP32's 2^-24) the forward fields stay
    as close to FP64 as with the FP32 M2L (velocity 2.2e-7 on this case) but
    the 3-step gradient differs by up to 1.0e-5 (6.0e-6 with the CUDA-core
    M2L)."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.leapfrog(16, seed=7)
    res = {}
    for prec in ("fp64", "mixed"):
        with FMMCalculator(p=8, ncrit=32, theta=0.47, precision=prec, **kw) as c:
            res[prec] = c.adjoint(b, 0.01, 3, 2)
    for k in (1, 2):
        a, r = res["mixed"][k], res["fp64"][k]
        assert np.linalg.norm(a - r) / np.linalg.norm(r) < tol


def test_adjoint_rejects_what_it_does_not_cover(vfmm_lib):
    from uvlm_gb300 import FMMCalculator, VfmmError, workloads
    b = workloads.cloud(500, seed=8)
    for kw in (dict(viscous="PSE", nu=0.01), dict(viscous="CSM", nu=0.01)):
        with FMMCalculator(p=4, ncrit=32, theta=0.5, **kw) as c:
            with pytest.raises(VfmmError):
                c.adjoint(b, 0.01, 1)


def _complex_step(b, P, ncrit, theta, scheme, dt, steps, dirs_x, dirs_a, energy=1.0, impulse=(0.0, 0.0, 1.0), relax=0.0,
                  formulation=0):
    import ctypes
    from oracle.oracle import oracle
    L = oracle()
    n, nd = b.size, dirs_x.shape[0]
    wI = np.array(impulse, float)
    val, der = ctypes.c_double(), np.zeros(nd)
    dx, da = np.ascontiguousarray(dirs_x), np.ascontiguousarray(dirs_a)
    assert L.vo_cs_objective(b.ctypes.data, n, P, ncrit, theta, scheme, 0, dt, steps, energy, wI.ctypes.data, dx.ctypes.data,
                             da.ctypes.data, nd, ctypes.byref(val), der.ctypes.data, relax, formulation, 0, 0.0) == 0
    return val.value, der


# the oracle's scheme numbers: 2 RK3, 3 RK4 with the reference's half-step
# third stage, 4 RK4 with a full-step third stage
@pytest.mark.parametrize("theta,steps,integration,rk4_fixed", [(0.5, 0, "RK3", False), (0.47, 2, "RK3", False),
                                                               (0.47, 2, "RK4", False), (0.47, 1, "RK4", True)])
def test_gradient_matches_complex_step(vfmm_lib, theta, steps, integration, rk4_fixed):
    """Directional derivatives from the adjoint against the oracle's whole-step
    complex step (real parts, trees and lists untouched by the step).  Multi-step
    runs use theta = 0.47: CPU and GPU trajectories differ by rounding, and only
    without exact MAC ties do both runs take the same branch at every stage."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(16, seed=3)
    rng = np.random.default_rng(11)
    nd = 3
    dx = rng.normal(size=(nd, b.size, 3))
    da = rng.normal(size=(nd, b.size, 3)) * np.abs(b["alpha"]).max()
    with FMMCalculator(p=8, ncrit=32, theta=theta, integration=integration, rk4_fixed=rk4_fixed) as c:
        v, gx, ga = c.adjoint(b, 0.02, steps, 1)
    scheme = 2 if integration == "RK3" else (4 if rk4_fixed else 3)
    vc, der = _complex_step(b, 8, 32, theta, scheme, 0.02, steps, dx, da)
    assert abs(v - vc) <= 1e-10 * abs(vc)
    for k in range(nd):
        an = float((gx * dx[k]).sum() + (ga * da[k]).sum())
        assert abs(an - der[k]) <= 1e-8 * abs(der[k]), (k, an, der[k])


@pytest.mark.parametrize("integration,scheme", [("RK2", 1), ("RK3", 2)])
def test_gradient_with_relaxation(vfmm_lib, integration, scheme):
    """Relaxation after each step (relaxation.hpp:8-19): the adjoint against
    the oracle's complex step of the same relaxed steps, and against central
    differences.  The ring of seed 5: on it the oracle's one-sided differences
    along these directions agree to rounding for both schemes (on the rings
    of seeds 2 and 3 relaxation puts the map on a branch boundary)."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(16, seed=5)
    rng = np.random.default_rng(13)
    nd = 3
    dx = rng.normal(size=(nd, b.size, 3))
    da = rng.normal(size=(nd, b.size, 3)) * np.abs(b["alpha"]).max()
    with FMMCalculator(p=8, ncrit=32, theta=0.47, integration=integration, relax=0.3) as c:
        v, gx, ga = c.adjoint(b, 0.02, 2, 1)
        _, _, _, errs = fd_check(c, b, 0.02, 2, every=1, nd=2, h=1e-8, seed=4)
    assert worst(errs) < 1e-5, errs
    vc, der = _complex_step(b, 8, 32, 0.47, scheme, 0.02, 2, dx, da, relax=0.3)
    assert abs(v - vc) <= 1e-10 * abs(vc)
    for k in range(nd):
        an = float((gx * dx[k]).sum() + (ga * da[k]).sum())
        assert abs(an - der[k]) <= 1e-8 * abs(der[k]), (k, an, der[k])
    with FMMCalculator(p=8, ncrit=32, theta=0.47, integration=integration) as c:
        v0, gx0, _ = c.adjoint(b, 0.02, 2, 1)
    assert abs(v0 - v) > 1e-6 * abs(v) and not np.allclose(gx0, gx), "relaxation made no difference"


@pytest.mark.parametrize("integration,scheme,seed", [("RK2", 1, 4), ("RK3", 2, 5)])
def test_gradient_rvpm(vfmm_lib, integration, scheme, seed):
    """rVPM (fmmCalculator.hpp:407-418): the radii evolve with dr/dt, so the
    gradient runs through the radius cotangents of the pair weights, the rVPM
    terms and the stage updates.  Against the oracle's complex step of the
    same steps (rings on which the oracle's complex step and central
    differences agree to 1e-5 along these directions), and mixed against
    FP64."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(16, seed=seed)
    rng = np.random.default_rng(11)
    nd = 3
    dx = rng.normal(size=(nd, b.size, 3))
    da = rng.normal(size=(nd, b.size, 3)) * np.abs(b["alpha"]).max()
    res = {}
    for prec in ("fp64", "mixed"):
        with FMMCalculator(p=8, ncrit=32, theta=0.47, integration=integration, formulation="rVPM", precision=prec) as c:
            res[prec] = c.adjoint(b, 0.02, 2, 1)
    v, gx, ga = res["fp64"]
    vc, der = _complex_step(b, 8, 32, 0.47, scheme, 0.02, 2, dx, da, formulation=1)
    assert abs(v - vc) <= 1e-10 * abs(vc)
    for k in range(nd):
        an = float((gx * dx[k]).sum() + (ga * da[k]).sum())
        assert abs(an - der[k]) <= 1e-8 * abs(der[k]), (k, an, der[k])
    for k in (1, 2):
        a, r = res["mixed"][k], res["fp64"][k]
        err = np.linalg.norm(a - r) / np.linalg.norm(r)
        print(f"rVPM {integration}: mixed vs FP64 gradient {err:.3e}")
        assert err < 1e-4


@pytest.mark.parametrize("n,p,ncrit,theta", [(20000, 12, 64, 0.5), (8000, 8, 16, 0.3)])
def test_mixed_evaluation_gradient_close_to_fp64(vfmm_lib, n, p, ncrit, theta):
    """One evaluation (steps = 0) of a cloud: the FP32 transposes against the
    FP64 ones.  At theta = 0.3 (the reference's default) and leaves of 16 most
    P2P rows span more than 32 leaves, so the transposed P2P kernels stage
    their rows in several groups."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(n, seed=12)
    res = {}
    for prec in ("fp64", "mixed"):
        with FMMCalculator(p=p, ncrit=ncrit, theta=theta, integration="Euler", precision=prec) as c:
            res[prec] = c.adjoint(b, 0.01, 0)
    for k in (1, 2):
        a, r = res["mixed"][k], res["fp64"][k]
        assert np.linalg.norm(a - r) / np.linalg.norm(r) < 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_edge_cases(vfmm_lib, precision):
    """One body (no pairs, a root leaf), two bodies, and a cloud with coincident
    bodies (pairs at zero distance are skipped, as in the forward)."""
    from uvlm_gb300 import FMMCalculator, workloads
    one = workloads.cloud(1, seed=40)
    two = workloads.cloud(2, seed=41)
    dup = workloads.cloud(600, seed=42)
    dup[300:]["X"] = dup[:300]["X"]
    for b in (one, two, dup):
        with FMMCalculator(p=6, ncrit=16, theta=0.47, integration="RK2", precision=precision) as c:
            v, gx, ga = c.adjoint(b, 0.01, 2, 1)
            assert np.isfinite(v) and np.isfinite(gx).all() and np.isfinite(ga).all()
            if b.size == 1:
                # one body: u = 0, so only the impulse term 1/2 (x cross alpha)_z acts and nothing moves
                x, al = b["X"][0], b["alpha"][0]
                assert v == pytest.approx(0.5 * (x[0] * al[1] - x[1] * al[0]), rel=1e-14)
                assert np.allclose(gx[0], [0.5 * al[1], -0.5 * al[0], 0.0], rtol=1e-14, atol=0)
                assert np.allclose(ga[0], [-0.5 * x[1], 0.5 * x[0], 0.0], rtol=1e-14, atol=0)
            elif precision == "fp64" and b.size == 2:
                # (coincident bodies are a jump of the forward map itself: a pair's J term
                # tends to a nonzero limit as the distance goes to 0 but is skipped at 0)
                _, _, _, errs = fd_check(c, b, 0.01, 2, nd=2, h=1e-7, seed=3)
                assert worst(errs) < 1e-5, errs
