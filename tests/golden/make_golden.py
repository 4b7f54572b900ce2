"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference (kursatyurt/UVLM, src/*.hpp) is compiled from its own sources
against the project's Kokkos shim (oracle/ref_driver.cpp, oracle/Makefile,
serial backend: bitwise reproducible) for each (P, ncrit, theta) used below,
run on seeded inputs, and its outputs saved as .npz.  Needs the reference's
src/ directory, named by UVLM_REF_SRC (default: the checkout at
/root/reference/src); the fixtures it writes are committed and read by the
tests everywhere.

Each body carries its input index in `drdt_old`, a field the evaluation never
touches, so the tree permutation can be read from the permuted output.

Usage:  python tests/golden/make_golden.py [viscous|rbf|rvpm]   (only those cases)
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from uvlm_gb300 import workloads  # noqa: E402
from uvlm_gb300._lib import BODY_DTYPE, CELL_DTYPE  # noqa: E402

L_ = ctypes.c_long


def tag(b):
    b = b.copy()
    b["drdt_old"] = np.arange(b.size)
    return b


def ref_tree(R, b):
    bb = b.copy()
    cap = 4 * b.size + 64
    cells = np.zeros(cap, CELL_DTYPE)
    nc = R.ref_build_tree(bb.ctypes.data, bb.size, cells.ctypes.data, cap)
    return bb, cells[:nc].copy()


def ref_lists(R, b):
    bb = b.copy()
    a, c = L_(), L_()
    R.ref_lists(bb.ctypes.data, bb.size, None, 0, ctypes.byref(a), None, 0, ctypes.byref(c))
    p2p = np.zeros((a.value, 2), np.uint64)
    m2l = np.zeros((c.value, 2), np.uint64)
    R.ref_lists(bb.ctypes.data, bb.size, p2p.ctypes.data, a.value, ctypes.byref(a), m2l.ctypes.data, c.value,
                ctypes.byref(c))
    # as sets: sorted by (target, source)
    p2p = p2p[np.lexsort((p2p[:, 1], p2p[:, 0]))]
    m2l = m2l[np.lexsort((m2l[:, 1], m2l[:, 0]))]
    return p2p, m2l


def ref_calc(R, b, P, stretching=0, formulation=0, expansions=False, cell_stride=1):
    bb = b.copy()
    nc = L_()
    if expansions:
        cap = 4 * b.size + 64
        K3 = 3 * P * (P + 1) // 2
        M = np.zeros((cap, K3), np.complex128)
        Lx = np.zeros((cap, K3), np.complex128)
        R.ref_calculate(bb.ctypes.data, bb.size, stretching, formulation, M.ctypes.data, Lx.ctypes.data, cap,
                        ctypes.byref(nc))
        sel = np.arange(0, nc.value, cell_stride)
        return bb, sel, M[sel], Lx[sel]
    R.ref_calculate(bb.ctypes.data, bb.size, stretching, formulation, None, None, 0, ctypes.byref(nc))
    return bb


def inputs_of(b):
    return dict(X=b["X"], alpha=b["alpha"], radius=b["radius"])


def save(name, **kw):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **kw)
    print(f"{name}: {os.path.getsize(path) / 1024:.0f} KB")


def eval_case(name, b, P, ncrit, theta, stretching=0, formulation=0, expansions=False, cell_stride=1):
    R = O.ref(P, ncrit, theta)
    b = tag(b)
    tb, cells = ref_tree(R, b)
    p2p, m2l = ref_lists(R, b)
    kw = dict(P=P, ncrit=ncrit, theta=theta, stretching=stretching, formulation=formulation, **inputs_of(b),
              perm=tb["drdt_old"].astype(np.int64), cells=cells, p2p=p2p, m2l=m2l)
    if expansions:
        out, sel, M, Lx = ref_calc(R, b, P, stretching, formulation, True, cell_stride)
        kw.update(cell_sel=sel, M=M, L=Lx)
    else:
        out = ref_calc(R, b, P, stretching, formulation)
    assert (out["drdt_old"] == tb["drdt_old"]).all()
    kw.update(velocity=out["velocity"], J=out["J"], dadt=out["dadt"], drdt=out["drdt"])
    save(name, **kw)


def advance_case(name, b, P, ncrit, theta, dt, steps, scheme, stretching=0):
    R = O.ref(P, ncrit, theta)
    b = tag(b)
    out = b.copy()
    R.ref_advance(out.ctypes.data, out.size, dt, steps, scheme, stretching)
    # bodies come back in the last stage's tree order; RK stages overwrite drdt_old, so no index tag here
    save(name, P=P, ncrit=ncrit, theta=theta, dt=dt, steps=steps, scheme=scheme, stretching=stretching, **inputs_of(b),
         out_X=out["X"], out_alpha=out["alpha"], out_radius=out["radius"], out_velocity=out["velocity"],
         out_J=out["J"])


def viscous_case(name, b, P, ncrit, theta, dt, steps, scheme, viscous, nu):
    """advance with Vortex::PSE (viscous 1) or Vortex::CSM (2), viscosity nu."""
    R = O.ref(P, ncrit, theta)
    out = b.copy()
    rc = R.ref_advance_viscous(out.ctypes.data, out.size, dt, steps, scheme, viscous, nu)
    assert rc == 0
    save(name, P=P, ncrit=ncrit, theta=theta, dt=dt, steps=steps, scheme=scheme, stretching=0, viscous=viscous, nu=nu,
         **inputs_of(b), out_X=out["X"], out_alpha=out["alpha"], out_radius=out["radius"], out_velocity=out["velocity"],
         out_J=out["J"])


def rvpm_case(name, b, P, ncrit, theta, dt, steps, scheme):
    """advance with Vortex::rVPM (the radii evolve), transposed stretching."""
    R = O.ref(P, ncrit, theta)
    out = b.copy()
    rc = R.ref_advance_rvpm(out.ctypes.data, out.size, dt, steps, scheme)
    assert rc == 0
    save(name, P=P, ncrit=ncrit, theta=theta, dt=dt, steps=steps, scheme=scheme, stretching=0, formulation=1,
         **inputs_of(b), out_X=out["X"], out_alpha=out["alpha"], out_radius=out["radius"], out_velocity=out["velocity"],
         out_J=out["J"])


def rvpm_cases():
    rvpm_case("advance_rvpm_rk2_ring", workloads.ring(8, seed=17), 6, 32, 0.5, 0.01, 2, 1)
    rvpm_case("advance_rvpm_rk3_cloud", workloads.cloud(600, seed=18), 6, 16, 0.5, 0.05, 2, 2)


def viscous_cases():
    viscous_case("advance_pse_cloud", workloads.cloud(700, seed=14), 6, 16, 0.5, 0.05, 2, 1, 1, 0.01)
    viscous_case("advance_pse_rk3_ring", workloads.ring(8, seed=15), 6, 32, 0.5, 0.01, 1, 2, 1, 0.005)
    viscous_case("advance_csm_cloud", workloads.cloud(600, seed=16), 6, 16, 0.5, 0.05, 2, 1, 2, 0.01)


def rbf_case(name, b, lo, hi, k, rfac, P, ncrit, theta):
    """FMMCalculator::RBF of particles b onto a k^3 lattice over [lo, hi]^3
    with point radius rfac * spacing."""
    R = O.ref(P, ncrit, theta)
    g = np.linspace(lo, hi, k)
    pts = np.zeros(k ** 3, BODY_DTYPE)
    pts["X"] = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pts["radius"] = rfac * (g[1] - g[0])
    bb, pp, m = b.copy(), pts.copy(), ctypes.c_long()
    assert R.ref_rbf(bb.ctypes.data, bb.size, pp.ctypes.data, pp.size, ctypes.byref(m)) == 0
    pp = pp[:m.value]
    save(name, P=P, ncrit=ncrit, theta=theta, **inputs_of(b), points_X=pts["X"], points_radius=pts["radius"],
         out_particles_X=bb["X"], out_X=pp["X"], out_alpha=pp["alpha"], out_vorticity=pp["velocity_old"])


def rbf_cases():
    rbf_case("rbf_cloud", workloads.cloud(800, seed=18), -1.8, 1.8, 14, 0.6, 6, 16, 0.5)
    rbf_case("rbf_ring_c32", workloads.ring(6, seed=19), -1.4, 1.4, 16, 0.5, 6, 32, 0.5)


def sensor_case(name, b, s, P, ncrit, theta):
    R = O.ref(P, ncrit, theta)
    bb, ss = b.copy(), s.copy()
    ss["drdt_old"] = np.arange(ss.size)
    s_in = ss.copy()
    R.ref_sensors(bb.ctypes.data, bb.size, ss.ctypes.data, ss.size)
    save(name, P=P, ncrit=ncrit, theta=theta, **inputs_of(b), sensor_X=s_in["X"],
         sensor_perm=ss["drdt_old"].astype(np.int64), sensor_velocity=ss["velocity"], sensor_J=ss["J"])


def main():
    rng = np.random.default_rng(12345)
    # FMM evaluation: tree, lists, expansions and rates
    eval_case("cloud_p6_c16_t05", workloads.cloud(1500, seed=1), 6, 16, 0.5, expansions=True, cell_stride=8)
    eval_case("ring_p8_c32_t05", workloads.ring(12, seed=2), 8, 32, 0.5)
    eval_case("cloud_p10_c64_t05", workloads.cloud(2500, seed=3), 10, 64, 0.5, expansions=True, cell_stride=16)
    eval_case("cloud_p4_c128_t03", workloads.cloud(1200, seed=4), 4, 128, 0.3)
    eval_case("cloud_p14_c32_t05", workloads.cloud(1000, seed=5), 14, 32, 0.5)
    eval_case("classic_rvpm_p6", workloads.cloud(800, seed=6), 6, 16, 0.5, stretching=1, formulation=1)
    # edge cases
    small = workloads.cloud(10, seed=7)
    small["radius"] = 0.3
    eval_case("root_leaf", small, 6, 16, 0.5)
    dup = workloads.cloud(600, seed=8)
    dup["X"][300:310] = dup["X"][0:10]  # coincident pairs: R2 == 0 is skipped
    eval_case("coincident", dup, 6, 8, 0.5)
    grid = np.zeros(729, BODY_DTYPE)  # on-plane points: strict x > centre comparisons
    g = np.linspace(-1.0, 1.0, 9)
    grid["X"] = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    grid["alpha"] = rng.normal(0, 1e-3, (729, 3))
    grid["radius"] = 0.3
    eval_case("lattice_ties", grid, 6, 8, 0.5)
    # time stepping (scheme 0 Euler, 1 RK2, 2 RK3, 3 RK4 with the reference's stage-3 0.5*dt)
    advance_case("advance_rk2_ring", workloads.ring(8, seed=9), 6, 32, 0.5, 0.01, 2, 1)
    advance_case("advance_rk3_cloud", workloads.cloud(700, seed=10), 6, 16, 0.5, 0.05, 2, 2)
    advance_case("advance_euler_cloud", workloads.cloud(500, seed=11), 4, 16, 0.5, 0.05, 2, 0)
    advance_case("advance_rk4_cloud", workloads.cloud(500, seed=12), 4, 16, 0.5, 0.05, 1, 3)
    # sensors
    sens = np.zeros(300, BODY_DTYPE)
    sens["X"] = rng.uniform(-1.2, 1.2, (300, 3))
    sensor_case("sensors_p6", workloads.cloud(1500, seed=13), sens, 6, 16, 0.5)


if __name__ == "__main__":
    if sys.argv[1:] == ["viscous"]:
        viscous_cases()
    elif sys.argv[1:] == ["rbf"]:
        rbf_cases()
    elif sys.argv[1:] == ["rvpm"]:
        rvpm_cases()
    else:
        main()
        viscous_cases()
        rbf_cases()
        rvpm_cases()
