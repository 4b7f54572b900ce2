"""ctypes access to the oracles.  TEST INFRASTRUCTURE ONLY: used by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.

* liboracle.so: the C++ restatement of the reference's FMM (vfmm_oracle.cpp),
  built everywhere by `make -C oracle`.
* _ref/libref_p{P}_c{ncrit}_t{theta}.so: the reference's own headers compiled
  against the project's Kokkos shim (ref_driver.cpp), built only where the
  reference sources exist.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
# the reference's src/ directory (its headers are compiled for the golden fixtures)
REF_SRC = os.environ.get("UVLM_REF_SRC", "/root/reference/src")

_vp, _L, _i, _d = ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_double
_PL = ctypes.POINTER(ctypes.c_long)


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORACLE_SO


_ORA = None


def oracle() -> ctypes.CDLL:
    global _ORA
    if _ORA is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.vo_set_threads.argtypes = [_i]
        L.vo_set_threads.restype = _i
        L.vo_build_tree.argtypes = [_vp, _L, _i, _vp, _L]
        L.vo_build_tree.restype = _L
        L.vo_lists.argtypes = [_vp, _vp, _d, _vp, _L, _PL, _vp, _L, _PL]
        L.vo_calculate.argtypes = [_vp, _L, _i, _i, _d, _i, _i, _vp, _vp, _L, _PL]
        L.vo_advance.argtypes = [_vp, _L, _i, _i, _d, _d, _i, _i, _i, _i, _d, _i, _i, _d]
        L.vo_sensors.argtypes = [_vp, _L, _vp, _L, _i, _i, _d]
        L.vo_direct.argtypes = [_vp, _L, _vp, _L]
        L.vo_direct.restype = None
        L.vo_direct_model.argtypes = [_vp, _L, _vp, _L, _vp, _L, _vp, _L, _vp]
        L.vo_direct_model.restype = None
        L.vo_relax.argtypes = [_vp, _L, _d]
        L.vo_relax.restype = None
        L.vo_cs_advance.argtypes = [_vp, _L, _i, _i, _d, _i, _i, _d, _i, _d, _i, _i, _d]
        L.vo_cs_objective.argtypes = [_vp, _L, _i, _i, _d, _i, _i, _d, _i, _d, _vp, _vp, _vp, _i, _vp, _vp, _d, _i, _i, _d]
        _ORA = L
    return _ORA


def ref_available() -> bool:
    return os.path.isdir(REF_SRC)


def ref(P: int, ncrit: int, theta: float, openmp: bool = False) -> ctypes.CDLL:
    """The reference compiled for (P, ncrit, theta); builds it on first use.
    openmp: the OpenMP build (timing), else the serial one (fixtures)."""
    tag = "omp_" if openmp else ""
    so = os.path.join(HERE, "_ref", f"libref_{tag}p{P}_c{ncrit}_t{theta}.so")
    if not os.path.exists(so) or ref_available():  # make rebuilds it when the driver or the shim changed
        subprocess.run(["make", "-s", "-C", HERE, "ref-omp" if openmp else "ref", f"REF_SRC={REF_SRC}", f"REF_P={P}",
                        f"REF_NCRIT={ncrit}", f"REF_THETA={theta}"], check=True)
    L = ctypes.CDLL(so)
    L.ref_build_tree.argtypes = [_vp, _L, _vp, _L]
    L.ref_build_tree.restype = _L
    L.ref_lists.argtypes = [_vp, _L, _vp, _L, _PL, _vp, _L, _PL]
    L.ref_lists.restype = _L
    L.ref_calculate.argtypes = [_vp, _L, _i, _i, _vp, _vp, _L, _PL]
    L.ref_advance.argtypes = [_vp, _L, _d, _i, _i, _i]
    L.ref_sensors.argtypes = [_vp, _L, _vp, _L]
    L.ref_advance_viscous.argtypes = [_vp, _L, _d, _i, _i, _i, _d]
    L.ref_advance_rvpm.argtypes = [_vp, _L, _d, _i, _i]
    L.ref_rbf.argtypes = [_vp, _L, _vp, _L, _PL]
    L.ref_direct.argtypes = [_vp, _L, _vp, _L]
    L.ref_direct.restype = None
    return L


# ---- convenience wrappers over the restatement -------------------------------
def build_tree(bodies: np.ndarray, ncrit: int):
    from uvlm_gb300._lib import CELL_DTYPE
    b = bodies.copy()
    cap = 4 * b.size + 64
    cells = np.zeros(cap, CELL_DTYPE)
    nc = oracle().vo_build_tree(b.ctypes.data, b.size, ncrit, cells.ctypes.data, cap)
    if nc < 0:
        raise RuntimeError("oracle: tree too deep")
    return b, cells[:nc].copy()


def lists(cells: np.ndarray, theta: float, scells: np.ndarray | None = None):
    scells = cells if scells is None else scells
    a, b = ctypes.c_long(), ctypes.c_long()
    oracle().vo_lists(cells.ctypes.data, scells.ctypes.data, theta, None, 0, ctypes.byref(a), None, 0, ctypes.byref(b))
    p2p = np.zeros((a.value, 2), np.uint64)
    m2l = np.zeros((b.value, 2), np.uint64)
    oracle().vo_lists(cells.ctypes.data, scells.ctypes.data, theta, p2p.ctypes.data, a.value, ctypes.byref(a),
                      m2l.ctypes.data, b.value, ctypes.byref(b))
    return p2p, m2l


def calculate(bodies: np.ndarray, P: int, ncrit: int, theta: float, stretching: int = 0, formulation: int = 0,
              want_expansions: bool = False):
    b = bodies.copy()
    nc = ctypes.c_long()
    M = L = None
    if want_expansions:
        cap = 4 * b.size + 64
        K3 = 3 * P * (P + 1) // 2
        M = np.zeros((cap, K3), np.complex128)
        L = np.zeros((cap, K3), np.complex128)
        rc = oracle().vo_calculate(b.ctypes.data, b.size, P, ncrit, theta, stretching, formulation, M.ctypes.data,
                                   L.ctypes.data, cap, ctypes.byref(nc))
    else:
        rc = oracle().vo_calculate(b.ctypes.data, b.size, P, ncrit, theta, stretching, formulation, None, None, 0,
                                   ctypes.byref(nc))
    if rc != 0:
        raise RuntimeError(f"oracle calculate failed ({rc})")
    if want_expansions:
        return b, M[:nc.value], L[:nc.value]
    return b


def advance(bodies: np.ndarray, P: int, ncrit: int, theta: float, dt: float, steps: int, scheme: int,
            stretching: int = 0, formulation: int = 0, relax: float = 0.0, rk4_fixed: int = 0, viscous: int = 0,
            nu: float = 0.0) -> np.ndarray:
    b = bodies.copy()
    rc = oracle().vo_advance(b.ctypes.data, b.size, P, ncrit, theta, dt, steps, scheme, stretching, formulation,
                             relax, rk4_fixed, viscous, nu)
    if rc != 0:
        raise RuntimeError(f"oracle advance failed ({rc})")
    return b


def sensors(bodies: np.ndarray, sens: np.ndarray, P: int, ncrit: int, theta: float):
    b = bodies.copy()
    s = sens.copy()
    rc = oracle().vo_sensors(b.ctypes.data, b.size, s.ctypes.data, s.size, P, ncrit, theta)
    if rc != 0:
        raise RuntimeError("oracle sensors failed")
    return b, s


def direct(targets: np.ndarray, sources: np.ndarray) -> np.ndarray:
    t = targets.copy()
    oracle().vo_direct(t.ctypes.data, t.size, sources.ctypes.data, sources.size)
    return t


def direct_model(bodies: np.ndarray, cells: np.ndarray, p2p: np.ndarray, targets) -> np.ndarray:
    """Direct sum with the FMM's kernel split (regularised on P2P-list leaf
    pairs, singular elsewhere) at tree-order bodies `targets`; [nt, 12]."""
    t = np.ascontiguousarray(np.asarray(targets, dtype=np.uint32))
    pairs = np.ascontiguousarray(p2p, dtype=np.uint64)
    out = np.zeros((t.size, 12))
    oracle().vo_direct_model(bodies.ctypes.data, bodies.size, cells.ctypes.data, cells.size, pairs.ctypes.data,
                             len(pairs), t.ctypes.data, t.size, out.ctypes.data)
    return out
