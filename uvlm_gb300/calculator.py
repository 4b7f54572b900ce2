"""Host-side mirror of the reference's Vortex::FMMCalculator (src/fmmCalculator.hpp).

The reference selects its behaviour with template policy tags
(fmmCalculator.hpp:9-26): integration scheme Euler/RK2/RK3/RK4, viscous
scheme Inviscid/PSE/CSM, formulation cVPM/rVPM, stretching Transposed/Classic;
and with compile-time constants P, ncrit, MAC_theta (exafmmTypes.hpp:12-15).
Here they are constructor arguments.  Methods keep the reference's names and
meaning: `init(bodies)` builds the tree and permutes `bodies` into tree order,
`calculate()` evaluates velocity, J and dadt on the device,
`copyBodies2Host(bodies)` brings them back, `advance(bodies, dt)` runs one
time step and overwrites `bodies`.  Every call goes through libvfmm.so.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from ._lib import BODY_DTYPE, CELL_DTYPE, check, lib

_SCHEMES = {"Euler": _lib.EULER, "RK2": _lib.RK2, "RK3": _lib.RK3, "RK4": _lib.RK4}
_STRETCH = {"Transposed": _lib.TRANSPOSED, "Classic": _lib.CLASSIC}
_FORM = {"cVPM": _lib.CVPM, "rVPM": _lib.RVPM}
_PREC = {"fp64": _lib.FP64, "mixed": _lib.MIXED}
_VISC = {"Inviscid": _lib.INVISCID, "PSE": _lib.PSE, "CSM": _lib.CSM}


class FMMCalculator:
    def __init__(self, p: int = 4, ncrit: int = 128, theta: float = 0.3, integration: str = "RK3",
                 viscous: str = "Inviscid", formulation: str = "cVPM", stretching: str = "Transposed",
                 precision: str = "fp64", relax: float = 0.0, rk4_fixed: bool = False, device: int = -1,
                 nu: float = 0.0, m2l_batch: int = 0, p2p_chunk: int = 0, m2l_kernel: str = "auto"):
        cfg = _lib.vfmm_config()
        lib().vfmm_default_config(ctypes.byref(cfg))
        cfg.p, cfg.ncrit, cfg.theta = int(p), int(ncrit), float(theta)
        cfg.precision = _PREC[precision]
        cfg.integrator = _SCHEMES[integration]
        cfg.stretching = _STRETCH[stretching]
        cfg.formulation = _FORM[formulation]
        cfg.relax = float(relax)
        cfg.rk4_fixed = int(bool(rk4_fixed))
        cfg.device = int(device)
        cfg.viscous = _VISC[viscous]
        cfg.nu = float(nu)
        cfg.m2l_batch = int(m2l_batch)
        cfg.p2p_chunk = int(p2p_chunk)
        cfg.m2l_kernel = {"auto": 0, "tensor": 1, "cuda": 2}[m2l_kernel]
        h = ctypes.c_void_p()
        code = lib().vfmm_create(ctypes.byref(cfg), ctypes.byref(h))
        if code != 0:
            raise _lib.VfmmError(code, "vfmm_create failed")
        self._h = h
        self.config = cfg
        self.n = 0

    # -- lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().vfmm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, code: int) -> None:
        check(self._h, code)

    # -- FMMCalculator surface (fmmCalculator.hpp)
    def init(self, bodies: np.ndarray) -> None:
        b = _lib.as_bodies(bodies)
        self._check(lib().vfmm_init(self._h, b.ctypes.data, b.size))
        self.n = b.size

    def calculate(self) -> None:
        self._check(lib().vfmm_calculate(self._h))

    def copyBodies2Host(self, bodies: np.ndarray) -> None:
        b = _lib.as_bodies(bodies)
        self._check(lib().vfmm_copy_bodies_to_host(self._h, b.ctypes.data, b.size))

    def advance(self, bodies: np.ndarray, dt: float) -> None:
        b = _lib.as_bodies(bodies)
        self._check(lib().vfmm_advance(self._h, b.ctypes.data, b.size, float(dt)))
        self.n = b.size

    def getSensorData(self, sensors: np.ndarray) -> None:
        s = _lib.as_bodies(sensors)
        self._check(lib().vfmm_get_sensor_data(self._h, s.ctypes.data, s.size))

    def RBF(self, particles: np.ndarray, points: np.ndarray) -> tuple[np.ndarray, int]:
        """FMMCalculator::RBF: permutes `particles` into tree order (in place)
        and returns (kept points with their new strengths, CG iterations)."""
        p = _lib.as_bodies(particles)
        q = _lib.as_bodies(points).copy()
        m, it = ctypes.c_size_t(), ctypes.c_int()
        self._check(lib().vfmm_rbf(self._h, p.ctypes.data, p.size, q.ctypes.data, q.size, ctypes.byref(m), ctypes.byref(it)))
        return q[:m.value], it.value

    def diagnostics(self) -> dict:
        """Circulation, linear and angular impulse of the bodies on the device (FP64)."""
        out = (ctypes.c_double * 9)()
        self._check(lib().vfmm_diagnostics(self._h, out))
        v = np.array(out[:])
        return {"circulation": v[0:3], "linear_impulse": v[3:6], "angular_impulse": v[6:9]}

    def autotune(self, bodies: np.ndarray, dt: float = 0.01) -> dict:
        """vfmm_autotune: time leaf sizes (and M2L batches in mixed mode) on
        these bodies and keep the fastest in this calculator (opt-in: another
        leaf size than the reference's builds another tree)."""
        b = _lib.as_bodies(bodies)
        t = _lib.vfmm_tuning()
        self._check(lib().vfmm_autotune(self._h, b.ctypes.data, b.size, float(dt), ctypes.byref(t)))
        return {"ncrit": t.ncrit, "m2l_batch": t.m2l_batch, "p2p_chunk": t.p2p_chunk, "ms_per_stage": t.ms_per_stage,
                "default_ms_per_stage": t.default_ms_per_stage, "tried": t.tried}

    def choose_order(self, bodies: np.ndarray, tol: float, pmin: int = 4, pmax: int = 16, targets: int = 2048) -> dict:
        """vfmm_choose_order: the lowest expansion order whose velocity error
        against the model-consistent FP64 direct sum is at most tol; this
        calculator keeps it."""
        b = _lib.as_bodies(bodies)
        p, err = ctypes.c_int(), ctypes.c_double()
        self._check(lib().vfmm_choose_order(self._h, b.ctypes.data, b.size, float(tol), int(pmin), int(pmax), int(targets),
                                            ctypes.byref(p), ctypes.byref(err)))
        self.config.p = p.value
        return {"p": p.value, "velocity_rel_l2_vs_model_direct": err.value}

    def adjoint(self, bodies: np.ndarray, dt: float, steps: int, checkpoint_every: int = 10, energy: float = 1.0,
                impulse=(0.0, 0.0, 1.0), seed_x=None, seed_alpha=None, gradient: bool = True):
        """vfmm_adjoint: the objective energy * E + impulse . I (+ seeds . final
        x, alpha) after `steps` steps of advance from `bodies` (not modified),
        and with gradient=True its gradients with respect to the initial
        positions and strengths, as (value, grad_x, grad_alpha) with n x 3
        arrays in the order of `bodies`."""
        b = _lib.as_bodies(bodies)
        n = b.size
        obj = _lib.vfmm_objective()
        obj.energy = float(energy)
        for k in range(3):
            obj.impulse[k] = float(impulse[k])
        keep = []
        for name, arr in (("seed_x", seed_x), ("seed_alpha", seed_alpha)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=np.float64).reshape(n, 3)
                keep.append(a)
                setattr(obj, name, a.ctypes.data)
        value = ctypes.c_double()
        gx = np.zeros((n, 3)) if gradient else None
        ga = np.zeros((n, 3)) if gradient else None
        self._check(lib().vfmm_adjoint(self._h, b.ctypes.data, n, float(dt), int(steps), int(checkpoint_every), ctypes.byref(obj),
                                       ctypes.byref(value), gx.ctypes.data if gradient else None,
                                       ga.ctypes.data if gradient else None))
        del keep
        return (value.value, gx, ga) if gradient else value.value

    def direct_model(self, targets) -> tuple[np.ndarray, np.ndarray]:
        """vfmm_direct_model: FP64 direct sum with this FMM's own kernel split
        (regularised on P2P-list leaf pairs, singular elsewhere) at the bodies
        with tree-order indices `targets`, on the tree of the last init;
        returns (velocity [nt, 3], J [nt, 3, 3])."""
        t = np.ascontiguousarray(np.asarray(targets, dtype=np.uint32))
        out = np.zeros((t.size, 12))
        self._check(lib().vfmm_direct_model(self._h, t.ctypes.data, t.size, out.ctypes.data))
        return out[:, :3].copy(), out[:, 3:].reshape(-1, 3, 3).copy()

    def relax(self, f: float) -> None:
        self._check(lib().vfmm_relax(self._h, float(f)))

    # -- inspection
    def tree(self) -> np.ndarray:
        n = ctypes.c_size_t()
        self._check(lib().vfmm_get_tree(self._h, None, 0, ctypes.byref(n)))
        cells = np.zeros(n.value, CELL_DTYPE)
        self._check(lib().vfmm_get_tree(self._h, cells.ctypes.data, cells.size, ctypes.byref(n)))
        return cells

    def lists(self) -> tuple[np.ndarray, np.ndarray]:
        a, b = ctypes.c_size_t(), ctypes.c_size_t()
        self._check(lib().vfmm_get_lists(self._h, None, 0, ctypes.byref(a), None, 0, ctypes.byref(b)))
        p2p = np.zeros((a.value, 2), np.uint64)
        m2l = np.zeros((b.value, 2), np.uint64)
        self._check(lib().vfmm_get_lists(self._h, p2p.ctypes.data, a.value, ctypes.byref(a),
                                         m2l.ctypes.data, b.value, ctypes.byref(b)))
        return p2p, m2l

    def expansions(self) -> tuple[np.ndarray, np.ndarray]:
        nc = self.stats()["cells"]
        p = self.config.p
        K3 = 3 * p * (p + 1) // 2
        M = np.zeros((nc, K3), np.complex128)
        L = np.zeros((nc, K3), np.complex128)
        self._check(lib().vfmm_get_expansions(self._h, M.ctypes.data, L.ctypes.data, nc))
        return M, L

    def stats(self) -> dict:
        v = (ctypes.c_uint64 * 7)()
        self._check(lib().vfmm_tree_stats(self._h, v, 7))
        return dict(zip(["cells", "leaves", "p2p_pairs", "m2l_pairs", "p2p_interactions", "max_level", "m2l_tensor"], map(int, v)))

    def phase_times(self) -> dict:
        v = (ctypes.c_float * 8)()
        self._check(lib().vfmm_phase_times(self._h, v, 8))
        return dict(zip(["tree_lists", "upward", "m2l", "l2l", "l2p_p2p", "update", "p2p_near", "l2p_far"], map(float, v)))

    # -- device-resident stepping
    def load(self, bodies: np.ndarray) -> None:
        b = _lib.as_bodies(bodies)
        self._check(lib().vfmm_load(self._h, b.ctypes.data, b.size))
        self.n = b.size

    def stage(self, stage: int, dt: float) -> None:
        self._check(lib().vfmm_stage(self._h, int(stage), float(dt)))

    @property
    def num_stages(self) -> int:
        return int(lib().vfmm_num_stages(self._h))

    @property
    def handle(self):
        return self._h


def direct(targets: np.ndarray, sources: np.ndarray) -> np.ndarray:
    """FP64 all-pairs velocity and J on the GPU (regularised kernel); returns a
    copy of `targets` with velocity and J filled."""
    t = np.ascontiguousarray(_lib.as_bodies(targets).copy())
    s = _lib.as_bodies(np.ascontiguousarray(sources))
    with FMMCalculator() as c:
        c._check(lib().vfmm_direct(c._h, t.ctypes.data, t.size, s.ctypes.data, s.size))
    return t


def new_bodies(n: int) -> np.ndarray:
    return np.zeros(n, BODY_DTYPE)


def write_vtk(bodies: np.ndarray, path: str, binary: bool = False) -> None:
    """vfmm_write_vtk: the particles as legacy-VTK polydata, the reference
    driver's writeTovtk file (src/main.cpp:127-164); ASCII is byte-identical
    to it, binary keeps full FP64 values.  Host only."""
    b = _lib.as_bodies(bodies)
    code = lib().vfmm_write_vtk(b.ctypes.data, b.size, os.fsencode(path), int(bool(binary)))
    if code != 0:
        raise _lib.VfmmError(code, f"cannot write {path}")


def advance_batch(calculators: list, bodies: list, dt: float) -> None:
    """vfmm_advance_batch: advance independent systems, bodies[b] on
    calculators[b] (distinct), each array overwritten as advance does."""
    bs = [_lib.as_bodies(b) for b in bodies]
    k = len(bs)
    if k != len(calculators) or k == 0:
        raise ValueError("one calculator per body array")
    hs = (ctypes.c_void_p * k)(*[c.handle for c in calculators])
    ps = (ctypes.c_void_p * k)(*[b.ctypes.data for b in bs])
    ns = (ctypes.c_size_t * k)(*[b.size for b in bs])
    code = lib().vfmm_advance_batch(hs, ps, ns, k, float(dt))
    if code != 0:
        raise _lib.VfmmError(code, lib().vfmm_last_error(calculators[0].handle).decode())
    for c, b in zip(calculators, bs):
        c.n = b.size
