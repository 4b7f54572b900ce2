"""ctypes binding of libvfmm.so (the C ABI declared in include/vfmm.h).

The product path has no fallback: if the library is missing or cannot be
loaded, `lib()` raises.  Build it with `python -m uvlm_gb300._build` (or
`__graft_entry__.build()`).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvfmm.so")

# exafmm::Body (exafmmTypes.hpp:18-32): 37 doubles, 296 bytes.
BODY_DTYPE = np.dtype([
    ("J", "f8", (3, 3)), ("X", "f8", 3), ("alpha", "f8", 3), ("velocity", "f8", 3), ("dadt", "f8", 3),
    ("velocity_old", "f8", 3), ("dadt_old", "f8", 3), ("X_old", "f8", 3), ("alpha_old", "f8", 3),
    ("radius", "f8"), ("drdt", "f8"), ("radius_old", "f8"), ("drdt_old", "f8"),
])
assert BODY_DTYPE.itemsize == 296

# exafmm::Cell without pointers (exafmmTypes.hpp:36-46): 72 bytes.
CELL_DTYPE = np.dtype([
    ("NCHILD", "u8"), ("NBODY", "u8"), ("ChildOffset", "u8"), ("BodyOffset", "u8"),
    ("X", "f8", 3), ("R", "f8"), ("level", "u8"),
])
assert CELL_DTYPE.itemsize == 72

VFMM_OK = 0
(VFMM_ERR_INVALID, VFMM_ERR_NONFINITE, VFMM_ERR_DEPTH, VFMM_ERR_CAPACITY, VFMM_ERR_CUDA, VFMM_ERR_TIMEOUT,
 VFMM_ERR_UNSUPPORTED, VFMM_ERR_STATE) = range(1, 9)
STATUS = {0: "OK", 1: "ERR_INVALID", 2: "ERR_NONFINITE", 3: "ERR_DEPTH", 4: "ERR_CAPACITY", 5: "ERR_CUDA",
          6: "ERR_TIMEOUT", 7: "ERR_UNSUPPORTED", 8: "ERR_STATE"}
EULER, RK2, RK3, RK4 = 0, 1, 2, 3
TRANSPOSED, CLASSIC = 0, 1
CVPM, RVPM = 0, 1
FP64, MIXED = 0, 1
INVISCID, PSE, CSM = 0, 1, 2


class vfmm_tuning(ctypes.Structure):
    _fields_ = [("ncrit", ctypes.c_int), ("m2l_batch", ctypes.c_int), ("ms_per_stage", ctypes.c_double),
                ("default_ms_per_stage", ctypes.c_double), ("tried", ctypes.c_int), ("p2p_chunk", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


class vfmm_objective(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("impulse", ctypes.c_double * 3), ("seed_x", ctypes.c_void_p),
                ("seed_alpha", ctypes.c_void_p)]


class vfmm_config(ctypes.Structure):
    _fields_ = [("p", ctypes.c_int), ("ncrit", ctypes.c_int), ("theta", ctypes.c_double),
                ("precision", ctypes.c_int), ("integrator", ctypes.c_int), ("stretching", ctypes.c_int),
                ("formulation", ctypes.c_int), ("relax", ctypes.c_double), ("rk4_fixed", ctypes.c_int),
                ("device", ctypes.c_int), ("viscous", ctypes.c_int), ("m2l_batch", ctypes.c_int),
                ("nu", ctypes.c_double), ("p2p_chunk", ctypes.c_int), ("m2l_kernel", ctypes.c_int)]


class VfmmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_vp, _sz, _i, _d = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_double
_H = ctypes.c_void_p
_PROTOS = {
    "vfmm_default_config": (None, [ctypes.POINTER(vfmm_config)]),
    "vfmm_create": (_i, [ctypes.POINTER(vfmm_config), ctypes.POINTER(_H)]),
    "vfmm_destroy": (_i, [_H]),
    "vfmm_last_error": (ctypes.c_char_p, [_H]),
    "vfmm_get_config": (_i, [_H, ctypes.POINTER(vfmm_config)]),
    "vfmm_init": (_i, [_H, _vp, _sz]),
    "vfmm_calculate": (_i, [_H]),
    "vfmm_copy_bodies_to_host": (_i, [_H, _vp, _sz]),
    "vfmm_advance": (_i, [_H, _vp, _sz, _d]),
    "vfmm_get_sensor_data": (_i, [_H, _vp, _sz]),
    "vfmm_relax": (_i, [_H, _d]),
    "vfmm_autotune": (_i, [_H, _vp, _sz, _d, _vp]),
    "vfmm_choose_order": (_i, [_H, _vp, _sz, _d, _i, _i, _i, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_d)]),
    "vfmm_adjoint": (_i, [_H, _vp, _sz, _d, _i, _i, _vp, ctypes.POINTER(_d), _vp, _vp]),
    "vfmm_diagnostics": (_i, [_H, ctypes.POINTER(_d)]),
    "vfmm_advance_batch": (_i, [ctypes.POINTER(_H), ctypes.POINTER(_vp), ctypes.POINTER(_sz), _i, _d]),
    "vfmm_rbf": (_i, [_H, _vp, _sz, _vp, _sz, ctypes.POINTER(_sz), ctypes.POINTER(ctypes.c_int)]),
    "vfmm_get_tree": (_i, [_H, _vp, _sz, ctypes.POINTER(_sz)]),
    "vfmm_get_lists": (_i, [_H, _vp, _sz, ctypes.POINTER(_sz), _vp, _sz, ctypes.POINTER(_sz)]),
    "vfmm_get_expansions": (_i, [_H, _vp, _vp, _sz]),
    "vfmm_load": (_i, [_H, _vp, _sz]),
    "vfmm_stage": (_i, [_H, _i, _d]),
    "vfmm_num_stages": (_i, [_H]),
    "vfmm_direct": (_i, [_H, _vp, _sz, _vp, _sz]),
    "vfmm_direct_model": (_i, [_H, _vp, _sz, _vp]),
    "vfmm_event_record": (_i, [_H, _i]),
    "vfmm_event_elapsed": (_i, [_H, _i, _i, ctypes.POINTER(ctypes.c_float)]),
    "vfmm_synchronize": (_i, [_H]),
    "vfmm_launch_count": (ctypes.c_uint64, [_H]),
    "vfmm_phase_times": (_i, [_H, ctypes.POINTER(ctypes.c_float), _i]),
    "vfmm_tree_stats": (_i, [_H, ctypes.POINTER(ctypes.c_uint64), _i]),
    "vfmm_host_register": (_i, [_vp, _sz]),
    "vfmm_host_unregister": (_i, [_vp]),
    "vfmm_flush_l2": (_i, [_H]),
    "vfmm_measure_fma_peak": (_i, [_H, _i, ctypes.POINTER(ctypes.c_double)]),
    "vfmm_bounds_noalloc": (_i, [_vp, _vp, _vp, _sz, _vp, _vp]),
    "vfmm_write_vtk": (_i, [_vp, _sz, ctypes.c_char_p, _i]),
    "vfmm_tcgen05_selftest": (_i, [_i, _i, _vp]),
}

_LIB = None


def lib() -> ctypes.CDLL:
    """The loaded libvfmm.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m uvlm_gb300._build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def exported_symbols() -> list[str]:
    return list(_PROTOS)


def check(h, code: int) -> None:
    if code != VFMM_OK:
        msg = lib().vfmm_last_error(h) if h else b""
        raise VfmmError(code, (msg or b"").decode())


def as_bodies(a: np.ndarray) -> np.ndarray:
    if a.dtype != BODY_DTYPE or not a.flags.c_contiguous:
        raise TypeError("bodies must be a C-contiguous array of BODY_DTYPE")
    return a
