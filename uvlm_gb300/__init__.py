"""uvlm_gb300 — GB300-native vortex-particle FMM (drop-in for the velocity and
stretching evaluation of kursatyurt/UVLM).  The compute runs in libvfmm.so
(hand-written sm_103a CUDA behind the C ABI of include/vfmm.h); this package
is the Python-side mirror of the reference's FMMCalculator interface."""
from ._lib import BODY_DTYPE, CELL_DTYPE, VfmmError, lib  # noqa: F401
from .calculator import FMMCalculator, advance_batch, direct, new_bodies, write_vtk  # noqa: F401
from . import workloads  # noqa: F401
