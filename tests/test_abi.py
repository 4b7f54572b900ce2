"""The C-ABI library: builds, loads, exports every entry point of include/vfmm.h
(no GPU needed; no compute calls)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "vfmm.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vfmm_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_reference_surface():
    fns = header_functions()
    for name in ["vfmm_create", "vfmm_init", "vfmm_calculate", "vfmm_advance", "vfmm_get_sensor_data", "vfmm_relax",
                 "vfmm_get_tree", "vfmm_get_lists", "vfmm_copy_bodies_to_host"]:
        assert name in fns


def test_library_exports_every_declared_symbol(vfmm_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", vfmm_lib._name], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (vfmm_\w+)", out))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing
    from uvlm_gb300._lib import exported_symbols
    assert set(exported_symbols()) == set(header_functions())


def test_default_config_matches_reference_constants(vfmm_lib):
    from uvlm_gb300._lib import vfmm_config
    c = vfmm_config()
    vfmm_lib.vfmm_default_config(ctypes.byref(c))
    # exafmmTypes.hpp:12-15 and main.cpp:119 (RK3, Inviscid, cVPM, Transposed)
    assert (c.p, c.ncrit, c.theta) == (4, 128, 0.3)
    assert (c.integrator, c.stretching, c.formulation, c.precision) == (2, 0, 0, 0)


def test_struct_layouts():
    from uvlm_gb300._lib import BODY_DTYPE, CELL_DTYPE, vfmm_config
    assert BODY_DTYPE.itemsize == 296 and CELL_DTYPE.itemsize == 72
    assert ctypes.sizeof(vfmm_config) == 72  # static_assert'ed in api.cu
    from uvlm_gb300._lib import vfmm_tuning
    assert ctypes.sizeof(vfmm_tuning) == 40
    from uvlm_gb300._lib import vfmm_objective
    assert ctypes.sizeof(vfmm_objective) == 48


def test_null_arguments_are_rejected_without_a_gpu(vfmm_lib):
    assert vfmm_lib.vfmm_create(None, None) == 1
    assert vfmm_lib.vfmm_destroy(None) == 1
    assert vfmm_lib.vfmm_init(None, None, 0) == 1
    assert vfmm_lib.vfmm_num_stages(None) == 0
