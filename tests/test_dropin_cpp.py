"""The C++ drop-in header (include/vfmm.hpp): a caller written against the
reference's FMMCalculator API (main.cpp:120, :200, :292) compiles unchanged
against it (CPU) and runs on the GPU through libvfmm.so."""
import os
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "dropin_ring.cpp")


def test_dropin_compiles():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I" + os.path.join(ROOT, "include"), SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_dropin_runs(vfmm_lib, tmp_path):
    from uvlm_gb300 import _lib
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "dropin_ring")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), SRC, "-L" + libdir, "-lvfmm",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vtk = tmp_path / "output1.vtk"
    r = subprocess.run([exe, str(vtk)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "centre uz" in r.stdout
    assert vtk.read_bytes().startswith(b"# vtk DataFile Version 3.0\nvtk output\nASCII\nDATASET POLYDATA\nPOINTS 2000 double\n")
