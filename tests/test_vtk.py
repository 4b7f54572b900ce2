"""vfmm_write_vtk: the particle file of the reference driver's writeTovtk
(src/main.cpp:127-164).  ASCII output against the oracle's restatement of
that writer, byte for byte; BINARY output read back exactly.  Host only (no
GPU): the writer is plain host code in libvfmm.so."""
import os

import numpy as np
import pytest

from oracle.vtk import reference_vtk_ascii


@pytest.fixture(scope="module")
def bodies():
    from uvlm_gb300 import workloads
    b = workloads.ring(8, seed=2)
    rng = np.random.default_rng(3)
    b["velocity"] = rng.normal(size=(b.size, 3)) * 10.0 ** rng.integers(-12, 12, size=(b.size, 3))
    b["X"][0] = (-0.0, 1e-300, 123456789.0)  # signed zero, a tiny and a long value
    b["alpha"][1] = (np.inf, -np.inf, 2.5e-7)
    return b


def test_ascii_is_the_reference_file(vfmm_lib, bodies, tmp_path):
    from uvlm_gb300 import write_vtk
    p = tmp_path / "output0.vtk"
    write_vtk(bodies, str(p))
    assert p.read_bytes() == reference_vtk_ascii(bodies)


def _read_binary(path, n):
    data = open(path, "rb").read()
    pos = 0

    def line():
        nonlocal pos
        e = data.index(b"\n", pos)
        s = data[pos:e].decode()
        pos = e + 1
        return s

    def block(dtype, count):
        nonlocal pos
        a = np.frombuffer(data, dtype=dtype, count=count, offset=pos)
        pos += a.nbytes
        return a

    assert [line() for _ in range(4)] == ["# vtk DataFile Version 3.0", "vtk output", "BINARY", "DATASET POLYDATA"]
    assert line() == f"POINTS {n} double"
    X = block(">f8", 3 * n).reshape(n, 3)
    assert line() == "" and line() == f"VERTICES {n} {2 * n}"
    V = block(">i4", 2 * n).reshape(n, 2)
    assert line() == "" and line() == f"POINT_DATA {n}" and line() == "VECTORS alpha double"
    A = block(">f8", 3 * n).reshape(n, 3)
    assert line() == "" and line() == "VECTORS velocity double"
    U = block(">f8", 3 * n).reshape(n, 3)
    assert line() == "" and line() == "SCALARS radius double" and line() == "LOOKUP_TABLE default"
    R = block(">f8", n)
    assert line() == "" and pos == len(data)
    return X, V, A, U, R


def test_binary_round_trip(vfmm_lib, bodies, tmp_path):
    from uvlm_gb300 import write_vtk
    p = tmp_path / "b.vtk"
    write_vtk(bodies, str(p), binary=True)
    X, V, A, U, R = _read_binary(p, bodies.size)
    assert np.array_equal(X, bodies["X"]) and np.array_equal(np.signbit(X), np.signbit(bodies["X"]))
    assert np.array_equal(V[:, 0], np.ones(bodies.size)) and np.array_equal(V[:, 1], np.arange(bodies.size))
    assert np.array_equal(A, bodies["alpha"]) and np.array_equal(U, bodies["velocity"])
    assert np.array_equal(R, bodies["radius"])


def test_empty_and_errors(vfmm_lib, tmp_path):
    from uvlm_gb300 import VfmmError, lib, new_bodies, write_vtk
    p = tmp_path / "empty.vtk"
    write_vtk(new_bodies(0), str(p))
    assert p.read_bytes() == reference_vtk_ascii(new_bodies(0))
    with pytest.raises(VfmmError):
        write_vtk(new_bodies(3), os.path.join(str(tmp_path), "no_such_dir", "x.vtk"))
    assert lib().vfmm_write_vtk(None, 3, str(p).encode(), 0) == 1
    assert lib().vfmm_write_vtk(None, 0, None, 0) == 1
