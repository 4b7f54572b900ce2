"""Vorticity re-interpolation (FMMCalculator::RBF, fmmCalculator.hpp:856-917)
through the C ABI against the reference's own RBF run on the same inputs.

The particle permutation, the set and order of the kept points are exact; the
strengths (the conjugate-gradient solution) within 1e-10 max-abs relative."""
import numpy as np
import pytest

from conftest import golden, golden_bodies, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["rbf_cloud", "rbf_ring_c32"])
def test_rbf_matches_reference(vfmm_lib, name):
    from uvlm_gb300 import FMMCalculator
    from uvlm_gb300._lib import BODY_DTYPE
    d = golden(name)
    particles = golden_bodies(d)
    pts = np.zeros(len(d["points_X"]), BODY_DTYPE)
    pts["X"] = d["points_X"]
    pts["radius"] = d["points_radius"]
    with FMMCalculator(p=int(d["P"]), ncrit=int(d["ncrit"]), theta=float(d["theta"])) as c:
        kept, iters = c.RBF(particles, pts)
    assert (particles["X"] == d["out_particles_X"]).all(), "particles in tree order"
    assert len(kept) == len(d["out_X"]), "points kept"
    assert (kept["X"] == d["out_X"]).all(), "kept points in their tree order"
    assert rel(kept["velocity_old"], d["out_vorticity"]) < 1e-10
    assert rel(kept["alpha"], d["out_alpha"]) < 1e-10
    assert 0 < iters <= 100


def test_rbf_rejects_empty(vfmm_lib):
    from uvlm_gb300 import FMMCalculator, VfmmError, workloads
    from uvlm_gb300._lib import BODY_DTYPE
    with FMMCalculator(p=4, ncrit=16, theta=0.5) as c:
        with pytest.raises(VfmmError):
            c.RBF(workloads.cloud(100, seed=1), np.zeros(0, BODY_DTYPE))
