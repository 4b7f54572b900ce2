"""Sensor points (FMMCalculator::getSensorData, fmmCalculator.hpp:726-731)
through the C ABI against the reference's golden fixture and the oracle.

The sensor tree and its order are bit-exact; velocity and J within 1e-10
(max-abs relative).  J of sensors within sin(theta) < 1e-4 of their leaf's z
axis is held to 1e-6 instead: there the reference's complex-step L2P loses
accuracy that the Cartesian derivatives here keep (see near_axis_mask)."""
import numpy as np
import pytest

from conftest import golden, golden_bodies, rel
from test_gpu_parity import near_axis_mask

pytestmark = pytest.mark.gpu
TOL = 1e-10


def sensor_points(n, lo, hi, seed, j_scale=0.0):
    from uvlm_gb300._lib import BODY_DTYPE
    rng = np.random.default_rng(seed)
    s = np.zeros(n, BODY_DTYPE)
    s["X"] = rng.uniform(lo, hi, (n, 3))
    if j_scale:
        s["J"] = rng.normal(0, j_scale, (n, 3, 3))  # kept and added to, as the reference's L2P does
        s["dadt"] = 1.0  # reset to zero by getSensorData
    return s


def at_leaf_centre(cells, X):
    """Sensors that sit exactly on their leaf's centre (r = 0 in L2P)."""
    hit = np.zeros(len(X), bool)
    for c in cells[cells["NCHILD"] == 0]:
        sl = slice(int(c["BodyOffset"]), int(c["BodyOffset"] + c["NBODY"]))
        hit[sl] = (X[sl] == c["X"]).all(1)
    return hit


def check_against(s, ref, ncrit, bodies=None, P=None, theta=0.5):
    """s (GPU) against ref (oracle or fixture).  The reference's L2P converts
    the offset from the leaf centre to spherical coordinates and yields NaN
    at r = 0 (the n/r factors of multipoleKernels.hpp:662-677 are 0/0 there;
    cart2sph, :27-32, returns r = 0); the Cartesian L2P here gives the
    finite limit.  Such a point is checked against the oracle for the point
    plus a companion 1e-9 away, which moves it off the leaf centre."""
    from oracle import oracle as O
    assert (s["X"] == ref["X"]).all(), "sensor tree order"
    _, cells = O.build_tree(ref, ncrit)
    nan = np.isnan(ref["velocity"]).any(1) | np.isnan(ref["J"].reshape(-1, 9)).any(1)
    assert (nan == (nan & at_leaf_centre(cells, ref["X"]))).all(), "NaN in the reference only at r = 0"
    ok = ~nan
    axis = near_axis_mask(cells, ref["X"])
    assert rel(s["velocity"][ok], ref["velocity"][ok]) < TOL
    assert rel(s["J"][ok & ~axis], ref["J"][ok & ~axis]) < TOL
    assert rel(s["J"][ok], ref["J"][ok]) < 1e-6
    assert (s["dadt"] == 0).all()
    if nan.any():
        from uvlm_gb300._lib import BODY_DTYPE
        assert np.isfinite(s["velocity"][nan]).all() and np.isfinite(s["J"][nan]).all()
        for x in ref["X"][nan]:
            pair = np.zeros(2, BODY_DTYPE)
            pair["X"] = [x, x + 1e-9]
            _, r2 = O.sensors(bodies, pair, P, ncrit, theta)
            k = np.flatnonzero((r2["X"] == x).all(1))[0]
            i = np.flatnonzero((s["X"] == x).all(1))[0]
            assert rel(s["velocity"][i], r2["velocity"][k]) < 1e-6


def test_sensors_match_reference(vfmm_lib):
    from uvlm_gb300 import FMMCalculator
    from uvlm_gb300._lib import BODY_DTYPE
    d = golden("sensors_p6")
    b = golden_bodies(d)
    s = np.zeros(len(d["sensor_X"]), BODY_DTYPE)
    s["X"] = d["sensor_X"]
    with FMMCalculator(p=int(d["P"]), ncrit=int(d["ncrit"]), theta=float(d["theta"])) as c:
        c.init(b)
        c.calculate()
        c.getSensorData(s)
    ref = np.zeros_like(s)
    ref["X"] = d["sensor_X"][d["sensor_perm"]]
    ref["velocity"] = d["sensor_velocity"]
    ref["J"] = d["sensor_J"]
    check_against(s, ref, int(d["ncrit"]))


@pytest.mark.parametrize("n,ns,P,ncrit,box", [(20000, 5000, 8, 32, 1.5), (3000, 40000, 10, 64, 0.8), (500, 1, 6, 16, 1.0),
                                              (1, 200, 4, 16, 1.0)])
def test_sensors_against_oracle(vfmm_lib, n, ns, P, ncrit, box):
    """Sensor sets larger and smaller than the particle cloud, inside and
    around it; one sensor; one particle."""
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(n, seed=31)
    s = sensor_points(ns, -box, box, seed=32, j_scale=0.1)
    _, ref = O.sensors(b, s, P, ncrit, 0.5)
    with FMMCalculator(p=P, ncrit=ncrit, theta=0.5) as c:
        bb = b.copy()
        c.init(bb)
        c.calculate()
        ss = s.copy()
        c.getSensorData(ss)
    check_against(ss, ref, ncrit, b, P)


def test_sensors_on_particles(vfmm_lib):
    """Sensors placed on particles: the R^2 == 0 pairs are skipped, as in the
    reference's P2P (multipoleKernels.hpp:321)."""
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(4000, seed=5)
    s = sensor_points(600, -1, 1, seed=6)
    s["X"][:300] = b["X"][:300]
    _, ref = O.sensors(b, s, 6, 32, 0.5)
    with FMMCalculator(p=6, ncrit=32, theta=0.5) as c:
        bb = b.copy()
        c.init(bb)
        c.calculate()
        c.getSensorData(s)
    check_against(s, ref, 32)


def test_sensors_mixed_precision(vfmm_lib):
    """Mixed mode: multipoles from the FP32 P2M; the sensor pass itself is FP64."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(30000, seed=8)
    s = sensor_points(3000, -1.2, 1.2, seed=9)
    out = {}
    for prec in ["fp64", "mixed"]:
        with FMMCalculator(p=8, ncrit=32, theta=0.5, precision=prec) as c:
            bb = b.copy()
            c.init(bb)
            c.calculate()
            ss = s.copy()
            c.getSensorData(ss)
            out[prec] = ss
    assert (out["fp64"]["X"] == out["mixed"]["X"]).all()
    err = np.linalg.norm(out["mixed"]["velocity"] - out["fp64"]["velocity"]) / np.linalg.norm(out["fp64"]["velocity"])
    assert err < 1e-6


def test_sensors_need_an_evaluation(vfmm_lib):
    from uvlm_gb300 import FMMCalculator, VfmmError, workloads
    from uvlm_gb300._lib import VFMM_ERR_STATE
    b = workloads.cloud(300, seed=1)
    s = sensor_points(10, -1, 1, seed=2)
    with FMMCalculator(p=4, ncrit=16, theta=0.5) as c:
        c.init(b)
        with pytest.raises(VfmmError) as e:
            c.getSensorData(s)
        assert e.value.code == VFMM_ERR_STATE
        c.calculate()
        c.getSensorData(s)  # and the particle state stays usable afterwards
        c.calculate()
        c.getSensorData(s)
