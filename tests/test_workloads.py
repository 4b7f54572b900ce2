"""The synthetic workloads' host-side construction (no GPU)."""
import numpy as np

from uvlm_gb300 import workloads


def test_wing_wake_shedding_rule():
    """400 particles per step (40 TE panels x 10 segments), 160,000 after 400
    steps; the trailing (side-line) vorticity of one step sums to zero along
    the chord direction (the neighbour halves cancel and the tips close the
    loop); the spanwise part is the TE line times the change of Gamma (the
    starting vortex at the first step, none after it for the steady
    prescribed Gamma), or times Gamma every step under the reference
    driver's rule (src/main.cpp:246-289)."""
    r = workloads.WingWake(rule="reference")
    r.shed()
    assert np.allclose(r.shed()["alpha"][:, 1], -r.gamma * r.b / r.ns)
    w = workloads.WingWake()
    p = w.shed()
    assert p.size == 400
    side = p["alpha"] @ w.ex / np.linalg.norm(w.side)  # chordwise component per unit side-line length
    assert abs(side.sum()) < 1e-12 * np.abs(side).sum()
    dy = w.b / w.ns
    assert np.allclose(p["alpha"][:, 1], -w.gamma * dy)
    assert np.allclose(p["radius"], 1.3 * dy)
    # the wing moves by -U dt per step; shed particles sit one step behind its TE
    q = w.shed()
    assert np.allclose(q["X"][:, 0] - p["X"][:, 0], -w.U * w.dt)
    assert np.all(q["alpha"][:, 1] == 0)
    for _ in range(398):
        w.shed()
    assert w.step_index * w.ns == 160000


def test_ring_configuration_size():
    b = workloads.ring(256, seed=0)
    assert b.size == 32512
    assert np.allclose(b["radius"], 1.3 * 2 * np.pi / 256)
