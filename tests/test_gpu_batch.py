"""Batched advance of independent systems (vfmm_advance_batch): every system
must come out exactly as from its own vfmm_advance (same kernels, same order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,integration", [("fp64", "RK2"), ("mixed", "RK3")])
def test_batch_equals_single(vfmm_lib, precision, integration):
    from uvlm_gb300 import FMMCalculator, advance_batch, workloads
    systems = workloads.ring_batch(6, seed=3, n_min=1500, n_max=20000) + [workloads.cloud(5000, seed=4)]
    kw = dict(p=8, ncrit=32, theta=0.5, integration=integration, precision=precision)
    ref = []
    for b in systems:
        bb = b.copy()
        with FMMCalculator(**kw) as c:
            c.advance(bb, 0.01)
            c.advance(bb, 0.01)
        ref.append(bb)
    calcs = [FMMCalculator(**kw) for _ in systems]
    out = [b.copy() for b in systems]
    advance_batch(calcs, out, 0.01)
    advance_batch(calcs, out, 0.01)
    for c in calcs:
        c.close()
    for a, r in zip(out, ref):
        for f in ["X", "alpha", "radius", "velocity", "J", "dadt"]:
            assert np.array_equal(a[f], r[f]), f


def test_batch_mixed_configurations(vfmm_lib):
    """Handles with different orders, leaf sizes and schemes in one batch."""
    from uvlm_gb300 import FMMCalculator, advance_batch, workloads
    cfgs = [dict(p=6, ncrit=16, integration="Euler"), dict(p=10, ncrit=64, integration="RK4"), dict(p=8, ncrit=32, integration="RK2",
                                                                                                   viscous="PSE", nu=0.01)]
    systems = [workloads.cloud(3000 + 2000 * k, seed=10 + k) for k in range(3)]
    ref = []
    for cfg, b in zip(cfgs, systems):
        bb = b.copy()
        with FMMCalculator(theta=0.5, **cfg) as c:
            c.advance(bb, 0.02)
        ref.append(bb)
    calcs = [FMMCalculator(theta=0.5, **cfg) for cfg in cfgs]
    out = [b.copy() for b in systems]
    advance_batch(calcs, out, 0.02)
    for c in calcs:
        c.close()
    for a, r in zip(out, ref):
        assert np.array_equal(a["X"], r["X"]) and np.array_equal(a["alpha"], r["alpha"])


def test_batch_rejects_repeated_handles(vfmm_lib):
    from uvlm_gb300 import FMMCalculator, VfmmError, advance_batch, workloads
    with FMMCalculator(p=4, ncrit=16, theta=0.5) as c:
        with pytest.raises(VfmmError):
            advance_batch([c, c], [workloads.cloud(100, seed=1), workloads.cloud(100, seed=2)], 0.01)


@pytest.mark.parametrize("P,kernel,tried", [(8, "auto", 72), (10, "tensor", 18)])
def test_autotune(vfmm_lib, P, kernel, tried):
    """The opt-in tuner returns a timed leaf size, P2P tile and (where M2L may
    run on the CUDA cores) M2L batch, keeps them, and the tuned calculator
    still meets the mixed-mode bar against FP64 at that leaf size."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(60000, seed=21)
    with FMMCalculator(p=P, ncrit=64, theta=0.5, integration="Euler", precision="mixed", m2l_kernel=kernel) as c:
        t = c.autotune(b, 0.01)
        assert t["tried"] == tried and t["ncrit"] in (16, 24, 32, 48, 64, 96, 128, 192, 256)
        assert t["p2p_chunk"] in (512, 768)
        import ctypes
        from uvlm_gb300._lib import vfmm_config
        cfg = vfmm_config()
        assert vfmm_lib.vfmm_get_config(c.handle, ctypes.byref(cfg)) == 0
        assert (cfg.ncrit, cfg.p2p_chunk) == (t["ncrit"], t["p2p_chunk"])
        if kernel == "auto":
            assert t["m2l_batch"] in (16, 24, 30, 32)
        assert t["ms_per_stage"] <= t["default_ms_per_stage"]
        bb = b.copy()
        c.init(bb)
        c.calculate()
        c.copyBodies2Host(bb)
    with FMMCalculator(p=P, ncrit=t["ncrit"], theta=0.5, precision="fp64") as c64:
        ref = b.copy()
        c64.init(ref)
        c64.calculate()
        c64.copyBodies2Host(ref)
    assert (bb["X"] == ref["X"]).all()
    err = np.linalg.norm(bb["velocity"] - ref["velocity"]) / np.linalg.norm(ref["velocity"])
    assert err < 1e-6


def test_m2l_batch_config(vfmm_lib):
    """vfmm_config.m2l_batch selects the mixed M2L source batch (what the tuner
    sets); any allowed value stays within the mixed-mode bar, others are refused."""
    from uvlm_gb300 import FMMCalculator, VfmmError, workloads
    b = workloads.cloud(30000, seed=31)
    out = {}
    for prec, mb in (("fp64", 0), ("mixed", 16), ("mixed", 24), ("mixed", 30), ("mixed", 32)):
        with FMMCalculator(p=10, ncrit=64, theta=0.5, precision=prec, m2l_batch=mb) as c:
            assert c.config.m2l_batch == mb
            bb = b.copy()
            c.init(bb)
            c.calculate()
            c.copyBodies2Host(bb)
            out[mb] = bb
    for mb in (16, 24, 30, 32):
        assert np.array_equal(out[mb]["X"], out[0]["X"])
        err = np.linalg.norm(out[mb]["velocity"] - out[0]["velocity"]) / np.linalg.norm(out[0]["velocity"])
        assert err < 1e-6
    with pytest.raises(VfmmError):
        FMMCalculator(p=10, ncrit=64, theta=0.5, precision="mixed", m2l_batch=12)
    for p, mb in ((15, 32), (16, 30)):  # staging above a block's 227 KB of shared memory
        with pytest.raises(VfmmError):
            FMMCalculator(p=p, ncrit=64, theta=0.5, precision="mixed", m2l_batch=mb)
    with FMMCalculator(p=16, ncrit=64, theta=0.5, precision="mixed", m2l_batch=24) as c:
        assert c.config.m2l_batch == 24


def test_choose_order(vfmm_lib):
    """vfmm_choose_order picks the lowest order whose velocity error against
    the model-consistent direct sum meets the tolerance: the order below it
    misses the tolerance, and the reported error is the error an evaluation at
    that order has against vfmm_direct_model."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(20000, seed=33)
    tol = 5e-3
    with FMMCalculator(p=4, ncrit=64, theta=0.5, precision="mixed") as c:
        r = c.choose_order(b, tol, pmin=4, pmax=14, targets=1000)
        p = r["p"]
        assert 4 < p < 14 and r["velocity_rel_l2_vs_model_direct"] <= tol
        lower = c.choose_order(b, tol, pmin=4, pmax=p - 1, targets=1000)
        assert lower["p"] == p - 1 and lower["velocity_rel_l2_vs_model_direct"] > tol
    with FMMCalculator(p=p, ncrit=64, theta=0.5, precision="mixed") as c:
        bb = b.copy()
        c.init(bb)
        tgt = (np.arange(1000) * b.size) // 1000
        u, _ = c.direct_model(tgt)
        c.calculate()
        c.copyBodies2Host(bb)
    err = np.linalg.norm(bb["velocity"][tgt] - u) / np.linalg.norm(u)
    assert abs(err - r["velocity_rel_l2_vs_model_direct"]) < 1e-9
