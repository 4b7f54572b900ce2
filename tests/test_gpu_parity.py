"""CUDA path (libvfmm.so through the C ABI) against the reference's golden
fixtures and the oracle restatement.  Bit-exact for the tree, the body order
and the interaction lists; FP64 fields within 1e-10 (max-abs relative), the
bar the drop-in must meet against the reference's own FMM."""
import numpy as np
import pytest

from conftest import golden, golden_bodies, rel

pytestmark = pytest.mark.gpu

EVAL = ["cloud_p6_c16_t05", "ring_p8_c32_t05", "cloud_p10_c64_t05", "cloud_p4_c128_t03", "cloud_p14_c32_t05",
        "classic_rvpm_p6", "root_leaf", "coincident", "lattice_ties"]
ADV = ["advance_rk2_ring", "advance_rk3_cloud", "advance_euler_cloud", "advance_rk4_cloud", "advance_rvpm_rk2_ring",
       "advance_rvpm_rk3_cloud"]
TOL = 1e-10
SCHEMES = {0: "Euler", 1: "RK2", 2: "RK3", 3: "RK4"}


def calc_for(d, **kw):
    from uvlm_gb300 import FMMCalculator
    form = int(d["formulation"]) if "formulation" in d.files else 0
    return FMMCalculator(p=int(d["P"]), ncrit=int(d["ncrit"]), theta=float(d["theta"]),
                         stretching="Classic" if int(d["stretching"]) else "Transposed",
                         formulation="rVPM" if form else "cVPM", **kw)


def near_axis_mask(cells, X, limit=1e-4):
    """Bodies (tree order) whose offset from their leaf centre is within
    sin(theta) < limit of the leaf's z axis.  There the reference's L2P, which
    differentiates in spherical coordinates by a complex step and divides by
    sin(theta) (multipoleKernels.hpp:44-47, :94-134), loses up to ~1e-8 of
    J's absolute accuracy; the Cartesian derivatives used here do not."""
    mask = np.zeros(len(X), bool)
    for c in cells[cells["NCHILD"] == 0]:
        s = slice(int(c["BodyOffset"]), int(c["BodyOffset"] + c["NBODY"]))
        d = X[s] - c["X"]
        r = np.sqrt((d ** 2).sum(1))
        mask[s] = np.hypot(d[:, 0], d[:, 1]) < limit * np.maximum(r, 1e-300)
    return mask


@pytest.mark.parametrize("name", EVAL)
def test_tree_lists_exact(vfmm_lib, name):
    d = golden(name)
    b = golden_bodies(d)
    with calc_for(d) as c:
        bb = b.copy()
        c.init(bb)
        assert (bb["X"] == b["X"][d["perm"]]).all(), "body order"
        cells = c.tree()
        ref = d["cells"]
        assert cells.shape == ref.shape
        for f in ["NCHILD", "NBODY", "ChildOffset", "BodyOffset", "level"]:
            assert (cells[f] == ref[f]).all(), f
        assert (cells["X"] == ref["X"]).all() and (cells["R"] == ref["R"]).all()
        p2p, m2l = c.lists()
        assert (p2p == d["p2p"]).all()
        assert (m2l == d["m2l"]).all()


@pytest.mark.parametrize("name", EVAL)
def test_evaluation_matches_reference(vfmm_lib, name):
    d = golden(name)
    b = golden_bodies(d)
    with calc_for(d) as c:
        bb = b.copy()
        c.init(bb)
        c.calculate()
        c.copyBodies2Host(bb)
        if "M" in d.files:
            M, L = c.expansions()
            sel = d["cell_sel"]
            assert rel(M[sel], d["M"]) < TOL
            assert rel(L[sel], d["L"]) < TOL
    axis = near_axis_mask(d["cells"], bb["X"])
    for f in ["velocity", "J", "dadt", "drdt"]:
        assert rel(bb[f][~axis], d[f][~axis]) < TOL, f
        assert rel(bb[f], d[f]) < 1e-6, f


@pytest.mark.parametrize("name", ADV)
def test_advance_matches_reference(vfmm_lib, name):
    d = golden(name)
    b = golden_bodies(d)
    with calc_for(d, integration=SCHEMES[int(d["scheme"])]) as c:
        for _ in range(int(d["steps"])):
            c.advance(b, float(d["dt"]))
    for f in ["X", "alpha", "radius", "velocity", "J"]:
        assert rel(b[f], d["out_" + f]) < TOL, f


@pytest.mark.parametrize("kind,n,P,ncrit", [("cloud", 20000, 8, 32), ("ring", 64, 8, 32), ("cloud", 30000, 12, 64)])
def test_larger_against_oracle(vfmm_lib, kind, n, P, ncrit):
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(n, seed=21) if kind == "cloud" else workloads.ring(n, seed=21)
    ob, oc = O.build_tree(b, ncrit)
    ref = O.calculate(b, P, ncrit, 0.5)
    with FMMCalculator(p=P, ncrit=ncrit, theta=0.5) as c:
        bb = b.copy()
        c.init(bb)
        assert (bb["X"] == ob["X"]).all()
        cells = c.tree()
        assert cells.shape == oc.shape and (cells == oc).all()
        p2p, m2l = c.lists()
        op2p, om2l = O.lists(oc, 0.5)
        assert (p2p == op2p[np.lexsort((op2p[:, 1], op2p[:, 0]))]).all()
        assert (m2l == om2l[np.lexsort((om2l[:, 1], om2l[:, 0]))]).all()
        c.calculate()
        c.copyBodies2Host(bb)
    for f in ["velocity", "J", "dadt"]:
        assert rel(bb[f], ref[f]) < TOL, f


def test_ring_configuration_against_oracle(vfmm_lib):
    """The plain FP64 ring configuration as specified: 256 stations x 127
    points (32,512 bodies), p = 8, theta = 0.5, leaf 32, ten RK2 steps of
    dt = 0.01 with relaxation (factor 0.3) after each step, through
    vfmm_advance, against the oracle restatement of the reference's advance.

    At theta = 0.5 cells two apart on the octree lattice sit exactly on the
    MAC boundary |dX| theta = Ri + Rj, so the last bit of the centre
    arithmetic decides between M2L and P2P for them, in the reference too: on
    the oracle alone, a 1-ulp nudge of one body's position moves this
    configuration's 10-step result by 1e-4 (by 7e-16 at theta = 0.47).  Two
    codes that sum in different orders therefore cannot follow one another for
    ten free-running steps at theta = 0.5.  So every step is compared from the
    same input state (the oracle restarted from the GPU's state each step), at
    1e-10; and ten free-running steps are compared at theta = 0.47.  The
    strengths after relaxation (factor 0.3) are held to 1e-9: relaxation
    turns alpha towards w / |w|, w a difference of J entries, which amplifies
    the rounding differences of J (measured 1.04e-10 at the first step).
    Within a step the ties stay: the first stage's positions differ from the
    oracle's by a few units in the last place (the velocity sums run in another
    order), and that can flip a MAC tie of the second stage's tree (at the
    first step, 4 of the 32,512 bodies, J off by 2.7e-9 of its largest entry;
    Euler steps match to 1e-12).  So J is held to 1e-10 on all but at most
    0.1% of the bodies and to 1e-6 on all."""
    import time
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(256, seed=0)
    assert b.size == 32512
    t_cpu = t_gpu = 0.0
    with FMMCalculator(p=8, ncrit=32, theta=0.5, integration="RK2", relax=0.3) as c:
        c.advance(b.copy(), 0.01)  # warm-up (buffers, kernels)
        state = b.copy()
        for step in range(10):
            t0 = time.perf_counter()
            ref = O.advance(state, 8, 32, 0.5, 0.01, 1, 1, relax=0.3)
            t_cpu += time.perf_counter() - t0
            t0 = time.perf_counter()
            c.advance(state, 0.01)
            t_gpu += time.perf_counter() - t0
            for f in ["X", "alpha", "radius", "velocity"]:
                assert rel(state[f], ref[f]) < (1e-9 if f == "alpha" else TOL), (step, f)
            dJ = np.abs(state["J"] - ref["J"]).reshape(-1, 9).max(1) / np.abs(ref["J"]).max()
            assert np.mean(dJ > TOL) <= 1e-3 and dJ.max() < 1e-6, (step, np.sum(dJ > TOL), dJ.max())
    print(f"ring 32,512 bodies, 10 RK2 steps with relaxation, theta 0.5: GPU FP64 {t_gpu:.3f} s, oracle (CPU) {t_cpu:.2f} s")
    ref = O.advance(b, 8, 32, 0.47, 0.01, 10, 1, relax=0.3)
    with FMMCalculator(p=8, ncrit=32, theta=0.47, integration="RK2", relax=0.3) as c:
        bb = b.copy()
        for _ in range(10):
            c.advance(bb, 0.01)
    for f in ["X", "alpha", "radius", "velocity", "J"]:
        assert rel(bb[f], ref[f]) < (1e-9 if f == "alpha" else TOL), f


def test_direct_model_against_oracle(vfmm_lib):
    """vfmm_direct_model (regularised kernel on P2P-list leaf pairs, singular
    elsewhere) against the oracle's restatement on the same tree; and the FMM's
    distance from it equals the oracle FMM's (the truncation error)."""
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(20000, seed=31)
    with FMMCalculator(p=10, ncrit=64, theta=0.5) as c:
        bb = b.copy()
        c.init(bb)
        cells = c.tree()
        p2p, _ = c.lists()
        tgt = np.arange(0, bb.size, 61)
        u, J = c.direct_model(tgt)
        c.calculate()
        c.copyBodies2Host(bb)
    ref = O.direct_model(bb, cells, p2p, tgt)
    # J: the near pairs' (regularised - singular) terms are differences of
    # values up to ~1/R^3 that cancel to a small remainder, and the device and
    # host sum them in different orders (measured 7e-12): the FP64 fields' bar
    assert rel(u, ref[:, :3]) < 1e-12
    assert rel(J.reshape(-1, 9), ref[:, 3:]) < 1e-10
    e_gpu = rel_l2(bb["velocity"][tgt], u)
    fmm = O.calculate(b, 10, 64, 0.5)
    e_cpu = rel_l2(fmm["velocity"][tgt], ref[:, :3])
    assert e_cpu > 1e-6 and abs(e_gpu - e_cpu) < 1e-8, (e_gpu, e_cpu)


def test_direct_sum_against_oracle(vfmm_lib):
    from oracle import oracle as O
    from uvlm_gb300 import direct, workloads
    src = workloads.cloud(5000, seed=3)
    tgt = src[:700].copy()
    out = direct(tgt, src)
    ref = O.direct(tgt, src)
    assert rel(out["velocity"], ref["velocity"]) < 1e-13
    assert rel(out["J"], ref["J"]) < 1e-13


def test_relaxation_matches_oracle(vfmm_lib):
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(16, seed=4)
    ref = O.advance(b, 6, 32, 0.5, 0.01, 2, 1, relax=0.3)
    with FMMCalculator(p=6, ncrit=32, theta=0.5, integration="RK2", relax=0.3) as c:
        for _ in range(2):
            c.advance(b, 0.01)
    for f in ["X", "alpha", "velocity"]:
        assert rel(b[f], ref[f]) < TOL, f


def test_errors_are_reported(vfmm_lib):
    from uvlm_gb300 import FMMCalculator, VfmmError, workloads
    b = workloads.cloud(500, seed=1)
    b["X"][17, 1] = np.nan
    with FMMCalculator(p=6, ncrit=16, theta=0.5) as c:
        with pytest.raises(VfmmError) as e:
            c.init(b.copy())
        assert e.value.code == 2
        dup = workloads.cloud(100, seed=2)
        dup["X"][:40] = dup["X"][0]  # 40 coincident bodies > ncrit: no depth splits them
        with pytest.raises(VfmmError) as e:
            c.init(dup)
        assert e.value.code == 3
        with pytest.raises(VfmmError) as e:
            c.calculate()  # no valid tree after the failed init
        # a good call still works on the same handle afterwards
        good = workloads.cloud(300, seed=3)
        c.init(good)
        c.calculate()
    with pytest.raises(VfmmError):
        FMMCalculator(p=40)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("kind,n,P,ncrit,theta", [("cloud", 40000, 10, 64, 0.5), ("cloud", 20000, 14, 64, 0.5), ("cloud", 20000, 6, 64, 0.5),
                                                  ("ring", 96, 8, 32, 0.5), ("cloud", 15000, 16, 64, 0.5), ("ring", 48, 15, 32, 0.5),
                                                  ("cloud", 3000, 3, 16, 0.5), ("cloud", 20000, 8, 32, 0.3),
                                                  ("cloud", 30000, 9, 64, 0.5), ("ring", 64, 10, 32, 0.5), ("cloud", 20000, 10, 32, 0.3)])
def test_mixed_matches_fp64_fmm(vfmm_lib, kind, n, P, ncrit, theta):
    """The mixed path (FP32 expansion kernels and P2P, FP64 tree) against the
    FP64 path on the same tree: relative L2 error of velocity and of J below
    1e-6 (the precision bar of the mixed mode).  At theta = 0.3 (the
    reference's default) many P2P rows span more than 128 leaves, which the
    leaf kernel stages in several groups."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(n, seed=5) if kind == "cloud" else workloads.ring(n, seed=5)
    out = {}
    for prec in ["fp64", "mixed"]:
        with FMMCalculator(p=P, ncrit=ncrit, theta=theta, precision=prec) as c:
            bb = b.copy()
            c.init(bb)
            c.calculate()
            c.copyBodies2Host(bb)
            out[prec] = bb
    assert (out["fp64"]["X"] == out["mixed"]["X"]).all()
    ev = rel_l2(out["mixed"]["velocity"], out["fp64"]["velocity"])
    eJ = rel_l2(out["mixed"]["J"], out["fp64"]["J"])
    ed = rel_l2(out["mixed"]["dadt"], out["fp64"]["dadt"])
    print(f"{kind} n={n} P={P}: velocity {ev:.3e}  J {eJ:.3e}  dadt {ed:.3e}")
    assert ev < 1e-6 and eJ < 1e-6 and ed < 1e-6, (ev, eJ, ed)


def test_tensor_m2l_repeatable(vfmm_lib):
    """The tensor-core M2L is bit-reproducible: repeated evaluations on one
    handle (the first builds the classes beyond its initial operator table
    inside the kernel, later ones read the grown table; tiles go to whichever
    block is free, and the pre-pass runs on a second stream) and an evaluation
    on a fresh handle give identical fields."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(200000, seed=41)
    outs = []
    kw = dict(p=10, ncrit=64, theta=0.5, precision="mixed", m2l_kernel="tensor")
    with FMMCalculator(**kw) as c:
        for _ in range(3):
            bb = b.copy()
            c.init(bb)
            c.calculate()
            c.copyBodies2Host(bb)
            outs.append(bb)
        assert c.stats()["m2l_tensor"] == 1
    with FMMCalculator(**kw) as c:
        bb = b.copy()
        c.init(bb)
        c.calculate()
        c.copyBodies2Host(bb)
        outs.append(bb)
    for o in outs[1:]:
        for f in ("velocity", "J", "dadt"):
            assert np.array_equal(o[f], outs[0][f]), f


@pytest.mark.parametrize("P,formulation,stretching", [(10, "cVPM", "Transposed"), (9, "rVPM", "Classic"), (8, "rVPM", "Transposed")])
def test_split_leaf_kernel_matches_fused(vfmm_lib, monkeypatch, P, formulation, stretching):
    """With the tensor-core M2L the leaf kernel runs in two passes: the near
    field on a second stream beside M2L (its combined sums kept per body as
    float-float pairs), then the far field, those sums and the epilogue after
    L2L; VFMM_P2P_OVERLAP=0 keeps the fused kernel.  The two add the same terms
    in another order: they agree to FP32 rounding, and the split form is
    bit-reproducible."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(150000, seed=8)
    out = {}
    for ov in ("0", "1", "1"):
        monkeypatch.setenv("VFMM_P2P_OVERLAP", ov)
        with FMMCalculator(p=P, ncrit=64, theta=0.5, precision="mixed", m2l_kernel="tensor", formulation=formulation,
                           stretching=stretching) as c:
            bb = b.copy()
            c.init(bb)
            c.calculate()
            c.copyBodies2Host(bb)
            assert c.stats()["m2l_tensor"] == 1
        if ov in out:
            for f in ("velocity", "J", "dadt", "drdt"):
                assert np.array_equal(bb[f], out[ov][f]), f
        out[ov] = bb
    fields = ("velocity", "J", "dadt") + (("drdt",) if formulation == "rVPM" else ())
    for f in fields:
        assert rel_l2(out["1"][f], out["0"][f]) < 1e-6, f


@pytest.mark.parametrize("ncrit,formulation,stretching", [(256, "rVPM", "Transposed"), (128, "cVPM", "Classic"), (64, "rVPM", "Classic"),
                                                         (16, "rVPM", "Transposed")])
def test_mixed_leaf_sizes_and_stretching(vfmm_lib, ncrit, formulation, stretching):
    """The mixed leaf kernel's per-body epilogue (four lanes per body: velocity
    and one dadt component each, the rVPM dot product summed across the four)
    against the FP64 path: leaves of up to 256 bodies (target chunks of 128, so
    several passes of the four-lane loop), classic and transposed stretching,
    cVPM and rVPM."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(40000, seed=9)
    out = {}
    for prec in ["fp64", "mixed"]:
        with FMMCalculator(p=10, ncrit=ncrit, theta=0.5, precision=prec, formulation=formulation, stretching=stretching) as c:
            bb = b.copy()
            c.init(bb)
            c.calculate()
            c.copyBodies2Host(bb)
            out[prec] = bb
    assert (out["fp64"]["X"] == out["mixed"]["X"]).all()
    ev = rel_l2(out["mixed"]["velocity"], out["fp64"]["velocity"])
    eJ = rel_l2(out["mixed"]["J"], out["fp64"]["J"])
    ed = rel_l2(out["mixed"]["dadt"], out["fp64"]["dadt"])
    assert ev < 1e-6 and eJ < 1e-6 and ed < 1e-6, (ev, eJ, ed)


@pytest.mark.parametrize("kind,n,P,ncrit,theta", [("cloud", 40000, 10, 64, 0.5), ("cloud", 30000, 9, 64, 0.5), ("cloud", 20000, 8, 32, 0.3),
                                                  ("ring", 96, 8, 32, 0.5), ("ring", 64, 10, 32, 0.5), ("leapfrog", 64, 10, 32, 0.47),
                                                  ("wing", 60, 10, 64, 0.5)])
def test_tensor_m2l_matches_fp64_fmm(vfmm_lib, kind, n, P, ncrit, theta):
    """The tensor-core M2L (forced: small sets choose the CUDA-core kernel by
    size) against the FP64 FMM on the same tree, within the mixed-mode bar:
    uniform clouds, thin rings and two rings (cross-level pairs, many offset
    classes: some built in the kernel beyond the first evaluation's table),
    and a wing wake after `n` steps of shedding (an adaptive sheet)."""
    from uvlm_gb300 import FMMCalculator, workloads
    if kind == "cloud":
        b = workloads.cloud(n, seed=5)
    elif kind == "ring":
        b = workloads.ring(n, seed=5)
    elif kind == "leapfrog":
        b = workloads.leapfrog(n, seed=5)
    else:
        w = workloads.WingWake()
        b = np.concatenate([w.shed() for _ in range(n)])
        b["X"] += np.random.default_rng(5).normal(0.0, 0.02, b["X"].shape)  # a roughened sheet
    out = {}
    for prec, kernel in (("fp64", "auto"), ("mixed", "tensor")):
        with FMMCalculator(p=P, ncrit=ncrit, theta=theta, precision=prec, m2l_kernel=kernel) as c:
            bb = b.copy()
            c.init(bb)
            c.calculate()
            c.copyBodies2Host(bb)
            out[prec] = bb
    assert (out["fp64"]["X"] == out["mixed"]["X"]).all()
    ev = rel_l2(out["mixed"]["velocity"], out["fp64"]["velocity"])
    eJ = rel_l2(out["mixed"]["J"], out["fp64"]["J"])
    ed = rel_l2(out["mixed"]["dadt"], out["fp64"]["dadt"])
    print(f"tensor M2L {kind} n={n} P={P}: velocity {ev:.3e}  J {eJ:.3e}  dadt {ed:.3e}")
    assert ev < 1e-6 and eJ < 1e-6 and ed < 1e-6, (ev, eJ, ed)


VISC = {"advance_pse_cloud": "PSE", "advance_pse_rk3_ring": "PSE", "advance_csm_cloud": "CSM"}


@pytest.mark.parametrize("name", list(VISC))
def test_advance_viscous_matches_reference(vfmm_lib, name):
    """PSE and CSM (calculateViscosity, fmmCalculator.hpp:713-724) against the
    reference's own advance with the viscosity set."""
    d = golden(name)
    b = golden_bodies(d)
    with calc_for(d, integration=SCHEMES[int(d["scheme"])], viscous=VISC[name], nu=float(d["nu"])) as c:
        for _ in range(int(d["steps"])):
            c.advance(b, float(d["dt"]))
    for f in ["X", "alpha", "radius", "velocity", "J"]:
        assert rel(b[f], d["out_" + f]) < TOL, f


def test_pse_mixed_matches_fp64(vfmm_lib):
    """The FP32 PSE of the mixed mode against the FP64 one: the viscous part of
    the strengths after one Euler stage (PSE run minus inviscid run), relative L2."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.cloud(30000, seed=17)
    da = {}
    for prec in ["fp64", "mixed"]:
        out = {}
        for visc in ["Inviscid", "PSE"]:
            with FMMCalculator(p=8, ncrit=32, theta=0.5, integration="Euler", precision=prec, viscous=visc, nu=0.01) as c:
                bb = b.copy()
                c.advance(bb, 0.01)
                out[visc] = bb
        assert (out["PSE"]["X"] == out["Inviscid"]["X"]).all()  # same tree order
        da[prec] = out["PSE"]["alpha"] - out["Inviscid"]["alpha"]
    assert np.abs(da["fp64"]).max() > 0
    assert rel_l2(da["mixed"], da["fp64"]) < 1e-5


def test_diagnostics_against_host(vfmm_lib):
    """Circulation and impulses of the device bodies against a host FP64 sum,
    before and after an advance."""
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(64, seed=2)
    with FMMCalculator(p=8, ncrit=32, theta=0.5, integration="RK2") as c:
        c.load(b)
        for step in range(2):
            d = c.diagnostics()
            if step:
                c.copyBodies2Host(b)
            x, a = b["X"], b["alpha"]
            xa = np.cross(x, a)
            xxa = np.cross(x, xa)
            host = {"circulation": (a.sum(0), np.abs(a).sum()), "linear_impulse": (0.5 * xa.sum(0), np.abs(xa).sum()),
                    "angular_impulse": (xxa.sum(0) / 3, np.abs(xxa).sum())}
            for k, (v, mag) in host.items():  # the sums may cancel: compare against the size of their terms
                assert np.abs(d[k] - v).max() < 1e-13 * mag, k
            c.advance(b, 0.01)
            c.load(b)
