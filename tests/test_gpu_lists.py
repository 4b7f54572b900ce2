"""Interaction lists that outgrow their buffers: a handle whose list buffers
were sized on a small body set meets a much larger one, overflows, grows its
buffers and traverses again.  The lists and fields must equal those of a fresh
handle sized for the large set."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_list_overflow_retry_matches_fresh_handle(vfmm_lib, precision):
    from uvlm_gb300 import FMMCalculator, workloads
    kw = dict(p=6, ncrit=16, theta=0.5, integration="Euler", precision=precision)
    large = workloads.cloud(200000, seed=31)
    with FMMCalculator(**kw) as c:
        small = workloads.cloud(300, seed=30)
        c.init(small)
        c.calculate()
        out = large.copy()
        c.init(out)
        c.calculate()
        c.copyBodies2Host(out)
        st = c.stats()
        lists = c.lists()
    # the first buffers hold a few thousand pairs: the large set overflowed them
    assert st["m2l_pairs"] > 100000 and st["p2p_pairs"] > 10000
    with FMMCalculator(**kw) as f:
        ref = large.copy()
        f.init(ref)
        f.calculate()
        f.copyBodies2Host(ref)
        assert f.stats() == st
        ref_lists = f.lists()
    for a, b in zip(lists, ref_lists):
        assert np.array_equal(a, b)
    for fld in ["X", "velocity", "J", "dadt"]:
        assert np.array_equal(out[fld], ref[fld]), fld


def test_mixed_mode_degenerate_bounding_box(vfmm_lib):
    """One body, or every body at one point: the bounding box has R0 = 0 and the
    tree is a single root leaf.  The mixed kernels' scaling length must stay
    positive (it once became 1/0); the step leaves the bodies where they are."""
    from uvlm_gb300 import FMMCalculator, workloads
    for n in (1, 5):
        b = workloads.cloud(n, seed=50)
        b["X"] = b["X"][0]
        for prec in ("fp64", "mixed"):
            bb = b.copy()
            with FMMCalculator(p=8, ncrit=16, theta=0.5, integration="RK2", precision=prec) as c:
                c.advance(bb, 0.01)
            assert np.isfinite(bb["velocity"]).all() and np.isfinite(bb["J"]).all()
            assert np.array_equal(bb["X"], b["X"]) and np.array_equal(bb["alpha"], b["alpha"])


def test_tree_deeper_than_the_key_hint(vfmm_lib):
    """A tree build computes keys only a few levels below the depth of the
    tree its handle built last (at least 8 levels) and rebuilds with full
    keys when a cell at that depth still holds more than ncrit bodies.  A
    handle whose previous tree was shallow then gets a cluster 12 levels
    deep: tree, lists and body order must equal a fresh handle's, as must
    an advance step through the same two trees."""
    from uvlm_gb300 import FMMCalculator, workloads
    shallow = workloads.cloud(3000, seed=1)
    deep = workloads.cloud(6000, seed=2)
    deep["X"][:300] = deep["X"][0] + 1e-5 * np.random.default_rng(3).normal(size=(300, 3))
    out = []
    for warm in (True, False):
        with FMMCalculator(p=6, ncrit=16, theta=0.5) as c:
            if warm:
                b0 = shallow.copy()
                c.init(b0)
                assert c.stats()["max_level"] <= 4
            b = deep.copy()
            c.init(b)
            cells = c.tree()
            p2p, m2l = c.lists()
            depth = c.stats()["max_level"]
            c.calculate()
            c.copyBodies2Host(b)
            out.append((b, cells, p2p, m2l, depth))
    (b1, c1, p1, m1, d1), (b2, c2, p2, m2, d2) = out
    assert d1 == d2 and d1 > 11
    assert np.array_equal(b1, b2) and np.array_equal(c1, c2)
    assert np.array_equal(p1, p2) and np.array_equal(m1, m2)
