"""vfmm_bounds_noalloc: the allocation-free root-cell computation, for callers
that cannot call cudaMalloc (CUDA-graph capture, pooled device memory,
plugins that must not touch the allocator).  Collected last on purpose.

Checked through the C ABI against the existing entry points (vfmm_init +
vfmm_get_tree, whose cell 0 is the root): the centre and half-width must be
identical, as the tree tests require of all tree quantities.  Two calls in a
row with different bodies, so that a stale scratch array would show."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _root_from_tree(bodies):
    from uvlm_gb300 import FMMCalculator
    with FMMCalculator(p=4, ncrit=64, theta=0.5) as c:
        b = bodies.copy()
        c.init(b)
        root = c.tree()[0]
    return np.array([*root["X"], root["R"]])


def test_bounds_noalloc_matches_tree_root(vfmm_lib):
    import torch
    from uvlm_gb300 import workloads
    for n, seed, shift in [(100_000, 1, 0.0), (777, 2, 3.5)]:
        b = workloads.cloud(n, seed=seed)
        b["X"] += shift
        xyz = [torch.tensor(np.ascontiguousarray(b["X"][:, d]), dtype=torch.float64, device="cuda") for d in range(3)]
        out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = vfmm_lib.vfmm_bounds_noalloc(xyz[0].data_ptr(), xyz[1].data_ptr(), xyz[2].data_ptr(), n, out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        want = _root_from_tree(b)
        assert (got == want).all(), (got, want)


def test_bounds_noalloc_rejects_bad_sizes(vfmm_lib):
    import torch
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    assert vfmm_lib.vfmm_bounds_noalloc(p, p, p, 0, p, None) == 1
    assert vfmm_lib.vfmm_bounds_noalloc(p, p, p, 2**31, p, None) == 1
    assert vfmm_lib.vfmm_bounds_noalloc(None, p, p, 4, p, None) == 1
