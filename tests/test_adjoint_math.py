"""The closed-form adjoint of one near-field pair used by the reverse-mode P2P
(adjoint.cu pair_adj), restated in numpy and checked against 40-digit central
differences of the forward pair terms of the team P2P
(multipoleKernels.hpp:239-283).  CPU only."""
import numpy as np
import pytest


def forward_s(mp, d, al, sg, ub, Jb):
    """ubar . u + Jbar : J of one pair (target - source = d, source strength al,
    source radius sg), in mpmath, following the reference's operation order."""
    d = [mp.mpf(x) for x in d]
    al = [mp.mpf(x) for x in al]
    sg = mp.mpf(sg)
    R2 = sum(x * x for x in d)
    S2 = sg * sg
    RS = R2 / S2 / 2
    sRS = mp.sqrt(RS)
    t2 = 2 / mp.sqrt(mp.pi) * sRS * mp.exp(-RS)
    c4 = mp.mpf(1) / 4 / mp.pi / R2 / mp.sqrt(R2)
    gg = mp.erf(sRS) - t2
    cr = [c4 * (d[1] * al[2] - d[2] * al[1]), c4 * (d[2] * al[0] - d[0] * al[2]), c4 * (d[0] * al[1] - d[1] * al[0])]
    aux, a2 = t2 / S2 - 3 * gg / R2, gg * c4
    M = [[0, al[2], -al[1]], [-al[2], 0, al[0]], [al[1], -al[0], 0]]
    s = sum(-ub[a] * cr[a] * gg for a in range(3))
    for a in range(3):
        for b in range(3):
            s += Jb[a][b] * (-aux * cr[a] * d[b] - a2 * M[a][b])
    return s


def pair_adj(d, al, sg, ub, Jb):
    """(ds/dd, ds/dalpha) as adjoint.cu computes them."""
    from math import erf, exp, pi, sqrt
    R2 = d @ d
    S2 = sg * sg
    RS = R2 / S2 / 2
    sRS = sqrt(RS)
    t2 = 2 / sqrt(pi) * sRS * exp(-RS)
    c4 = 0.25 / pi / R2 / sqrt(R2)
    g = erf(sRS) - t2
    q = g * c4
    h = c4 * (t2 / S2 - 3 * g / R2)
    hR2 = c4 * (-2.5 * t2 / (S2 * R2) - 0.5 * t2 / (S2 * S2) + 7.5 * g / (R2 * R2))
    ct = np.array([Jb[1, 2] - Jb[2, 1], Jb[2, 0] - Jb[0, 2], Jb[0, 1] - Jb[1, 0]])
    m = Jb @ d
    uxd, mxd = np.cross(ub, d), np.cross(m, d)
    A, B, C = al @ uxd, al @ mxd, al @ ct
    wa = -q * uxd - h * mxd - q * ct
    gd = (-h * (A + C) - 2 * hR2 * B) * d - q * np.cross(al, ub) - h * (Jb.T @ np.cross(d, al) + np.cross(al, m))
    return gd, wa


def test_pair_adjoint_against_high_precision_differences():
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(2)
    hh = mp.mpf("1e-15")
    for _ in range(60):
        d = rng.normal(size=3) * rng.uniform(0.02, 1.0)
        al, sg = rng.normal(size=3), rng.uniform(0.02, 0.5)
        ub, Jb = rng.normal(size=3), rng.normal(size=(3, 3))
        gd, wa = pair_adj(d, al, sg, ub, Jb)
        for k in range(3):
            e = [hh if i == k else 0 for i in range(3)]
            fd = (forward_s(mp, [mp.mpf(x) + y for x, y in zip(d, e)], al, sg, ub, Jb)
                  - forward_s(mp, [mp.mpf(x) - y for x, y in zip(d, e)], al, sg, ub, Jb)) / (2 * hh)
            assert abs(float(fd) - gd[k]) <= 1e-9 * np.abs(gd).max()
            fa = (forward_s(mp, d, [mp.mpf(x) + y for x, y in zip(al, e)], sg, ub, Jb)
                  - forward_s(mp, d, [mp.mpf(x) - y for x, y in zip(al, e)], sg, ub, Jb)) / (2 * hh)
            assert abs(float(fa) - wa[k]) <= 1e-9 * np.abs(wa).max()
