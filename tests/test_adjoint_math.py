"""The closed-form adjoint of one near-field pair used by the reverse-mode P2P
(adjoint.cu pair_adj), restated in numpy and checked against 40-digit central
differences of the forward pair terms of the team P2P
(multipoleKernels.hpp:239-283), including the derivative in the source's
radius; and the transpose of the rVPM terms (fmmCalculator.hpp:407-418) of
k_adj_seeds.  CPU only."""
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
    """(ds/dd, ds/dalpha, ds/dsigma) as adjoint.cu computes them."""
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
    sgb = ((3 * q + R2 * h) * (A + C) + (5 * h + 2 * R2 * hR2) * B) / sg
    return gd, wa, sgb


def test_pair_adjoint_against_high_precision_differences():
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(2)
    hh = mp.mpf("1e-15")
    for _ in range(60):
        d = rng.normal(size=3) * rng.uniform(0.02, 1.0)
        al, sg = rng.normal(size=3), rng.uniform(0.02, 0.5)
        ub, Jb = rng.normal(size=3), rng.normal(size=(3, 3))
        gd, wa, sgb = pair_adj(d, al, sg, ub, Jb)
        fs = (forward_s(mp, d, al, mp.mpf(sg) + hh, ub, Jb) - forward_s(mp, d, al, mp.mpf(sg) - hh, ub, Jb)) / (2 * hh)
        assert abs(float(fs) - sgb) <= 1e-9 * max(abs(sgb), np.abs(wa).max())
        for k in range(3):
            e = [hh if i == k else 0 for i in range(3)]
            fd = (forward_s(mp, [mp.mpf(x) + y for x, y in zip(d, e)], al, sg, ub, Jb)
                  - forward_s(mp, [mp.mpf(x) - y for x, y in zip(d, e)], al, sg, ub, Jb)) / (2 * hh)
            assert abs(float(fd) - gd[k]) <= 1e-9 * np.abs(gd).max()
            fa = (forward_s(mp, d, [mp.mpf(x) + y for x, y in zip(al, e)], sg, ub, Jb)
                  - forward_s(mp, d, [mp.mpf(x) - y for x, y in zip(al, e)], sg, ub, Jb)) / (2 * hh)
            assert abs(float(fa) - wa[k]) <= 1e-9 * np.abs(wa).max()


def test_rvpm_terms_transpose():
    """k_adj_seeds' transpose of the rVPM terms: with d the stretching term,
    dalpha/dt = d - 3/5 (d.alpha) alpha/|alpha|^2 and dr/dt = -1/5 r (d.alpha)/|alpha|^2;
    cotangents (ca, cr) of (dalpha/dt, dr/dt) give those of d, alpha and r."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(4)

    def fwd(al, ds, r, ca, cr):
        na = mp.sqrt(sum(x * x for x in al))
        ah = [x / na for x in al]
        dot = sum(x * y for x, y in zip(ds, ah))
        dadt = [x - mp.mpf(3) / 5 * dot * y for x, y in zip(ds, ah)]
        drdt = -mp.mpf(1) / 5 * r / na * dot
        return sum(mp.mpf(c) * x for c, x in zip(ca, dadt)) + mp.mpf(cr) * drdt

    hh = mp.mpf("1e-15")
    for _ in range(40):
        al, ds, ca = rng.normal(size=3), rng.normal(size=3), rng.normal(size=3)
        r, cr = rng.uniform(0.05, 0.5), rng.normal()
        q2, sd, cal = al @ al, ds @ al, ca @ al
        ab = -0.6 * (cal * ds + sd * ca) / q2 + 1.2 * sd * cal * al / q2**2 - 0.2 * r * cr * (ds / q2 - 2 * sd * al / q2**2)
        rb = -0.2 * sd * cr / q2
        cs = ca - (0.6 * cal + 0.2 * r * cr) * al / q2
        A = [mp.mpf(x) for x in al]
        D = [mp.mpf(x) for x in ds]
        R = mp.mpf(r)
        for k in range(3):
            e = [hh if i == k else 0 for i in range(3)]
            fa = (fwd([x + y for x, y in zip(A, e)], D, R, ca, cr) - fwd([x - y for x, y in zip(A, e)], D, R, ca, cr)) / (2 * hh)
            fd = (fwd(A, [x + y for x, y in zip(D, e)], R, ca, cr) - fwd(A, [x - y for x, y in zip(D, e)], R, ca, cr)) / (2 * hh)
            assert abs(float(fa) - ab[k]) <= 1e-10 * (1 + np.abs(ab).max())
            assert abs(float(fd) - cs[k]) <= 1e-10 * (1 + np.abs(cs).max())
        fr = (fwd(A, D, R + hh, ca, cr) - fwd(A, D, R - hh, ca, cr)) / (2 * hh)
        assert abs(float(fr) - rb) <= 1e-10 * (1 + abs(rb))
