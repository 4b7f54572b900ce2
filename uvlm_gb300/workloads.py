"""Seeded synthetic particle sets of the benchmark shapes (no dataset involved).

* ring: a thin vortex ring of radius R, core radius a, circulation Gamma;
  `stations` azimuthal stations x a 127-point cross-section (7 layers with
  1, 6, 12, ..., 36 points at radii k*a/6).  Each point's weight is its
  layer's annulus-area share divided by the layer's point count (the centre
  point covers a disc of radius a/12; shares sum to 1).  Strength
  alpha = Gamma * ds * weight * tangent with ds = 2 pi R / stations; smoothing
  radius sigma = 1.3 * ds; positions jittered by 1e-4 * ds from the seed.
* cloud: positions uniform in [-1, 1]^3, alpha components normal with
  standard deviation 1e-3, sigma = 1.3 * 2 * N^(-1/3).
* leapfrog: two coaxial rings at z = 0 and z = 0.5.
"""
from __future__ import annotations

import numpy as np

from ._lib import BODY_DTYPE

LAYERS = (1, 6, 12, 18, 24, 30, 36)


def _cross_section(a: float):
    """Offsets (rho, psi) and area weights of the 127-point core cross-section."""
    pts, w = [], []
    for k, cnt in enumerate(LAYERS):
        if k == 0:
            share = (1.0 / 12.0) ** 2
        elif k < 6:
            share = ((k + 0.5) / 6.0) ** 2 - ((k - 0.5) / 6.0) ** 2
        else:
            share = 1.0 - (5.5 / 6.0) ** 2
        for j in range(cnt):
            pts.append((k * a / 6.0, 2.0 * np.pi * j / cnt))
            w.append(share / cnt)
    return np.array(pts), np.array(w)


def ring(stations: int = 256, R: float = 1.0, a: float = 0.1, gamma: float = 1.0, seed: int = 0,
         center=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0)) -> np.ndarray:
    rng = np.random.default_rng(seed)
    cs, w = _cross_section(a)
    ds = 2.0 * np.pi * R / stations
    phi = 2.0 * np.pi * np.arange(stations) / stations
    P = len(w)
    n = stations * P
    rho = np.tile(cs[:, 0], stations)
    psi = np.tile(cs[:, 1], stations)
    ph = np.repeat(phi, P)
    ww = np.tile(w, stations)
    rhat = np.stack([np.cos(ph), np.sin(ph), np.zeros(n)], 1)
    zhat = np.array([0.0, 0.0, 1.0])
    that = np.stack([-np.sin(ph), np.cos(ph), np.zeros(n)], 1)
    X = (R + rho * np.cos(psi))[:, None] * rhat + (rho * np.sin(psi))[:, None] * zhat
    X += rng.normal(0.0, 1e-4 * ds, X.shape)
    A = (gamma * ds * ww)[:, None] * that
    axis = np.asarray(axis, float)
    axis /= np.linalg.norm(axis)
    if not np.allclose(axis, zhat):
        v = np.cross(zhat, axis)
        c = float(np.dot(zhat, axis))
        vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
        Rm = np.eye(3) + vx + vx @ vx / (1.0 + c)
        X = X @ Rm.T
        A = A @ Rm.T
    b = np.zeros(n, BODY_DTYPE)
    b["X"] = X + np.asarray(center)
    b["alpha"] = A
    b["radius"] = 1.3 * ds
    return b


def cloud(n: int, seed: int = 0, alpha_std: float = 1e-3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    b = np.zeros(n, BODY_DTYPE)
    b["X"] = rng.uniform(-1.0, 1.0, (n, 3))
    b["alpha"] = rng.normal(0.0, alpha_std, (n, 3))
    b["radius"] = 1.3 * 2.0 * n ** (-1.0 / 3.0)
    return b


def leapfrog(stations: int = 512, seed: int = 0) -> np.ndarray:
    r1 = ring(stations, seed=seed, center=(0.0, 0.0, 0.0))
    r2 = ring(stations, seed=seed + 1, center=(0.0, 0.0, 0.5))
    return np.concatenate([r1, r2])


def ring_batch(count: int = 64, seed: int = 0, n_min: int = 2000, n_max: int = 60000) -> list[np.ndarray]:
    """Independent vortex rings for batched runs: N log-uniform in [n_min, n_max]
    (rounded to whole 127-point stations), R ~ U[0.5, 2], a/R ~ U[0.05, 0.15],
    Gamma ~ U[0.5, 2], random orientation and centre."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        stations = max(8, int(round(n / 127)))
        R = rng.uniform(0.5, 2.0)
        axis = rng.normal(size=3)
        out.append(ring(stations, R=R, a=R * rng.uniform(0.05, 0.15), gamma=rng.uniform(0.5, 2.0), seed=seed * 1000 + k,
                        center=tuple(rng.uniform(-1, 1, 3)), axis=tuple(axis / np.linalg.norm(axis))))
    return out


class WingWake:
    """Wing + wake: a flat rectangular wing of aspect ratio `aspect` (chord c,
    span b = aspect * c), `nspan` x `nchord` vortex-lattice panels, pitched by
    `alpha_deg` about the spanwise (y) axis, moving through still fluid with
    velocity -U (U = (|U|, 0, 0)) like the reference driver's wing
    (src/main.cpp:183), and shedding wake particles at its trailing edge every
    step after the reference driver (src/main.cpp:246-289):

    * each trailing-edge (TE) panel p sheds at the TE midpoint plus U dt a
      particle carrying half the circulation differences to its neighbours
      on the panel's side lines, and the full Gamma on the side line at a wing
      tip (the trailing vorticity);
    * its spanwise part is the TE vortex line times the change of the panel's
      circulation since the last step (rule="unsteady", the default: with a
      steady prescribed Gamma only the first step sheds it, the starting
      vortex), or times Gamma_p itself every step (rule="reference", the
      driver's line 255-257: at 400 particles per step the resulting vortex
      sheet went unstable within 60 steps in FP64 as in mixed precision,
      speeds above 500 |U| and then coinciding particles, so it is kept only
      as an option);
    * here each TE panel is cut into `subdiv` equal spanwise segments that
      shed one particle each (the reference sheds one per panel: 40 x 400 =
      16k particles after 400 steps; subdivided, 400 per step reach ~160k);
    * the bound circulation is prescribed, an elliptic lifting-line
      distribution Gamma(y) = Gamma0 sqrt(1 - (2y/b)^2) with Gamma0 =
      2 C_L |U| c / pi and C_L = 2 pi alpha / (1 + 2 / aspect) (the
      reference solves its vortex lattice with Eigen instead; that solver is
      not part of the accelerated path);
    * radius sigma = 1.3 x the shedding spacing b / (nspan subdiv) (the
      reference uses 2.5 x the TE panel width).

    Ring orientation of a TE panel: its leading line runs along +y (bound
    vorticity +Gamma y for lift +z), the trailing line along -y, the right
    side line (larger y) along +x and the left one along -x, all in the
    pitched wing plane."""

    def __init__(self, aspect: float = 8.0, chord: float = 1.0, nspan: int = 40, nchord: int = 10, alpha_deg: float = 5.0,
                 U: float = 1.0, dt: float = 0.02, subdiv: int = 10, rule: str = "unsteady"):
        if rule not in ("unsteady", "reference"):
            raise ValueError("rule must be 'unsteady' or 'reference'")
        self.rule = rule
        a = np.deg2rad(alpha_deg)
        self.c, self.b, self.U, self.dt = chord, aspect * chord, U, dt
        self.ex = np.array([np.cos(a), 0.0, -np.sin(a)])  # chordwise unit vector in the pitched plane
        cl = 2.0 * np.pi * a / (1.0 + 2.0 / aspect)
        self.gamma0 = 2.0 * cl * U * chord / np.pi
        ns = nspan * subdiv
        self.ns = ns
        edges = np.linspace(-self.b / 2, self.b / 2, ns + 1)
        self.y0, self.y1 = edges[:-1], edges[1:]
        ym = 0.5 * (self.y0 + self.y1)
        self.gamma = self.gamma0 * np.sqrt(np.clip(1.0 - (2.0 * ym / self.b) ** 2, 0.0, None))
        self.side = (chord / nchord) * self.ex  # side vortex line of a TE panel (along the chord)
        self.sigma = 1.3 * (self.b / ns)
        self.step_index = 0

    def shed(self) -> np.ndarray:
        """The particles shed at the current step (the wing then moves on)."""
        k = self.step_index
        te_x = self.c * self.ex - np.array([self.U * self.dt * k, 0.0, 0.0])  # TE point at y = 0, wing moved by -U t
        g = self.gamma
        n = self.ns
        b = np.zeros(n, BODY_DTYPE)
        X = np.zeros((n, 3))
        X[:, 0] = te_x[0] + self.U * self.dt
        X[:, 1] = 0.5 * (self.y0 + self.y1)
        X[:, 2] = te_x[2]
        te_line = np.zeros((n, 3))
        te_line[:, 1] = -(self.y1 - self.y0)  # trailing line along -y
        shed = g if (self.rule == "reference" or k == 0) else np.zeros_like(g)  # circulation change (steady after the start)
        A = te_line * shed[:, None]
        # side lines: left along -x (shared with the left neighbour), right along +x
        gl = np.concatenate([[0.0], g[:-1]])
        gr = np.concatenate([g[1:], [0.0]])
        wl = np.where(np.arange(n) == 0, 1.0, 0.5)
        wr = np.where(np.arange(n) == n - 1, 1.0, 0.5)
        A += (-self.side)[None, :] * ((g - np.where(np.arange(n) == 0, 0.0, gl)) * wl)[:, None]
        A += self.side[None, :] * ((g - np.where(np.arange(n) == n - 1, 0.0, gr)) * wr)[:, None]
        b["X"] = X
        b["alpha"] = A
        b["radius"] = self.sigma
        self.step_index += 1
        return b
