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
