"""Fit of the scaled complementary error function used by the mixed-precision
P2P kernel (mixed.cu, p2p_weights2).

For rho >= 0.5 the kernel writes the regularised kernel's
g(rho) = erf(rho) - (2/sqrt(pi)) rho e^(-rho^2) as
    g = 1 - e^(-rho^2) (erfcx(rho) + (2/sqrt(pi)) rho),
reusing the e^(-rho^2) it needs anyway, with
    erfcx(rho) ~ t (c1 + c2 t + c3 t^2 + c4 t^3 + c5 t^4),  t = 1 / (1 + a rho).
The coefficients come from a weighted least-squares fit (iteratively
reweighted toward the minimax solution) of erfcx on rho in [0.5, 14], weighted
by e^(-rho^2) / g(rho), so that the fit error is measured as relative error of g;
the scale a is the best of a scan.  Run this file to regenerate the constants
(numpy and scipy); it prints them in the form the kernel uses.
"""
import numpy as np
from scipy.special import erf, erfcx

DEGREE = 5


def fit(degree: int = DEGREE):
    rho = np.concatenate([np.linspace(0.5, 2, 4000), np.linspace(2, 6, 4000), np.linspace(6, 14, 1000)])
    ex = np.exp(-rho ** 2)
    g = erf(rho) - 2 / np.sqrt(np.pi) * rho * ex
    f = erfcx(rho)
    w = ex / g
    best = None
    for a in np.linspace(0.2, 1.2, 101):
        t = 1 / (1 + a * rho)
        A = np.stack([t ** k for k in range(1, degree + 1)], 1)
        ww = w.copy()
        for _ in range(40):
            c, *_ = np.linalg.lstsq(A * ww[:, None], f * ww, rcond=None)
            e = (A @ c - f) * w
            ww = w * (np.abs(e) / np.abs(e).max()) ** 0.5 + 1e-30
        err = np.abs((A @ c - f) * w).max()
        if best is None or err < best[0]:
            best = (err, a, c, A, f, w, ww)
    # FP32 constants: round one coefficient at a time and refit the others
    _, a, c, A, f, w, ww = best
    a = float(np.float32(a))
    t = 1 / (1 + a * rho)
    A = np.stack([t ** k for k in range(1, degree + 1)], 1)
    fixed = []
    for k in range(degree):
        r = f - (A[:, :k] @ np.array(fixed) if fixed else 0.0)
        ck, *_ = np.linalg.lstsq(A[:, k:] * ww[:, None], r * ww, rcond=None)
        fixed.append(float(np.float32(ck[0])))
    c = np.array(fixed)
    err = np.abs((A @ c - f) * w).max()
    return err, a, [float(x) for x in c]


if __name__ == "__main__":
    err, a, c = fit()
    print(f"max relative error of g from the fit with FP32 constants (FP64 arithmetic): {err:.3e}")
    print(f"constexpr float kErfcxA = {float(np.float32(a))!r}f;")
    for k, ck in enumerate(c, 1):
        print(f"constexpr float kErfcx{k} = {float(np.float32(ck))!r}f;")
