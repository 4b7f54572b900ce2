"""The fields of the caller's records that an advance reads.

vfmm_advance loads only the fields a step reads from the caller's
exafmm::Body records (uvlm_gb300/csrc/api.cu `advance_input_fields`): the
evaluation of the first stage stores velocity, J, dadt and dr/dt before
anything reads them, and the first stage update stores the RK registers
(all six for RK2 and RK4, which call storeInitialState; the velocity, dadt and
dr/dt registers for RK3).  Here that claim is checked on the CPU against the
oracle restatement of the reference's advance (fmmCalculator.hpp:919-1005)
and, where its sources are present, the reference itself: changing the
fields left out must change no field of the records after the step."""
import numpy as np
import pytest

from oracle import oracle as O
from uvlm_gb300 import BODY_DTYPE, workloads

SCHEMES = {0: "Euler", 1: "RK2", 2: "RK3", 3: "RK4"}


def dropped(scheme: int) -> list[str]:
    """The fields an advance with `scheme` does not read (advance_input_fields)."""
    d = ["J", "velocity", "dadt", "drdt"]
    if scheme in (1, 2, 3):
        d += ["velocity_old", "dadt_old", "drdt_old"]
    if scheme in (1, 3):
        d += ["X_old", "alpha_old", "radius_old"]
    return d


def with_fields(b: np.ndarray, names: list[str], seed: int) -> np.ndarray:
    out = b.copy()
    rng = np.random.default_rng(seed)
    for f in names:
        out[f] = rng.standard_normal(out[f].shape)
    return out


def start(n: int = 600) -> np.ndarray:
    b = workloads.cloud(n, seed=13)
    return with_fields(b, [f for f in BODY_DTYPE.names if f not in ("X", "alpha", "radius")], 1)


def assert_same(a: np.ndarray, b: np.ndarray):
    for f in BODY_DTYPE.names:
        assert (a[f] == b[f]).all(), f


@pytest.mark.parametrize("scheme", list(SCHEMES))
@pytest.mark.parametrize("formulation,viscous", [(0, 0), (1, 0), (0, 1), (0, 2)])
def test_oracle_advance_ignores_the_fields_left_out(scheme, formulation, viscous):
    b = start()
    nu = 1e-3 if viscous else 0.0
    outs = [O.advance(with_fields(b, dropped(scheme), seed), 6, 16, 0.5, 0.01, 2, scheme, formulation=formulation,
                      viscous=viscous, nu=nu) for seed in (2, 3)]
    assert_same(*outs)
    for f in BODY_DTYPE.names:
        assert np.isfinite(outs[0][f]).all(), f


def test_oracle_advance_reads_the_fields_kept():
    """The other direction, for RK3 and Euler: the registers they keep pass
    through to the output, so changing them changes the records."""
    b = start()
    for scheme, kept in [(2, "X_old"), (0, "velocity_old")]:
        x = O.advance(with_fields(b, [kept], 4), 6, 16, 0.5, 0.01, 1, scheme)
        y = O.advance(with_fields(b, [kept], 5), 6, 16, 0.5, 0.01, 1, scheme)
        assert not (x[kept] == y[kept]).all(), (SCHEMES[scheme], kept)


@pytest.mark.skipif(not O.ref_available(), reason="the reference's sources are not present")
@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_reference_advance_ignores_the_fields_left_out(scheme):
    R = O.ref(6, 16, 0.5)
    b = start()
    outs = []
    for seed in (2, 3):
        x = with_fields(b, dropped(scheme), seed)
        assert R.ref_advance(x.ctypes.data, x.size, 0.01, 2, scheme, 0) == 0
        outs.append(x)
    assert_same(*outs)
