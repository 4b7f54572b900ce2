"""Tensor-core primitives (tcgen05 on sm_100-family GPUs): the operand layouts
that the mixed-precision M2L kernel builds on, checked element by element on
small integers (exact in TF32 and FP32)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def expected(swap: bool) -> np.ndarray:
    """D = A B with A[m][k] = (3m + 5k) % 11 - 5 and B[k][n] = (7k + 3n) % 13 - 6,
    B read through the descriptor: stored with core matrices adjacent in K 256
    bytes apart and adjacent in N 128 bytes apart; with swap the descriptor
    gives the two offsets the other way round, so element (k, n) is read from
    where another element was stored."""
    m = np.arange(128)[:, None]
    k = np.arange(8)[None, :]
    A = ((3 * m + 5 * k) % 11 - 5).astype(np.float64)
    Bst = np.zeros(128, np.float64)  # the 512-byte buffer as 128 floats
    for n in range(16):
        for kk in range(8):
            Bst[((kk // 4) * 256 + (n // 8) * 128 + (n % 8) * 16 + (kk % 4) * 4) // 4] = (7 * kk + 3 * n) % 13 - 6
    lbo, sbo = (128, 256) if swap else (256, 128)
    B = np.zeros((8, 16))
    for n in range(16):
        for kk in range(8):
            B[kk, n] = Bst[((kk // 4) * lbo + (n // 8) * sbo + (n % 8) * 16 + (kk % 4) * 4) // 4]
    return A @ B


def test_tcgen05_tf32_mma_layouts(vfmm_lib):
    out = np.zeros((128, 16), np.float32)
    rc = vfmm_lib.vfmm_tcgen05_selftest(0, 0, out.ctypes.data)
    assert rc == 0, rc
    ok0 = np.array_equal(out, expected(False))
    out1 = np.zeros((128, 16), np.float32)
    assert vfmm_lib.vfmm_tcgen05_selftest(0, 1, out1.ctypes.data) == 0
    ok1 = np.array_equal(out1, expected(True))
    print("layout as documented:", ok0, " offsets swapped:", ok1)
    if not ok0:
        print(out[:4], expected(False)[:4], out1[:4], sep="\n")
    assert ok0 and ok1


def test_tcgen05_m64_lane_map(vfmm_lib):
    """An M = 64 MMA with A in tensor memory: which TMEM lanes it reads A
    rows from and writes D rows to.  D[lane][0] = (a + 1) B[0][0] with
    B[0][0] = -6 names the A lane a that fed lane `lane` (0: untouched).  The
    M2L kernel keeps the rows that need high K columns in exactly these lanes
    and runs its high-K steps at M = 64."""
    out = np.zeros((128, 16), np.float32)
    assert vfmm_lib.vfmm_tcgen05_selftest(0, 2, out.ctypes.data) == 0
    src = np.rint(-out[:, 0] / 6.0).astype(int) - 1  # -1: lane untouched
    written = np.flatnonzero(src >= 0)
    print("M=64 lanes written:", written.tolist())
    print("fed from A lanes:", src[written].tolist())
    assert len(written) == 64
    assert (src[written] == written).all()  # each D row comes from the A row of the same lane
    expect = np.array([q * 32 + i for q in range(4) for i in range(16)])
    assert (written == expect).all(), written
