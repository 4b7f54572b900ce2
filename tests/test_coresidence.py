"""The split leaf kernel runs its near-field pass on a second stream beside the
tensor-core M2L, one near-pass block next to the M2L block on every SM.  That
holds only while the two kernels' registers fit one SM's 65,536 together:
the build's ptxas reports give both kernels' registers, and neither may spill.
(Shared memory: 160.8 KB for the M2L block and 38.3 KB for the near-pass block
at p = 10, set by the kernels' constants, within the 227 KB an SM offers.)"""
import os
import re

import pytest

from uvlm_gb300 import _build

SM_REGISTERS = 65536
M2L_THREADS, NEAR_THREADS = 384, 128


def report(name: str) -> str:
    path = _build.ptxas_report(name)
    if not os.path.exists(path):
        _build.build()
    with open(path) as f:
        return f.read()


def usage(text: str, entry: str) -> tuple[int, int]:
    """(registers per thread, spilled bytes) of one kernel in a ptxas report."""
    i = text.index(f"Compiling entry function '{entry}'")
    block = text[i:i + 800]
    regs = int(re.search(r"Used (\d+) registers", block).group(1))
    st, ld = map(int, re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", block).groups())
    return regs, st + ld


def allocated(regs: int) -> int:
    return (regs + 7) // 8 * 8  # registers are allocated per thread in steps of 8


@pytest.mark.parametrize("P", [8, 9, 10])
@pytest.mark.parametrize("chunk", [768])
def test_m2l_and_near_pass_share_an_sm(P, chunk):
    m2l = usage(report("m2l_tensor"), f"_ZN4vfmm8k_m2l_tcILi{P}EEEvNS_6TcArgsE")
    near = usage(report("mixed"), f"_ZN4vfmm11k_l2p_p2p32ILi{P}ELi{chunk}ELi1EEEvNS_8DevMixedEPd")
    assert M2L_THREADS * allocated(m2l[0]) + NEAR_THREADS * allocated(near[0]) <= SM_REGISTERS, (m2l, near)
    assert m2l[1] == 0 and near[1] == 0, (m2l, near)
