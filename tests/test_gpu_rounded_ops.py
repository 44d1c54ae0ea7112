"""The exact arithmetic's branch-free correctly rounded operations
(csrc/em_math.cuh: sqrt_rn_nb, rcp_rn_nb, div_rn_nb — Markstein's
FMA-residual corrections) against the compiler's rounded operations, bit for
bit, over the operand ranges the exact tracer admits (other operands take
the rounded operations): every root operand, every divisor, and 4e9 seeded
random quotients.  The exact tracer's bit-for-bit agreement with the
reference (test_gpu_parity.py) rests on these."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_rounded_ops_match_bit_for_bit(gpu):
    bad = (ctypes.c_ulonglong * 3)()
    rc = gpu.em_selftest_rounded_ops(4_000_000_000, bad)
    assert rc == 0
    assert list(bad) == [0, 0, 0], list(bad)


def test_rounded_ops_argument_check(gpu):
    assert gpu.em_selftest_rounded_ops(0, None) != 0
