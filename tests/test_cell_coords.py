"""The fast cell-coordinate split used by the move kernels: the quotient by
an FP32 reciprocal with one remainder correction equals integer division
for every cell index below 2^24 and every grid shape (checked exhaustively
on the CPU over a restatement of the same arithmetic in numpy's float32)."""
import numpy as np
import pytest


def udiv24(c, d):
    rcp = np.float32(1.0) / np.float32(d)
    q = np.trunc(c.astype(np.float32) * rcp).astype(np.int64)
    r = c - q * d
    q = np.where(r < 0, q - 1, np.where(r >= d, q + 1, q))
    return q


@pytest.mark.parametrize("d", [1, 2, 3, 7, 10, 30, 64, 100, 127, 128, 255, 256, 1000, 4096, 16384, 32768,
                               65535, 100003, 1 << 20, (1 << 24) - 1])
def test_fp32_reciprocal_quotient_is_exact_below_2_24(d):
    c = np.arange(0, 1 << 24, dtype=np.int64)
    np.testing.assert_array_equal(udiv24(c, d), c // d)
