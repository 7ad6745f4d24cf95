"""The Python bridge's frame copy: the callee owns an exact copy of the
library's staging buffer, whatever the frame size (chunked copies for large
frames, one copy for small ones)."""
import ctypes

import numpy as np
import pytest


@pytest.mark.parametrize("n", [0, 1, 1000, (1 << 19) - 1, (1 << 19) + 7, 3_000_001])
def test_copy_frame_exact_and_owned(n):
    from openpstd_gb300.kernel import _copy_frame
    src = np.random.default_rng(n).standard_normal(max(n, 1)).astype(np.float32)
    ptr = src.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    got = _copy_frame(ptr, n)
    assert got.dtype == np.float32 and got.shape == (n,)
    assert np.array_equal(got, src[:n])
    src[:] = 0                                   # the staging buffer is reused
    if n:
        assert not np.shares_memory(got, src) and np.any(got != 0)
