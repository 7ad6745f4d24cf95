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


def test_frame_buffers_recycled_only_when_no_view_lives():
    """Large frames are copied into recycled buffers: a buffer returns to the
    pool only when the callee holds no view of the frame (views of views
    included), and a new frame never shares memory with a live one."""
    import gc
    from openpstd_gb300 import kernel
    src = np.arange(1 << 20, dtype=np.float32)
    ptr = src.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    kernel._free_frames.pop(src.size, None)
    a = kernel._copy_frame(ptr, src.size)
    assert np.array_equal(a, src) and a.dtype == np.float32 and a.flags.writeable
    kept = a.reshape(1024, 1024)[::2]
    del a
    gc.collect()
    assert not kernel._free_frames.get(src.size)
    b = kernel._copy_frame(ptr, src.size)
    assert not np.shares_memory(b, kept)
    del kept, b
    gc.collect()
    assert len(kernel._free_frames[src.size]) == 2
    c = kernel._copy_frame(ptr, src.size)
    assert np.array_equal(c, src) and len(kernel._free_frames[src.size]) == 1
