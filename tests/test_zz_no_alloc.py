"""pstd_solve_noalloc (the allocation-free solve) against the existing entry
points pstd_create + pstd_advance + pstd_snapshot / pstd_get_receivers.

The entry point keeps its state sets and tables in one static device array
that every call shares, so the GPU test makes two calls in a row (and then
alternates two scenes of different layouts) and checks every call against
the existing path, at the relative-L2 tolerance of the other GPU parity
tests.  This file is collected last on purpose: it must pass in a fresh
process and after every other test of the suite.
"""
import ctypes

import numpy as np
import pytest

from parity import rel

TOL = 1e-5          # relative L2, as the GPU parity tests


def _configs():
    from openpstd_gb300 import scenes
    a = scenes.plain_square(seed=3, n=64 + 9, steps=12, pml=40)
    b = scenes.batch_scenes(seed=7, n=1, steps=12, max_cells=(256, 192))[0]
    return a, b


def _existing(conf, steps):
    """Frame (p0 of the non-PML domains, scene order) and receiver samples
    after `steps` steps through pstd_create + pstd_advance, with the variant
    the allocation-free solve runs (each length's first one; PSTD_VARIANT=0):
    variants differ in rounding, and each divides its filter by its own
    transform's gain."""
    import os
    from openpstd_gb300.kernel import PSTDKernel
    keep = os.environ.get("PSTD_VARIANT")
    os.environ["PSTD_VARIANT"] = "0"
    try:
        k = PSTDKernel()
        k.initialize_kernel(conf)
    finally:
        if keep is None:
            del os.environ["PSTD_VARIANT"]
        else:
            os.environ["PSTD_VARIANT"] = keep
    k.advance(steps)
    k.synchronize()
    frame = [k.snapshot(i, "p0").ravel() for i in range(k.domain_count()) if not k.domain_info(i)["is_pml"]]
    rec = k.receivers()
    k.close()
    return np.concatenate(frame), rec


def _noalloc(conf, steps, n_frame, n_rec):
    """One pstd_solve_noalloc call through the C ABI; outputs are device
    buffers owned by the caller (here torch tensors), pre-filled with NaN."""
    import torch
    from openpstd_gb300 import _lib
    from openpstd_gb300.config import CConfig
    cc = CConfig(conf)
    frame = torch.full((n_frame,), float("nan"), dtype=torch.float32, device="cuda")
    rec = torch.full((max(steps * n_rec, 1),), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = _lib.lib().pstd_solve_noalloc(ctypes.byref(cc.c), steps, ctypes.c_void_p(frame.data_ptr()), frame.numel(),
                                       ctypes.c_void_p(rec.data_ptr()), steps * n_rec, None)
    _lib.check(rc)
    torch.cuda.synchronize()
    return frame.cpu().numpy(), rec[: steps * n_rec].cpu().numpy().reshape(steps, n_rec)


def _compare(conf, steps, want):
    wf, wr = want
    gf, gr = _noalloc(conf, steps, wf.size, wr.shape[1])
    assert np.isfinite(gf).all() and np.isfinite(gr).all()
    assert rel(gf, wf) <= TOL, rel(gf, wf)
    assert rel(gr, wr) <= TOL, rel(gr, wr)


@pytest.mark.gpu
def test_noalloc_matches_existing_two_calls():
    a, _ = _configs()
    steps = 12
    want = _existing(a, steps)
    for _ in range(2):                       # two calls in a row share the scratch array
        _compare(a, steps, want)


@pytest.mark.gpu
def test_noalloc_leaves_device_memory_unchanged():
    """After a warm-up call (which loads the kernels' modules), a further call
    takes no device memory: the free bytes the driver reports are the same
    before and after it, with the outputs allocated beforehand."""
    import torch
    from openpstd_gb300 import _lib
    from openpstd_gb300.config import CConfig
    a, _ = _configs()
    steps = 12
    want = _existing(a, steps)
    _compare(a, steps, want)                 # warm-up: modules loaded
    cc = CConfig(a)
    frame = torch.empty(want[0].size, dtype=torch.float32, device="cuda")
    rec = torch.empty(steps * want[1].shape[1], dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc = _lib.lib().pstd_solve_noalloc(ctypes.byref(cc.c), steps, ctypes.c_void_p(frame.data_ptr()), frame.numel(),
                                       ctypes.c_void_p(rec.data_ptr()), rec.numel(), None)
    _lib.check(rc)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert rel(frame.cpu().numpy(), want[0]) <= TOL


@pytest.mark.gpu
def test_noalloc_alternating_layouts():
    a, b = _configs()
    wa, wb = _existing(a, 10), _existing(b, 7)
    for conf, steps, want in ((b, 7, wb), (a, 10, wa), (b, 7, wb)):
        _compare(conf, steps, want)


def test_noalloc_rejects_scene_beyond_scratch(pstd_lib):
    """A scene whose state does not fit PSTD_NOALLOC_SCRATCH_BYTES is refused
    with PSTD_ERR_INVALID before any device work (no GPU needed)."""
    from openpstd_gb300 import _lib, scenes
    from openpstd_gb300.config import CConfig
    cc = CConfig(scenes.l_shape(0, steps=4))
    rc = _lib.lib().pstd_solve_noalloc(ctypes.byref(cc.c), 4, None, 0, None, 0, None)
    assert rc == _lib.PSTD_ERR_INVALID
    msg = _lib.lib().pstd_last_error().decode()
    assert "bytes of scratch" in msg and str(16 << 20) in msg


def test_noalloc_rejects_bad_arguments(pstd_lib):
    from openpstd_gb300 import _lib
    from openpstd_gb300.config import CConfig
    a, _ = _configs()
    cc = CConfig(a)
    L = _lib.lib()
    assert L.pstd_solve_noalloc(None, 4, None, 0, None, 0, None) == _lib.PSTD_ERR_INVALID
    assert L.pstd_solve_noalloc(ctypes.byref(cc.c), 0, None, 0, None, 0, None) == _lib.PSTD_ERR_INVALID
    assert L.pstd_solve_noalloc(ctypes.byref(cc.c), 4, None, 16, None, 0, None) == _lib.PSTD_ERR_INVALID
    # an output shorter than the scene's frame is refused before device work
    assert L.pstd_solve_noalloc(ctypes.byref(cc.c), 4, ctypes.c_void_p(256), 3, None, 0, None) == _lib.PSTD_ERR_INVALID
    assert "frame output holds 3 floats" in L.pstd_last_error().decode()
