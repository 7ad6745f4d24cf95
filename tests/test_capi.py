"""C ABI boundary without a GPU: the library loads, exports every function
include/*.h declares, and reports errors as status codes."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from openpstd_gb300 import _lib, scenes
from openpstd_gb300 import kernel as K
from openpstd_gb300.config import CConfig

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(pstd_[a-z0-9_]+)\s*\(", src):
            if not re.search(r"\(\s*\*\s*" + m.group(1), src):
                names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("pstd_create", "pstd_run", "pstd_get_metadata", "pstd_destroy", "pstd_advance"):
        assert must in names


def test_library_exports_every_declared_symbol(pstd_lib):
    missing = [n for n in declared_functions() if not hasattr(pstd_lib, n)]
    assert not missing, missing


def test_binding_covers_header(pstd_lib):
    # the Python binding declares a signature for every exported entry point
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_status_codes_without_configuration(pstd_lib):
    L = pstd_lib
    assert L.pstd_run(None, None) == _lib.PSTD_ERR_NOT_CONFIGURED
    assert L.pstd_advance(None, 1, None) == _lib.PSTD_ERR_NOT_CONFIGURED
    assert b"not configured" in L.pstd_last_error()
    L.pstd_destroy(None)   # safe on NULL
    n = ctypes.c_int32()
    assert L.pstd_get_metadata(None, ctypes.byref(n), None, 0, None) == _lib.PSTD_ERR_NOT_CONFIGURED


def test_host_only_scene_refuses_device_calls(pstd_lib):
    cc = CConfig(scenes.plain_square(0, n=60, steps=5, pml=40))
    h = ctypes.c_void_p()
    _lib.check(pstd_lib.pstd_scene_build(ctypes.byref(cc.c), ctypes.byref(h)))
    try:
        assert pstd_lib.pstd_advance(h, 1, None) == _lib.PSTD_ERR_NOT_CONFIGURED
        n, fc = ctypes.c_int32(), ctypes.c_int32()
        dims = (ctypes.c_int32 * 30)()
        _lib.check(pstd_lib.pstd_get_metadata(h, ctypes.byref(n), dims, 10, ctypes.byref(fc)))
        assert n.value == 9 and fc.value == 5
        assert (dims[0], dims[1], dims[2]) == (60, 60, 0)
        runs = (ctypes.c_int32 * 64)()
        _lib.check(pstd_lib.pstd_scene_strip_runs(h, 0, 0, runs, 16, ctypes.byref(n)))
        assert n.value == 1 and runs[0] == 0 and runs[1] == 60   # one run: left/right PML
    finally:
        pstd_lib.pstd_destroy(h)


def test_invalid_configuration_is_a_status(pstd_lib):
    conf = scenes.plain_square(0, n=60, steps=5, pml=40)
    conf.Settings.SetGridSpacing(0.0)
    cc = CConfig(conf)
    h = ctypes.c_void_p()
    assert pstd_lib.pstd_scene_build(ctypes.byref(cc.c), ctypes.byref(h)) == _lib.PSTD_ERR_INVALID
    conf = scenes.plain_square(0, n=60, steps=5, pml=40)
    conf.Settings.SetRKCoefficients([0.5, 1.0])
    cc = CConfig(conf)
    assert pstd_lib.pstd_scene_build(ctypes.byref(cc.c), ctypes.byref(h)) == _lib.PSTD_ERR_INVALID


def test_kernel_interface_semantics():
    k = K.PSTDKernel()
    with pytest.raises(K.PSTDKernelNotConfiguredException):
        k.get_metadata()
    with pytest.raises(K.PSTDKernelNotConfiguredException):
        k.run(K.KernelCallback())
    with pytest.raises(ValueError):
        K.PSTDKernel(GPU=False)


def test_configuration_mirror():
    from openpstd_gb300.config import PSTDConfiguration, f32
    c = PSTDConfiguration.CreateDefaultConf()
    s = c.Settings
    assert s.GetWindowSize() == 32
    assert s.GetTimeStep() == f32(f32(f32(0.5) * f32(0.2)) / f32(340))
    assert s.GetBandWidth() == f32(3e-6 * 1700.0 * 1700.0) or abs(float(s.GetBandWidth()) - 8.67) < 1e-3
    assert len(c.Domains) == 2 and c.Domains[0].L.Absorption == pytest.approx(0.3)
    conf = scenes.plain_square(0)
    assert conf.Settings.framecount() == 500
    assert scenes.l_shape(0).Settings.framecount() == 4000


def test_stage_variant_list(pstd_lib):
    """pstd_stage_variants: the compiled variants of a length as "<index> <name>"
    lines (the indices PSTD_PLAN pins); host only."""
    import ctypes
    buf, n = ctypes.create_string_buffer(1 << 14), ctypes.c_int32()
    assert pstd_lib.pstd_stage_variants(128, buf, 1 << 14, ctypes.byref(n)) == 0
    lines = buf.value.decode().splitlines()
    assert n.value == len(lines) > 0
    for i, line in enumerate(lines):
        idx, name = line.split(" ", 1)
        assert int(idx) == i and name.startswith("L128 ")
    assert pstd_lib.pstd_stage_variants(100, buf, 1 << 14, ctypes.byref(n)) == 0 and n.value == 0


@pytest.mark.parametrize("L,radices,ctw,lane_pair", [
    (128, (16, 8), 0, 0), (128, (16, 8), 1, 0), (512, (8, 8, 8), 1, 0), (1024, (32, 32), 0, 0),
    (1024, (16, 8, 8), 0, 0), (256, (8, 32), 0, 1), (512, (16, 32), 1, 1)])
def test_transform_gain_model(pstd_lib, L, radices, ctw, lane_pair):
    """The per-bin round-trip gain the derivative filters are divided by
    (first order in the float constants' rounding) against an exact emulation
    of the transform's passes: equal to 1e-12; and the uncompensated gain is
    biased (every plan loses amplitude on average)."""
    import ctypes
    import numpy as np
    from transform_model import round_trip_gain
    r = (ctypes.c_int32 * 4)(*radices)
    out = np.zeros(2 * L)
    assert pstd_lib.pstd_transform_gain(L, r, len(radices), ctw, lane_pair,
                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
    model = out[0::2] + 1j * out[1::2]
    exact = round_trip_gain(L, radices, bool(ctw), bool(lane_pair))
    assert np.abs(model - exact).max() < 1e-12, np.abs(model - exact).max()
    assert (model - 1).real.mean() < -2e-8
