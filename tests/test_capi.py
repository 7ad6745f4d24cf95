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
