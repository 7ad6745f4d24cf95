"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm import this module, and only as the checker (or, for the reference arm,
as the stand-in for the reference's CPU PSTDKernel, which cannot be built
here).  The product (openpstd_gb300) never imports it.

The C++ source (pstd_oracle.cpp) restates openPSTD's kernel/core algorithms;
see its header for what it follows and which quirks it reproduces.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "pstd_oracle.cpp")
_LIB = os.path.join(_HERE, "liboracle.so")

sys.path.insert(0, os.path.dirname(_HERE))
from openpstd_gb300.config import CConfig, PSTDConfiguration, c_domain_info  # noqa: E402


REFERENCE = "/root/reference"


def unqlite_lib():
    """Path of the reference's unqlite store built into oracle/_ref (make), or
    None where the reference tree is absent."""
    out = os.path.join(_HERE, "_ref", "libunqlite.so")
    if os.path.exists(os.path.join(REFERENCE, "unqlite", "unqlite.c")):
        subprocess.check_call(["make", "-s", "-C", _HERE, "_ref/libunqlite.so", f"REF={REFERENCE}"])
    return out if os.path.exists(out) else None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (OpenMP on)."""
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", _LIB + ".tmp", _SRC]
        subprocess.check_call(cmd)
        os.replace(_LIB + ".tmp", _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        P = ctypes.POINTER
        i32, f64, vp = ctypes.c_int32, ctypes.c_double, ctypes.c_void_p
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_create.argtypes = [vp, i32, P(vp)]
        L.orc_destroy.argtypes = [vp]
        L.orc_framecount.argtypes = [vp, P(i32)]
        L.orc_run.argtypes = [vp, i32, i32, vp, vp]
        L.orc_receiver_count.argtypes = [vp, P(i32)]
        L.orc_get_receivers.argtypes = [vp, P(f64), ctypes.c_int64]
        L.orc_domain_count.argtypes = [vp, P(i32)]
        L.orc_domain_info.argtypes = [vp, i32, P(c_domain_info)]
        L.orc_neighbours.argtypes = [vp, i32, i32, P(i32), i32, P(i32)]
        L.orc_snapshot.argtypes = [vp, i32, i32, P(f64), ctypes.c_int64]
        L.orc_next_2_power.argtypes = [f64]
        L.orc_next_2_power.restype = i32
        L.orc_window_size.argtypes = [ctypes.c_float]
        L.orc_window_size.restype = i32
        L.orc_window.argtypes = [i32, i32, i32, P(f64)]
        L.orc_rho_array.argtypes = [f64, f64, f64, i32, P(f64)]
        L.orc_discretization.argtypes = [ctypes.c_float, i32, i32, P(i32), P(f64), P(f64), P(f64), P(f64), i32]
        L.orc_spatderp3.argtypes = [P(f64), i32, P(f64), i32, P(f64), i32, P(f64), i32, P(f64), i32,
                                    f64, f64, f64, i32, i32, P(f64)]
        L.orc_max_threads.restype = i32
        L.orc_fft_seconds.argtypes = [i32, i32, i32, i32, P(f64)]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oracle error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc != 0:
        raise OracleError(rc, lib().orc_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


FRAME_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                            ctypes.POINTER(ctypes.c_double), ctypes.c_int64)

FIELDS = {"p0": 0, "px": 1, "py": 2, "vx": 3, "vy": 4, "pml_px": 5, "pml_py": 6, "pml_vx": 7, "pml_vy": 8}


class OracleScene:
    """One scene of the CPU restatement, float (precision=32) or double (64)."""

    def __init__(self, conf: PSTDConfiguration, precision: int = 32):
        self._cc = CConfig(conf)
        self.precision = precision
        h = ctypes.c_void_p()
        _check(lib().orc_create(ctypes.cast(self._cc.ptr(), ctypes.c_void_p), precision, ctypes.byref(h)))
        self.h = h
        n = ctypes.c_int32()
        _check(lib().orc_framecount(self.h, ctypes.byref(n)))
        self.framecount = n.value
        _check(lib().orc_receiver_count(self.h, ctypes.byref(n)))
        self.n_receivers = n.value
        _check(lib().orc_domain_count(self.h, ctypes.byref(n)))
        self.n_domains = n.value
        self.steps_done = 0

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def run(self, n_steps: int = -1, threads: int = 1, on_frame=None):
        cb = None
        if on_frame is not None:
            def _cb(user, frame, dom, data, n):
                on_frame(frame, dom, np.ctypeslib.as_array(data, shape=(n,)).copy())
            cb = FRAME_CB(_cb)
        steps = self.framecount if n_steps < 0 else n_steps
        _check(lib().orc_run(self.h, steps, threads, ctypes.cast(cb, ctypes.c_void_p) if cb else None, None))
        self.steps_done += steps

    def receivers(self) -> np.ndarray:
        n = self.steps_done * self.n_receivers
        out = np.zeros(n, dtype=np.float64)
        _check(lib().orc_get_receivers(self.h, _dp(out), n))
        return out.reshape(self.steps_done, self.n_receivers)

    def domain_info(self, i: int) -> dict:
        d = c_domain_info()
        _check(lib().orc_domain_info(self.h, i, ctypes.byref(d)))
        return d.as_dict()

    def neighbours(self, i: int, direction: int):
        buf = (ctypes.c_int32 * 64)()
        n = ctypes.c_int32()
        _check(lib().orc_neighbours(self.h, i, direction, buf, 64, ctypes.byref(n)))
        return [buf[k] for k in range(n.value)]

    def field_shape(self, i: int, field: str):
        d = self.domain_info(i)
        nx, ny = d["size"]
        return {"p0": (ny, nx), "px": (ny, nx), "py": (ny, nx), "vx": (ny, nx + 1), "vy": (ny + 1, nx),
                "pml_px": (ny, nx), "pml_py": (ny, nx), "pml_vx": (ny, nx + 1), "pml_vy": (ny + 1, nx)}[field]

    def snapshot(self, i: int, field: str) -> np.ndarray:
        shp = self.field_shape(i, field)
        out = np.zeros(shp, dtype=np.float64)
        _check(lib().orc_snapshot(self.h, i, FIELDS[field], _dp(out), out.size))
        return out


# ---- known-answer helpers --------------------------------------------------
def next_2_power(n: float) -> int:
    return lib().orc_next_2_power(float(n))


def window_size(patcherror: float) -> int:
    return lib().orc_window_size(float(patcherror))


def window(W: int, patch_error: int, precision: int = 32) -> np.ndarray:
    out = np.zeros(2 * W + 1)
    _check(lib().orc_window(W, patch_error, precision, _dp(out)))
    return out


def rho_array(rho1, rho_self, rho2, precision: int = 32):
    out = np.zeros(16)
    _check(lib().orc_rho_array(rho1, rho_self, rho2, precision, _dp(out)))
    return out[:8].reshape(4, 2), out[8:].reshape(4, 2)


def discretization(dx: float, N: int, precision: int = 32):
    cap = 1 << 16
    k, ci = np.zeros(cap), np.zeros(cap)
    pd, vd = np.zeros(2 * cap), np.zeros(2 * cap)
    n = ctypes.c_int32()
    _check(lib().orc_discretization(dx, N, precision, ctypes.byref(n), _dp(k), _dp(ci), _dp(pd), _dp(vd), cap))
    m = n.value
    return {"wave_numbers": k[:m], "complex_imag": ci[:m],
            "pressure": pd[:2 * m:2] + 1j * pd[1:2 * m:2], "velocity": vd[:2 * m:2] + 1j * vd[1:2 * m:2]}


def spatderp3(p1, p2, p3, derfact, window_coeffs, wlen, rho1, rho_self, rho2, velocity: bool, precision: int = 32):
    p1, p2, p3 = (np.ascontiguousarray(x, dtype=np.float64) for x in (p1, p2, p3))
    df = np.ascontiguousarray(np.stack([np.real(derfact), np.imag(derfact)], axis=1).ravel(), dtype=np.float64)
    w = np.ascontiguousarray(window_coeffs, dtype=np.float64)
    nout = len(p2) - 1 if velocity else len(p2) + 1
    out = np.zeros(nout)
    _check(lib().orc_spatderp3(_dp(p1), len(p1), _dp(p2), len(p2), _dp(p3), len(p3), _dp(df), len(derfact),
                               _dp(w), wlen, rho1, rho_self, rho2, int(velocity), precision, _dp(out)))
    return out


def max_threads() -> int:
    return lib().orc_max_threads()


def fft_seconds(L: int, n_strips: int, threads: int, reps: int = 3) -> float:
    """Seconds for n_strips real strips of length L through the oracle's own
    r2c -> multiply -> c2r (the transform core of its strip derivative)."""
    out = ctypes.c_double()
    _check(lib().orc_fft_seconds(L, n_strips, threads, reps, ctypes.byref(out)))
    return out.value
