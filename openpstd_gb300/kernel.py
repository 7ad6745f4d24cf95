"""openPSTD's kernel API on the GB300 solver.

Mirrors ``KernelCallbackLog``, ``KernelCallback``, ``SimulationMetadata``,
``KernelInterface``, ``PSTDKernelNotConfiguredException`` and ``PSTDKernel``
(kernel/KernelInterface.h:243-361, kernel/PSTDKernel.h:52-150) with the same
method names and semantics:

* ``initialize_kernel(config, callbackLog)`` builds the scene (on the device);
* ``run(callback)`` advances Framecount time steps and calls
  ``WriteFrame(frame, domain, data)`` for every non-PML domain and
  ``WriteSample(frame, receiver, [p])`` for every receiver when
  ``frame % SaveNth == 0``, in frame order, on the calling thread;
* ``get_metadata()`` lists {Nx, Ny, 0} for every scene domain (PML included)
  and the frame count;
* ``run``/``get_metadata`` before ``initialize_kernel`` raise
  ``PSTDKernelNotConfiguredException`` (kernel/PSTDKernel.cpp:122-123,155-156).

Frames are numpy float32 arrays of length Nx*Ny, row-major with x fastest
(kernel/Solver.cpp:208-217); the callee may keep them.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional

import numpy as np

from . import _lib
from .config import CConfig, PSTDConfiguration, c_domain_info

LOG_LEVELS = ("Fatal", "Error", "Warning", "Info", "Debug")


class KernelCallbackLog:
    """kernel/KernelInterface.h:243-271; every method is a non-blocking no-op by default."""

    def Fatal(self, message: str): pass
    def Error(self, message: str): pass
    def Warning(self, message: str): pass
    def Info(self, message: str): pass
    def Debug(self, message: str): pass


class KernelCallback(KernelCallbackLog):
    """kernel/KernelInterface.h:279-304."""

    def Callback(self, status, message: str, frame: int):   # deprecated in the reference
        pass

    def WriteFrame(self, frame: int, domain: int, data: np.ndarray):
        raise NotImplementedError

    def WriteSample(self, startSample: int, receiver: int, data: List[float]):
        raise NotImplementedError


class SimulationMetadata:
    """kernel/KernelInterface.h:309-329."""

    def __init__(self):
        self.DomainMetadata: List[List[int]] = []
        self.Framecount = 0
        self.DomainPositions: List[List[int]] = []


class PSTDKernelNotConfiguredException(Exception):
    def __str__(self):
        return "The kernel is not yet configured"


class KernelInterface:
    """kernel/KernelInterface.h:332-351."""

    def initialize_kernel(self, config: PSTDConfiguration, callbackLog: KernelCallbackLog): raise NotImplementedError
    def run(self, callback: KernelCallback): raise NotImplementedError
    def get_metadata(self) -> SimulationMetadata: raise NotImplementedError


def _log_bridge(target: Optional[KernelCallbackLog]):
    def _log(user, level, msg):
        if target is None:
            return
        name = LOG_LEVELS[level] if 0 <= level < len(LOG_LEVELS) else "Debug"
        try:
            getattr(target, name)(msg.decode())
        except Exception:   # log callbacks must not break the run
            pass
    return _lib.LOG(_log)


_COPY_CHUNK = 1 << 18            # floats per copy task (1 MiB)
_COPY_THREADS = 8
_copy_pool = None
_POOL_KEEP = 32                  # free frame buffers kept per frame size
_free_frames = {}                # size -> list of float32 arrays no frame uses
_registered = set()              # addresses of pool buffers page-locked for direct device copies
_DIRECT_MIN = 2 * _COPY_CHUNK    # frames of at least this many floats go straight into pool buffers
_DIRECT_CAP = 512 << 20          # most bytes of page-locked pool buffers


_registered_bytes = 0


def _pool_take(n: int, register: bool = False) -> np.ndarray:
    """A pool buffer of n floats; `register`: page-locked if that keeps all
    page-locked pool buffers within _DIRECT_CAP bytes."""
    global _registered_bytes
    free = _free_frames.get(n)
    if free and register:   # prefer a buffer that is page-locked already
        for i in range(len(free) - 1, -1, -1):
            if free[i].ctypes.data in _registered:
                return free.pop(i)
    raw = free.pop() if free else np.empty(n, np.float32)
    if register and raw.ctypes.data not in _registered and _registered_bytes + raw.nbytes <= _DIRECT_CAP:
        if _lib.lib().pstd_host_register(ctypes.c_void_p(raw.ctypes.data), raw.nbytes) == _lib.PSTD_OK:
            _registered.add(raw.ctypes.data)
            _registered_bytes += raw.nbytes
    return raw


class _FrameLease:
    """Owner of a pooled frame buffer handed to a callback.  Every numpy view
    of the frame (and every view of those) keeps the lease alive, so the
    buffer goes back to the pool only when the callee holds no view of it."""
    __slots__ = ("raw", "__array_interface__", "__weakref__")

    def __init__(self, raw):
        self.raw = raw
        self.__array_interface__ = raw.__array_interface__

    def __del__(self):
        _pool_give(self.raw)


def _pool_give(raw):
    global _registered_bytes
    free = _free_frames.setdefault(raw.size, [])
    if len(free) < _POOL_KEEP:
        free.append(raw)
    elif raw.ctypes.data in _registered:
        try:
            _registered.discard(raw.ctypes.data)
            _registered_bytes -= raw.nbytes
            _lib.lib().pstd_host_unregister(ctypes.c_void_p(raw.ctypes.data))
        except Exception:   # interpreter shutdown
            pass


def _reserve_frames(sizes, sets: int):
    """Page-locked pool buffers for `sets` frames of the given domain sizes,
    made ahead of a run (kept for later runs of scenes with those sizes)."""
    need = {}
    for n in sizes:
        if n >= _DIRECT_MIN:
            need[n] = need.get(n, 0) + sets
    if sum(n * 4 * c for n, c in need.items()) > _DIRECT_CAP:
        return
    for n, c in need.items():
        have = [a for a in _free_frames.get(n, []) if a.ctypes.data in _registered]
        made = [_pool_take(n, register=True) for _ in range(max(0, min(c, _POOL_KEEP) - len(have)))]
        for a in made:
            _pool_give(a)


def _copy_frame(ptr, n: int) -> np.ndarray:
    """A float32 array the callee owns, copied from the library's staging
    buffer (valid only during the callback).  Large frames are copied into
    recycled buffers in 1 MiB chunks by a small thread pool (numpy releases
    the GIL while it copies)."""
    src = np.ctypeslib.as_array(ptr, shape=(n,))
    if n < 2 * _COPY_CHUNK:
        return src.copy()
    global _copy_pool
    if _copy_pool is None:
        from concurrent.futures import ThreadPoolExecutor
        _copy_pool = ThreadPoolExecutor(min(_COPY_THREADS, os.cpu_count() or 1), thread_name_prefix="pstd-frame")
    raw = _pool_take(n)
    parts = min(_COPY_THREADS, -(-n // _COPY_CHUNK))
    step = -(-n // parts)
    list(_copy_pool.map(lambda i: np.copyto(raw[i * step:(i + 1) * step], src[i * step:(i + 1) * step]),
                        range(parts)))
    return np.asarray(_FrameLease(raw))


class PSTDKernel(KernelInterface):
    """GPU solver behind the reference's PSTDKernel interface.

    ``GPU`` must be true: this package provides the GPU branch of
    ``PSTDKernel::run`` (kernel/PSTDKernel.cpp:126-141) and has no CPU
    solver.  ``MCPU`` is accepted for signature compatibility and ignored.
    """

    def __init__(self, GPU: bool = True, MCPU: bool = False):
        if not GPU:
            raise ValueError("openpstd_gb300 provides the GPU solver only (PSTDKernel(GPU=True))")
        self.GPU, self.MCPU = GPU, MCPU
        self._h = None
        self._cfg: Optional[PSTDConfiguration] = None
        self._keep = []

    # ---- reference API ---------------------------------------------------
    def initialize_kernel(self, config: PSTDConfiguration, callbackLog: Optional[KernelCallbackLog] = None):
        L = _lib.lib()
        self.close()
        self._cfg = config.copy()
        self._cc = CConfig(self._cfg)
        logcb = _log_bridge(callbackLog)
        cbs = _lib.c_callbacks(None, _lib.WRITE_FRAME(), _lib.WRITE_SAMPLE(), logcb)
        h = ctypes.c_void_p()
        rc = L.pstd_create(ctypes.byref(self._cc.c), ctypes.byref(cbs), ctypes.byref(h))
        _lib.check(rc)
        self._h = h
        self._keep = [logcb, cbs]
        # page-locked frame buffers for run(): the device copies large frames
        # straight into the arrays the callbacks receive (frames in flight + 2)
        sizes = [self.domain_info(i)["size"] for i in range(self.domain_count())]
        frame = [nx * ny for (nx, ny), i in zip(sizes, range(len(sizes))) if not self.domain_info(i)["is_pml"]]
        _reserve_frames(frame, min(8, max(3, (64 << 20) // max(4 * (sum(frame) + 64), 1))) + 2)

    def run(self, callback: KernelCallback, save_nth: int = 0, stride: int = 1):
        """Run Framecount steps with WriteFrame / WriteSample callbacks.

        ``save_nth`` (> 0) overrides the scene's SaveNth; ``stride`` > 1
        subsamples every frame on the device (every stride-th row and column)
        before it is copied to the host (pstd_run_sub)."""
        h = self._need()
        errors = []
        inflight = {}   # address -> pool buffer the device copies a frame into

        def _buffer(user, frame, domain, n):
            # a pool buffer page-locked at initialize_kernel, else the library's staging
            free = _free_frames.get(int(n)) if n >= _DIRECT_MIN else None
            for i in range(len(free) - 1, -1, -1) if free else ():
                if free[i].ctypes.data in _registered:
                    raw = free.pop(i)
                    inflight[raw.ctypes.data] = raw
                    return raw.ctypes.data
            return None

        def _frame(user, frame, domain, data, n):
            try:
                raw = inflight.pop(ctypes.cast(data, ctypes.c_void_p).value, None)
                arr = np.asarray(_FrameLease(raw)) if raw is not None else _copy_frame(data, n)
                callback.WriteFrame(int(frame), int(domain), arr)
                return 0
            except Exception as e:   # stop the run, re-raise after it returns
                errors.append(e)
                return 1

        def _sample(user, start, rec, data, n):
            try:
                callback.WriteSample(int(start), int(rec), [float(data[i]) for i in range(n)])
                return 0
            except Exception as e:
                errors.append(e)
                return 1

        fcb, scb, lcb = _lib.WRITE_FRAME(_frame), _lib.WRITE_SAMPLE(_sample), _log_bridge(callback)
        bcb = _lib.FRAME_BUFFER(_buffer)
        cbs = _lib.c_callbacks(None, fcb, scb, lcb, bcb)
        try:
            if save_nth or stride != 1:
                rc = _lib.lib().pstd_run_sub(h, ctypes.byref(cbs), int(save_nth), int(stride))
            else:
                rc = _lib.lib().pstd_run(h, ctypes.byref(cbs))
        finally:
            for raw in inflight.values():   # frames a stopped run never delivered
                _pool_give(raw)
            inflight.clear()
        if errors:
            raise errors[0]
        _lib.check(rc)

    def get_metadata(self) -> SimulationMetadata:
        h = self._need()
        n = ctypes.c_int32()
        fc = ctypes.c_int32()
        _lib.check(_lib.lib().pstd_get_metadata(h, ctypes.byref(n), None, 0, ctypes.byref(fc)))
        dims = (ctypes.c_int32 * (3 * n.value))()
        _lib.check(_lib.lib().pstd_get_metadata(h, ctypes.byref(n), dims, n.value, ctypes.byref(fc)))
        md = SimulationMetadata()
        md.DomainMetadata = [[dims[3 * i], dims[3 * i + 1], dims[3 * i + 2]] for i in range(n.value)]
        md.Framecount = fc.value
        return md

    # ---- device-resident extras -----------------------------------------
    def _need(self):
        if self._h is None:
            raise PSTDKernelNotConfiguredException()
        return self._h

    def close(self):
        if self._h is not None:
            _lib.lib().pstd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._need()

    def advance(self, n_steps: int, stream: Optional[int] = None):
        """Enqueue n_steps time steps (no callbacks); stream is a cudaStream_t handle or None."""
        _lib.check(_lib.lib().pstd_advance(self._need(), int(n_steps), ctypes.c_void_p(stream) if stream else None))

    def reset(self):
        _lib.check(_lib.lib().pstd_reset(self._need()))

    def synchronize(self):
        _lib.check(_lib.lib().pstd_synchronize(self._need()))

    def steps_done(self) -> int:
        n = ctypes.c_int32()
        _lib.check(_lib.lib().pstd_steps_done(self._need(), ctypes.byref(n)))
        return n.value

    def receivers(self, first: int = 0, n_steps: Optional[int] = None) -> np.ndarray:
        done = self.steps_done()
        n_steps = done - first if n_steps is None else n_steps
        nrec = len(self._cfg.Receivers)
        out = np.zeros((n_steps, nrec), dtype=np.float32)
        if nrec and n_steps:
            _lib.check(_lib.lib().pstd_get_receivers(self._need(), first, n_steps,
                                                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def domain_count(self) -> int:
        n = ctypes.c_int32()
        _lib.check(_lib.lib().pstd_scene_domain_count(self._need(), ctypes.byref(n)))
        return n.value

    def domain_info(self, i: int) -> dict:
        d = c_domain_info()
        _lib.check(_lib.lib().pstd_scene_domain_info(self._need(), i, ctypes.byref(d)))
        return d.as_dict()

    def neighbours(self, i: int, direction: int) -> List[int]:
        buf = (ctypes.c_int32 * 256)()
        n = ctypes.c_int32()
        _lib.check(_lib.lib().pstd_scene_neighbours(self._need(), i, direction, buf, 256, ctypes.byref(n)))
        return [buf[k] for k in range(n.value)]

    def attenuation(self, i: int):
        d = self.domain_info(i)
        nx, ny = d["size"]
        arrs = [np.zeros(nx, np.float32), np.zeros(nx + 1, np.float32), np.zeros(ny, np.float32),
                np.zeros(ny + 1, np.float32)]
        P = ctypes.POINTER(ctypes.c_float)
        _lib.check(_lib.lib().pstd_scene_attenuation(self._need(), i, *[a.ctypes.data_as(P) for a in arrs]))
        return arrs

    def snapshot(self, i: int, field: str) -> np.ndarray:
        d = self.domain_info(i)
        nx, ny = d["size"]
        shape = {"p0": (ny, nx), "px": (ny, nx), "py": (ny, nx), "vx": (ny, nx + 1), "vy": (ny + 1, nx)}[field]
        out = np.zeros(shape, dtype=np.float32)
        _lib.check(_lib.lib().pstd_snapshot(self._need(), i, _lib.FIELD[field],
                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.size))
        return out

    def profile_passes(self, n_steps: int, stream: Optional[int] = None):
        """Advance n_steps with CUDA events around every RK stage."""
        ms, mt = ctypes.c_float(), ctypes.c_float()
        ls, lt = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(_lib.lib().pstd_profile_passes(self._need(), int(n_steps), ctypes.c_void_p(stream) if stream else None,
                                                  ctypes.byref(ms), ctypes.byref(mt), ctypes.byref(ls),
                                                  ctypes.byref(lt)))
        return {"ms_stage": ms.value, "ms_total": mt.value, "stage_launches": ls.value, "total_launches": lt.value}

    def plan_info(self) -> str:
        buf = ctypes.create_string_buffer(1 << 16)
        _lib.check(_lib.lib().pstd_plan_info(self._need(), buf, 1 << 16))
        return buf.value.decode()

    def work_counts(self):
        c, a = ctypes.c_int64(), ctypes.c_int64()
        l_ = ctypes.c_int32()
        _lib.check(_lib.lib().pstd_work_counts(self._need(), ctypes.byref(c), ctypes.byref(a), ctypes.byref(l_)))
        return {"cells": c.value, "air_cells": a.value, "launches_per_step": l_.value}
