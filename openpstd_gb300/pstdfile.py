"""openPSTD scene files (.pstd) over the C ABI (include/pstd_gb300.h).

Mirrors the reference's ``OpenPSTD::Shared::PSTDFile`` (shared/PSTDFile.h:
161-415): an unqlite key/value file with the scene configuration (a Boost
text archive of ``PSTDConfiguration``), the configuration of the last results,
per-domain result frames and per-receiver samples.  The unqlite store is the
shared library the reference builds from its ``unqlite/unqlite.c``; pass its
path as ``unqlite_lib`` or set ``PSTD_UNQLITE_LIB``.

Errors raise :class:`PSTDFileError`; a wrong file version raises
:class:`PSTDFileVersionError` (the reference's ``PSTDFileVersionException``).
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from .config import CConfig, DomainConf, DomainConfEdge, PSTDConfiguration, c_config


class PSTDFileError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[pstd file status {code}] {message}")
        self.code = code


class PSTDFileVersionError(PSTDFileError):
    pass


def _check(rc: int):
    if rc != _lib.PSTD_OK:
        msg = _lib.lib().pstd_file_last_error().decode()
        if rc == _lib.PSTD_ERR_UNSUPPORTED and msg.startswith("Wrong version"):
            raise PSTDFileVersionError(rc, msg)
        raise PSTDFileError(rc, msg)


def config_from_c(c: c_config) -> PSTDConfiguration:
    """PSTDConfiguration from a C pstd_config (arrays copied)."""
    conf = PSTDConfiguration()
    s, cs = conf.Settings, c.settings
    for name in PSTDConfiguration._SETTINGS:
        setattr(s, name, float(getattr(cs, name)))
    s.rk_coefficients = [float(cs.rk_coefficients[k]) for k in range(cs.n_rk_coefficients)]
    s.spectral_interpolation = bool(cs.spectral_interpolation)
    s.PMLCells = int(cs.PMLCells)
    s.SaveNth = int(cs.SaveNth)
    conf.Speakers = [tuple(float(c.speakers[3 * i + e]) for e in range(3)) for i in range(c.n_speakers)]
    conf.Receivers = [tuple(float(c.receivers[3 * i + e]) for e in range(3)) for i in range(c.n_receivers)]
    edge = lambda e: DomainConfEdge(float(e.absorption), bool(e.lr))
    conf.Domains = [DomainConf((float(d.top_left[0]), float(d.top_left[1])), (float(d.size[0]), float(d.size[1])),
                               T=edge(d.T), L=edge(d.L), B=edge(d.B), R=edge(d.R))
                    for d in (c.domains[i] for i in range(c.n_domains))]
    return conf


def archive_text(conf: PSTDConfiguration) -> str:
    """The Boost text archive of ``conf`` as the scene file stores it."""
    cc = CConfig(conf)
    n = ctypes.c_int64()
    _check(_lib.lib().pstd_archive_encode(ctypes.byref(cc.c), None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(_lib.lib().pstd_archive_encode(ctypes.byref(cc.c), buf, n.value + 1, ctypes.byref(n)))
    return buf.value.decode()


class PSTDFile:
    """One open scene file (shared/PSTDFile.cpp)."""

    def __init__(self, path: str, create_new: bool, unqlite_lib: Optional[str] = None):
        h = ctypes.c_void_p()
        _check(_lib.lib().pstd_file_open(str(path).encode(), unqlite_lib.encode() if unqlite_lib else None,
                                         1 if create_new else 0, ctypes.byref(h)))
        self._h = h
        self.path = str(path)

    @staticmethod
    def Open(path: str, unqlite_lib: Optional[str] = None) -> "PSTDFile":
        """An existing file (its version record must be 4)."""
        return PSTDFile(path, False, unqlite_lib)

    @staticmethod
    def New(path: str, unqlite_lib: Optional[str] = None) -> "PSTDFile":
        """A new file: version 4, the CreateDefaultConf scene, an empty results scene."""
        return PSTDFile(path, True, unqlite_lib)

    def _need(self):
        if not self._h:
            raise PSTDFileError(_lib.PSTD_ERR_INVALID, "file is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().pstd_file_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- scene
    def _get(self, results: int) -> PSTDConfiguration:
        c = c_config()
        _check(_lib.lib().pstd_file_get_scene(self._need(), results, ctypes.byref(c)))
        return config_from_c(c)

    def GetSceneConf(self) -> PSTDConfiguration:
        return self._get(0)

    def GetResultsSceneConf(self) -> PSTDConfiguration:
        return self._get(1)

    def SetSceneConf(self, conf: PSTDConfiguration):
        cc = CConfig(conf)
        _check(_lib.lib().pstd_file_set_scene(self._need(), 0, ctypes.byref(cc.c)))

    # ---- results
    def InitializeResults(self):
        _check(_lib.lib().pstd_file_initialize_results(self._need()))

    def DeleteResults(self):
        _check(_lib.lib().pstd_file_delete_results(self._need()))

    def GetResultsDomainCount(self) -> int:
        return len(self.GetResultsSceneConf().Domains)

    def GetResultsReceiverCount(self) -> int:
        return len(self.GetResultsSceneConf().Receivers)

    def GetResultsFrameCount(self, domain: int) -> int:
        n = ctypes.c_int32()
        _check(_lib.lib().pstd_file_frame_count(self._need(), domain, ctypes.byref(n)))
        return n.value

    def SaveNextResultsFrame(self, domain: int, data):
        a = np.ascontiguousarray(data, dtype=np.float32).ravel()
        _check(_lib.lib().pstd_file_save_frame(self._need(), domain, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                               a.size))

    def GetResultsFrame(self, frame: int, domain: int) -> np.ndarray:
        n = ctypes.c_int64()
        _check(_lib.lib().pstd_file_get_frame(self._need(), domain, frame, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float32)
        _check(_lib.lib().pstd_file_get_frame(self._need(), domain, frame,
                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.size,
                                              ctypes.byref(n)))
        return out

    def SaveReceiverData(self, receiver: int, data):
        a = np.ascontiguousarray(data, dtype=np.float32).ravel()
        _check(_lib.lib().pstd_file_append_samples(self._need(), receiver,
                                                   a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), a.size))

    def GetReceiverData(self, receiver: int) -> np.ndarray:
        n = ctypes.c_int64()
        _check(_lib.lib().pstd_file_get_samples(self._need(), receiver, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float32)
        _check(_lib.lib().pstd_file_get_samples(self._need(), receiver,
                                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), out.size,
                                                ctypes.byref(n)))
        return out

    def Commit(self):
        _check(_lib.lib().pstd_file_commit(self._need()))

    def Rollback(self):
        _check(_lib.lib().pstd_file_rollback(self._need()))
