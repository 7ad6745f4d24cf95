"""Serving loop: continuous batching of scene solves on one GPU.

Thin ctypes layer over ``pstd_server_*`` (include/pstd_gb300.h).  A server
reserves its HBM budget once; ``submit`` queues a scene, ``tick`` admits
queued scenes whose fields fit, advances every active scene together and
finishes those that reached their step count; ``result`` returns a finished
request's receiver series (steps x receivers) and optional last frame.
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional

import numpy as np

from . import _lib
from .config import CConfig, PSTDConfiguration

QUEUED, ACTIVE, DONE, CANCELLED = 0, 1, 2, 3
FINAL_FRAME = 1
STATE_NAMES = {QUEUED: "queued", ACTIVE: "active", DONE: "done", CANCELLED: "cancelled"}


class Server:
    def __init__(self, hbm_budget_bytes: int, max_scenes: int = 1024):
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pstd_server_create(int(hbm_budget_bytes), int(max_scenes), None, ctypes.byref(h)))
        self._h = h
        self._nrec: Dict[int, int] = {}

    def close(self):
        if self._h is not None:
            _lib.lib().pstd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, conf: PSTDConfiguration, n_steps: int, final_frame: bool = False) -> int:
        cc = CConfig(conf)
        rid = ctypes.c_int64()
        _lib.check(_lib.lib().pstd_server_submit(self._h, ctypes.byref(cc.c), int(n_steps),
                                                 FINAL_FRAME if final_frame else 0, ctypes.byref(rid)))
        self._nrec[rid.value] = len(conf.Receivers)
        return rid.value

    def tick(self, max_steps: int = 64) -> dict:
        info = (ctypes.c_int32 * 4)()
        _lib.check(_lib.lib().pstd_server_tick(self._h, int(max_steps), info))
        return {"active": info[0], "queued": info[1], "finished": info[2], "steps": info[3]}

    def poll(self, rid: int) -> dict:
        st, done = ctypes.c_int32(), ctypes.c_int32()
        sizes = (ctypes.c_int64 * 2)()
        _lib.check(_lib.lib().pstd_server_poll(self._h, int(rid), ctypes.byref(st), ctypes.byref(done), sizes))
        return {"state": st.value, "steps_done": done.value, "receiver_floats": sizes[0], "frame_floats": sizes[1]}

    def result(self, rid: int):
        """(receivers [steps x n_receivers], frame or None) of a finished request; forgets it."""
        p = self.poll(rid)
        rec = np.zeros(p["receiver_floats"], np.float32)
        frame = np.zeros(p["frame_floats"], np.float32)
        P = ctypes.POINTER(ctypes.c_float)
        _lib.check(_lib.lib().pstd_server_result(self._h, int(rid), rec.ctypes.data_as(P), rec.size,
                                                 frame.ctypes.data_as(P), frame.size))
        nrec = self._nrec.pop(rid, 0)
        rec = rec.reshape(-1, nrec) if nrec else rec.reshape(0, 0)
        return rec, (frame if frame.size else None)

    def cancel(self, rid: int):
        _lib.check(_lib.lib().pstd_server_cancel(self._h, int(rid)))

    def stats(self) -> dict:
        s = (ctypes.c_int64 * 8)()
        _lib.check(_lib.lib().pstd_server_stats(self._h, s))
        keys = ["budget_bytes", "bytes_in_use", "peak_bytes", "cell_steps", "done", "rebuilds", "active", "queued"]
        out = dict(zip(keys, list(s)))
        f = (ctypes.c_int64 * 4)()
        _lib.check(_lib.lib().pstd_server_launch_stats(self._h, f))
        out.update(graph_captures=f[0], table_updates=f[1], persistent=bool(f[2]), launches_per_step=f[3])
        return out

    def run_until_idle(self, max_steps: int = 64, limit: Optional[int] = None) -> int:
        """Tick until nothing is queued or active; returns the number of ticks."""
        n = 0
        while True:
            t = self.tick(max_steps)
            n += 1
            if t["active"] == 0 and t["queued"] == 0:
                return n
            if limit is not None and n >= limit:
                return n
