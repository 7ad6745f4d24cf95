"""Batched solves: many independent scenes advanced together on one GPU.

Every RK stage launches the stage kernel once per strip length over the
strips of all scenes of the batch (strip-length buckets), so scenes of uneven
size share launches; the step is one CUDA graph.  Results of each scene are
those it gets when solved alone.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .config import CConfig, PSTDConfiguration
from .kernel import PSTDKernel


class BatchKernel(PSTDKernel):
    """A batch of scenes behind one handle (device-resident API only)."""

    def __init__(self, configs: Sequence[PSTDConfiguration], log=None):
        super().__init__()
        L = _lib.lib()
        self._cfgs = [c.copy() for c in configs]
        self._ccs = [CConfig(c) for c in self._cfgs]
        arr = (_lib.c_config * len(self._ccs))(*[cc.c for cc in self._ccs])
        from .kernel import _log_bridge
        logcb = _log_bridge(log)
        cbs = _lib.c_callbacks(None, _lib.WRITE_FRAME(), _lib.WRITE_SAMPLE(), logcb)
        h = ctypes.c_void_p()
        _lib.check(L.pstd_create_batch(arr, len(self._ccs), ctypes.byref(cbs), ctypes.byref(h)))
        self._h = h
        self._keep = [logcb, cbs, arr]
        self._cfg = self._cfgs[0]
        self.info = []
        for i in range(len(self._cfgs)):
            buf = (ctypes.c_int32 * 5)()
            _lib.check(L.pstd_batch_scene(h, i, buf))
            self.info.append({"domain_base": buf[0], "domains": buf[1], "receiver_base": buf[2],
                              "receivers": buf[3], "framecount": buf[4]})
        n = ctypes.c_int32()
        _lib.check(L.pstd_batch_size(h, None, ctypes.byref(n)))
        self.n_receivers = n.value

    def __len__(self):
        return len(self._cfgs)

    def run(self, callback):
        raise NotImplementedError("batches are advanced with advance(); run() delivers frames of one scene")

    def receivers(self, first: int = 0, n_steps: Optional[int] = None, scene: Optional[int] = None) -> np.ndarray:
        done = self.steps_done()
        n_steps = done - first if n_steps is None else n_steps
        out = np.zeros((n_steps, self.n_receivers), dtype=np.float32)
        if self.n_receivers and n_steps:
            _lib.check(_lib.lib().pstd_get_receivers(self._need(), first, n_steps,
                                                     out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        if scene is None:
            return out
        i = self.info[scene]
        return out[:, i["receiver_base"]:i["receiver_base"] + i["receivers"]]

    def scene_snapshot(self, scene: int, local_domain: int, field: str) -> np.ndarray:
        return self.snapshot(self.info[scene]["domain_base"] + local_domain, field)
