"""Serving loop (pstd_server_*): continuous batching on one GPU.

Each request's result must be the same alone and in the mix: receiver series
and last frame of a scene served together with others -- admitted at
different ticks, finishing at different times -- equal a solo
pstd_create + pstd_advance of that scene with the same kernel variants.
"""
import numpy as np
import pytest

from parity import rel

pytestmark = pytest.mark.gpu


def _scenes(n, seed, max_cells=(256, 192)):
    from openpstd_gb300 import scenes
    return scenes.batch_scenes(seed, n=n, steps=100, max_cells=max_cells)


def _solo(conf, steps):
    from openpstd_gb300.kernel import PSTDKernel
    k = PSTDKernel()
    k.initialize_kernel(conf)
    k.advance(steps)
    k.synchronize()
    rec = k.receivers()
    frame = np.concatenate([k.snapshot(i, "p0").ravel() for i in range(k.domain_count())
                            if not k.domain_info(i)["is_pml"]])
    k.close()
    return rec, frame


def test_served_results_equal_solo(monkeypatch):
    from openpstd_gb300.serving import Server
    monkeypatch.setenv("PSTD_VARIANT", "0")          # the solo runs use the same variants
    confs = _scenes(5, seed=11)
    steps = [37, 60, 23, 48, 31]
    with Server(512 << 20, max_scenes=16) as srv:
        ids = [srv.submit(confs[i], steps[i], final_frame=True) for i in range(2)]
        srv.tick(10)
        srv.tick(10)
        ids += [srv.submit(confs[i], steps[i], final_frame=True) for i in range(2, 5)]   # join a running batch
        srv.run_until_idle(16)
        st = srv.stats()
        assert st["done"] == 5 and st["active"] == 0 and st["rebuilds"] >= 2
        for i, rid in enumerate(ids):
            assert srv.poll(rid)["state"] == 2
            rec, frame = srv.result(rid)
            want_rec, want_frame = _solo(confs[i], steps[i])
            assert rec.shape == want_rec.shape
            assert rel(rec, want_rec) <= 1e-6, (i, rel(rec, want_rec))
            assert rel(frame, want_frame) <= 1e-6, (i, rel(frame, want_frame))


def test_admission_by_footprint(monkeypatch):
    """A budget that holds about two scenes at once: the rest wait, every
    request still completes with its solo result, memory stays in budget."""
    from openpstd_gb300.serving import Server
    monkeypatch.setenv("PSTD_VARIANT", "0")
    confs = _scenes(4, seed=5, max_cells=(320, 256))
    budget = 16 << 20                               # state-set arenas of 4 MiB: two of these scenes
    with Server(budget, max_scenes=8) as srv:
        ids = [srv.submit(c, 20) for c in confs]
        t = srv.tick(8)
        assert t["queued"] >= 1, t                   # not everything fits at once
        srv.run_until_idle(8)
        st = srv.stats()
        assert st["done"] == 4 and st["peak_bytes"] <= budget
        for c, rid in zip(confs, ids):
            rec, _ = srv.result(rid)
            want, _ = _solo(c, 20)
            assert rel(rec, want) <= 1e-6


def test_cancel_and_oversize(monkeypatch):
    from openpstd_gb300 import _lib, scenes
    from openpstd_gb300.serving import Server
    confs = _scenes(3, seed=2)
    with Server(64 << 20, max_scenes=4) as srv:
        a = srv.submit(confs[0], 50)
        b = srv.submit(confs[1], 50)
        srv.tick(5)
        srv.cancel(a)                                # active
        c = srv.submit(confs[2], 10)
        srv.cancel(c)                                # queued (or just admitted)
        assert srv.poll(a)["state"] == 3 and srv.poll(c)["state"] == 3
        srv.run_until_idle(25)
        assert srv.poll(b)["state"] == 2
        with pytest.raises(_lib.PSTDError) as e:
            srv.submit(scenes.l_shape(0, steps=10), 10)   # needs more than the arenas hold
        assert e.value.code == _lib.PSTD_ERR_NO_MEMORY
