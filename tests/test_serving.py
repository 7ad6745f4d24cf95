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


def _lengths(conf):
    """Strip transform lengths of a scene (host-side scene build)."""
    import ctypes
    from openpstd_gb300 import _lib
    from openpstd_gb300.config import CConfig, c_domain_info
    cc, h = CConfig(conf), ctypes.c_void_p()
    _lib.check(_lib.lib().pstd_scene_build(ctypes.byref(cc.c), ctypes.byref(h)))
    try:
        n, out = ctypes.c_int32(), set()
        _lib.check(_lib.lib().pstd_scene_domain_count(h, ctypes.byref(n)))
        for i in range(n.value):
            d = c_domain_info()
            _lib.check(_lib.lib().pstd_scene_domain_info(h, i, ctypes.byref(d)))
            out.update(x for x in d.fft_length if x)
        return out
    finally:
        _lib.lib().pstd_destroy(h)


def _form_env(monkeypatch, form):
    """Server form and the solo runs' plan that computes the same arithmetic:
    per_length (variant 0 everywhere), merged (the merged launch) or lengths
    (the per-length persistent configurations)."""
    for k in ("PSTD_VARIANT", "PSTD_SERVE_PERSISTENT", "PSTD_SERVE_FORM", "PSTD_MERGED", "PSTD_PLAN"):
        monkeypatch.delenv(k, raising=False)
    if form == "per_length":
        monkeypatch.setenv("PSTD_VARIANT", "0")
    elif form == "merged":
        monkeypatch.setenv("PSTD_SERVE_FORM", "merged")
        monkeypatch.setenv("PSTD_MERGED", "1")
    else:
        monkeypatch.setenv("PSTD_SERVE_FORM", "lengths")
        monkeypatch.setenv("PSTD_PLAN", "serving")


@pytest.mark.parametrize("form", ["per_length", "merged", "lengths"])
def test_admission_by_footprint(monkeypatch, form):
    """A budget that holds about two scenes at once: the rest wait, every
    request still completes with its solo result, memory stays in budget."""
    from openpstd_gb300.serving import Server
    _form_env(monkeypatch, form)
    confs = _scenes(4, seed=5, max_cells=(320, 256))
    budget = 16 << 20                               # state-set arenas of 4 MiB: two of these scenes
    with Server(budget, max_scenes=8) as srv:
        ids = [srv.submit(c, 20) for c in confs]
        t = srv.tick(8)
        assert t["queued"] >= 1, t                   # not everything fits at once
        assert srv.stats()["persistent"] == (form != "per_length")
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


@pytest.mark.parametrize("form", ["merged", "lengths"])
def test_persistent_form_updates_tables_in_place(monkeypatch, form):
    """The persistent form: each RK stage is one merged launch over the jobs
    of all active scenes (merged) or one persistent launch per strip length
    (lengths), counts read from device memory.  Scenes that join and leave
    rewrite the tables in place -- the step graphs are captured again only
    when a strip length appears that has no job region yet -- and every
    result equals a solo run of the same configurations."""
    from openpstd_gb300.serving import Server
    _form_env(monkeypatch, form)
    confs = _scenes(6, seed=23)
    steps = [41, 18, 66, 29, 52, 35]
    L = [_lengths(c) for c in confs]
    with Server(512 << 20, max_scenes=16) as srv:
        ids = [srv.submit(confs[i], steps[i], final_frame=True) for i in range(3)]
        srv.tick(8)
        ids += [srv.submit(confs[i], steps[i], final_frame=True) for i in range(3, 5)]   # join a running batch
        srv.tick(8)
        ids.append(srv.submit(confs[5], steps[5], final_frame=True))
        srv.run_until_idle(12)
        st = srv.stats()
        assert st["done"] == 6 and st["active"] == 0
        assert st["persistent"], st
        seen = set().union(*L[:3])
        want_captures = 1
        if form == "lengths":
            for group in (L[3] | L[4], L[5]):
                want_captures += not group <= seen
                seen |= group
        assert st["graph_captures"] == want_captures and st["table_updates"] >= 2, st
        for i, rid in enumerate(ids):
            rec, frame = srv.result(rid)
            want_rec, want_frame = _solo(confs[i], steps[i])
            if form == "merged":
                assert np.array_equal(rec, want_rec), (i, rel(rec, want_rec))
                assert np.array_equal(frame, want_frame), (i, rel(frame, want_frame))
            else:
                assert rel(rec, want_rec) <= 1e-6, (i, rel(rec, want_rec))
                assert rel(frame, want_frame) <= 1e-6, (i, rel(frame, want_frame))


@pytest.mark.parametrize("form", ["merged", "lengths"])
def test_persistent_form_launch_count(monkeypatch, form):
    """Launches per step of the persistent form: six stage launches (merged)
    or six per strip length (lengths), the PML pass and the receiver pass,
    whatever the number of scenes."""
    from openpstd_gb300.serving import Server
    _form_env(monkeypatch, form)
    confs = _scenes(4, seed=5)
    n_len = len(set().union(*[_lengths(c) for c in confs]))
    with Server(512 << 20, max_scenes=8) as srv:
        for c in confs:
            srv.submit(c, 20)
        srv.tick(4)
        st = srv.stats()
        assert st["launches_per_step"] == (8 if form == "merged" else 6 * n_len + 2), st
        assert st["active"] == 4 and st["graph_captures"] == 1, st
        srv.run_until_idle(8)


def _long_thin(steps):
    """One 2010 x 70-cell domain with PML: its x strips have transform length
    4096, which the merged persistent launch does not handle."""
    from openpstd_gb300 import scenes
    from openpstd_gb300.config import PSTDConfiguration
    conf = PSTDConfiguration()
    scenes.base_settings(conf, steps, dx=0.2, pml=50)
    conf.Domains.append(scenes._domain(0, 0, 2010, 70, 0.2, dict(left=1.0, right=1.0, top=1.0, bottom=1.0)))
    # the receiver lookup is transposed (row = x offset, as in the reference), so
    # a receiver at cell (20, 40) samples cell (40, 20), 0.72 m from the speaker:
    # the pulse reaches it within a dozen steps
    conf.Speakers.append((float(np.float32(43.25 * 0.2)), float(np.float32(22.25 * 0.2)), 0.0))
    conf.Receivers.append((float(np.float32(20.25 * 0.2)), float(np.float32(40.25 * 0.2)), 0.0))
    return conf


def test_form_switch_for_unmerged_length(monkeypatch):
    """Merged set: a scene with a strip length outside the merged launch's
    range turns the batch to the per-length form while it is active; the
    batch returns to the persistent form after it leaves.  Every result
    matches its solo run to FFT rounding (the per-length form runs its own
    tuned variants)."""
    from openpstd_gb300.serving import Server
    _form_env(monkeypatch, "merged")
    confs = _scenes(2, seed=31)
    thin = _long_thin(12)
    assert 4096 in _lengths(thin)
    with Server(512 << 20, max_scenes=8) as srv:
        a = srv.submit(confs[0], 60, final_frame=True)
        srv.tick(8)
        assert srv.stats()["persistent"]
        b = srv.submit(thin, 12, final_frame=True)
        assert srv.tick(4)["steps"] == 4
        assert not srv.stats()["persistent"]
        srv.tick(8)                                  # the thin scene takes its last 8 steps and leaves
        assert srv.poll(b)["state"] == 2
        c = srv.submit(confs[1], 30, final_frame=True)
        srv.tick(8)
        assert srv.stats()["persistent"]
        srv.run_until_idle(16)
        for conf, rid, n in ((confs[0], a, 60), (thin, b, 12), (confs[1], c, 30)):
            rec, frame = srv.result(rid)
            want_rec, want_frame = _solo(conf, n)
            assert rel(rec, want_rec) <= 1e-5, rel(rec, want_rec)
            assert rel(frame, want_frame) <= 1e-5, rel(frame, want_frame)


def test_lengths_form_takes_any_length(monkeypatch):
    """Per-length set: a 4096 strip length joins as a new job region (one
    more capture) without leaving the persistent form."""
    from openpstd_gb300.serving import Server
    _form_env(monkeypatch, "lengths")
    confs = _scenes(1, seed=31)
    thin = _long_thin(12)
    with Server(512 << 20, max_scenes=8) as srv:
        a = srv.submit(confs[0], 30, final_frame=True)
        srv.tick(8)
        b = srv.submit(thin, 12, final_frame=True)
        srv.tick(8)
        st = srv.stats()
        assert st["persistent"] and st["graph_captures"] == 2, st
        srv.run_until_idle(16)
        for conf, rid, n in ((confs[0], a, 30), (thin, b, 12)):
            rec, frame = srv.result(rid)
            want_rec, want_frame = _solo(conf, n)
            assert rel(rec, want_rec) <= 1e-6, rel(rec, want_rec)
            assert rel(frame, want_frame) <= 1e-6, rel(frame, want_frame)


@pytest.mark.parametrize("form", ["merged", "lengths"])
def test_persistent_tables_grow(monkeypatch, form):
    """Tables that start 512 times smaller grow (reallocated, contents and
    offsets kept, graphs captured again) several times as scenes join; every
    result still equals its solo run."""
    from openpstd_gb300.serving import Server
    _form_env(monkeypatch, form)
    monkeypatch.setenv("PSTD_SERVE_TABLE_DIVISOR", "512")
    confs = _scenes(5, seed=41)
    steps = [30, 22, 26, 18, 24]
    with Server(512 << 20, max_scenes=8) as srv:
        ids = []
        for c, n in zip(confs, steps):   # one scene joins per tick: each membership change grows the tables
            ids.append(srv.submit(c, n))
            srv.tick(3)
        srv.run_until_idle(6)
        st = srv.stats()
        assert st["done"] == 5 and st["persistent"] and st["graph_captures"] >= 3, st
        for conf, rid, n in zip(confs, ids, steps):
            rec, _ = srv.result(rid)
            want, _ = _solo(conf, n)
            if form == "merged":
                assert np.array_equal(rec, want)
            else:
                assert rel(rec, want) <= 1e-6
