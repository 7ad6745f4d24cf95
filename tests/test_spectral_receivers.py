"""Spectral receivers (pstd_settings.spectral_interpolation =
PSTD_RECEIVERS_SPECTRAL): p0 sampled at the receiver's exact location by
windowed Fourier shifts along x, then y (the interpolation of the reference's
Receiver::compute_with_si, kernel/core/Receiver.cpp:85-121, which is disabled
there).  The oracle's definition is pinned by physics, not by the reference:
a receiver a fraction of a cell off the grid must hear what a grid receiver
hears when the speaker is moved by the same fraction instead.  The GPU is
checked against that oracle (float and FP64)."""
import numpy as np
import pytest

from parity import rel

DX = 0.2


def _spectral(conf, points):
    from openpstd_gb300.config import PSTDConfiguration
    c = PSTDConfiguration.from_dict(conf.to_dict())
    c.Settings.SetReceiverInterpolation("spectral")
    c.Receivers = [(x * DX, y * DX, 0.0) for x, y in points]
    return c


def _l_shape_points():
    # a = 120 cells: A (0..240 x 0..120), B (240..360 x 0..120), C (240..360 x 120..360);
    # points within a window (32 cells) of the A|B and B|C interfaces, inside, near the PML
    a = 120
    return [(2 * a - 5.3, 0.5 * a + 0.41), (2 * a + 4.7, 0.5 * a - 0.27), (2.5 * a + 0.33, a - 3.6),
            (2.5 * a - 0.71, a + 6.2), (0.6 * a + 0.5, 0.4 * a + 0.5), (2.8 * a + 0.12, 2.7 * a + 0.88)]


def test_config_round_trip():
    from openpstd_gb300 import scenes
    from openpstd_gb300.config import CConfig, PSTD_RECEIVERS_SPECTRAL, PSTDConfiguration
    conf = _spectral(scenes.plain_square(0, n=60, steps=5, pml=40), [(30.5, 30.5)])
    back = PSTDConfiguration.from_dict(conf.to_dict())
    assert back.Settings.GetReceiverInterpolation() == "spectral"
    assert CConfig(back).c.settings.spectral_interpolation == PSTD_RECEIVERS_SPECTRAL
    plain = scenes.plain_square(0, n=60, steps=5, pml=40)
    assert "receiver_interpolation" not in plain.to_dict()["Settings"]      # default scenes unchanged
    assert CConfig(plain).c.settings.spectral_interpolation in (0, 1)
    with pytest.raises(ValueError):
        conf.Settings.SetReceiverInterpolation("linear")


def test_oracle_zero_offset_is_the_cell(oracle_mod):
    """On a grid point the shift is the identity: the value of the cell
    itself (x offset, y offset; not the reference's transposed lookup)."""
    from openpstd_gb300 import scenes
    conf = scenes.plain_square(4, n=120, steps=40, pml=40)
    a = oracle_mod.OracleScene(_spectral(conf, [(70.0, 95.0)]), 64)
    a.run(40)
    nn = _spectral(conf, [])
    nn.Settings.SetReceiverInterpolation("nearest")
    nn.Receivers = [(95.0 * DX, 70.0 * DX, 0.0)]          # p0(rel.x, rel.y) reads row 70, column 95 ... transposed
    b = oracle_mod.OracleScene(nn, 64)
    b.run(40)
    r = b.receivers()
    assert np.abs(r).max() > 1e-3
    assert rel(a.receivers(), r) < 1e-12


@pytest.mark.parametrize("fx,fy", [(0.3, 0.6), (0.5, 0.5), (0.9, 0.1)])
def test_oracle_shift_equals_moved_speaker(oracle_mod, fx, fy):
    """Receiver at (70 + fx, 95 + fy) cells == grid receiver at (70, 95) with
    the speaker moved by (-fx, -fy) cells (FP64, 60 steps, before any echo
    of the boundaries reaches the receiver).  The nearest cell is far off."""
    from openpstd_gb300 import scenes
    from openpstd_gb300.config import PSTDConfiguration
    conf = scenes.plain_square(4, n=120, steps=60, pml=40)
    sx, sy = conf.Speakers[0][:2]
    a = oracle_mod.OracleScene(_spectral(conf, [(70.0 + fx, 95.0 + fy)]), 64)
    a.run(60)
    moved = _spectral(conf, [(70.0, 95.0)])
    moved.Speakers = [(sx - fx * DX, sy - fy * DX, 0.0)]
    b = oracle_mod.OracleScene(moved, 64)
    b.run(60)
    got, want = a.receivers()[:, 0], b.receivers()[:, 0]
    scale = np.abs(want).max()
    assert scale > 1e-2
    assert np.abs(got - want).max() / scale < 2e-4           # measured 0.5-0.6e-4
    near = PSTDConfiguration.from_dict(conf.to_dict())
    near.Receivers = [(95.0 * DX, 70.0 * DX, 0.0)]          # the cell (70, 95) under the transposed lookup
    c = oracle_mod.OracleScene(near, 64)
    c.run(60)
    assert np.abs(c.receivers()[:, 0] - want).max() / scale > 0.1


def test_oracle_rejects_far_edge_and_narrow_neighbours(oracle_mod):
    from openpstd_gb300 import scenes
    conf = scenes.plain_square(0, n=60, steps=5, pml=40)
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.OracleScene(_spectral(conf, [(60.0, 30.5)]), 32)   # on the far x edge: no cell to shift from
    # PML (30 cells) narrower than the window (32): the y neighbours' x strips cannot be windowed
    narrow = _spectral(scenes.plain_square(0, n=60, steps=5, pml=30), [(30.5, 30.5)])
    s = oracle_mod.OracleScene(narrow, 32)
    with pytest.raises(oracle_mod.OracleError):
        s.run(1)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["square", "l_shape"])
def test_gpu_matches_oracle(oracle_mod, case):
    """GPU spectral receivers against the float and FP64 oracle: the gate of
    the nearest-neighbour receivers (1e-5 relative L2 against FP64 where the
    float oracle meets it, else 3x the float oracle's own distance)."""
    from openpstd_gb300 import kernel, scenes
    if case == "square":
        conf = _spectral(scenes.plain_square(4, n=120, steps=80, pml=40),
                         [(70.3, 95.6), (84.5, 100.5), (60.9, 60.1), (20.25, 110.75)])
    else:
        conf = _spectral(scenes.l_shape(3, scale=0.2, steps=80), _l_shape_points())
    steps = 80
    k = kernel.PSTDKernel()
    k.initialize_kernel(conf)
    k.advance(steps)
    k.synchronize()
    got = k.receivers().astype(np.float64)
    k.close()
    s32 = oracle_mod.OracleScene(conf, 32)
    s32.run(steps, threads=16)
    s64 = oracle_mod.OracleScene(conf, 64)
    s64.run(steps, threads=16)
    r32, r64 = s32.receivers(), s64.receivers()
    floor = rel(r32, r64)
    report = {"vs_f64": rel(got, r64), "vs_f32": rel(got, r32), "floor": floor}
    print(case, report)
    assert np.abs(r64).max() > 1e-3
    assert report["vs_f64"] <= max(1e-5, 3 * floor), report
    for j in range(r64.shape[1]):      # every receiver, on its own scale
        assert rel(got[:, j], r64[:, j]) <= max(1e-4, 3 * rel(r32[:, j], r64[:, j])), (j, report)


@pytest.mark.gpu
def test_gpu_batch_equals_alone(monkeypatch):
    """Spectral receivers of a batch equal the scenes run alone, bit for bit
    (both on the same stage-kernel variants)."""
    from openpstd_gb300 import kernel, scenes
    from openpstd_gb300.batch import BatchKernel
    monkeypatch.setenv("PSTD_VARIANT", "0")
    confs = [_spectral(scenes.plain_square(4, n=120, steps=30, pml=40), [(70.3, 95.6), (60.9, 60.1)]),
             _spectral(scenes.l_shape(3, scale=0.2, steps=30), _l_shape_points()[:3])]
    b = BatchKernel(confs)
    b.advance(30)
    b.synchronize()
    for i, c in enumerate(confs):
        k = kernel.PSTDKernel()
        k.initialize_kernel(c)
        k.advance(30)
        k.synchronize()
        assert np.array_equal(b.receivers(scene=i), k.receivers()), i
        k.close()


@pytest.mark.gpu
def test_gpu_paths_without_spectral_receivers_refuse():
    """The serving loop and the allocation-free solve keep nearest-neighbour
    receivers only and refuse spectral ones with PSTD_ERR_UNSUPPORTED."""
    import ctypes
    import torch
    from openpstd_gb300 import _lib, scenes
    from openpstd_gb300.config import CConfig
    from openpstd_gb300.serving import Server
    conf = _spectral(scenes.plain_square(0, n=60, steps=5, pml=40), [(30.5, 30.5)])
    srv = Server(1 << 30)
    with pytest.raises(Exception) as e:
        srv.submit(conf, 5)
    assert "spectral" in str(e.value)
    srv.close()
    cc = CConfig(conf)
    rec = torch.zeros(16, dtype=torch.float32, device="cuda")
    rc = _lib.lib().pstd_solve_noalloc(ctypes.byref(cc.c), 5, None, 0, ctypes.c_void_p(rec.data_ptr()), 16, None)
    assert rc == 4


def _plan(conf):
    import ctypes
    from openpstd_gb300 import _lib
    from openpstd_gb300.config import CConfig
    cc = CConfig(conf)
    sizes = (ctypes.c_int64 * 3)()
    L = _lib.lib()
    _lib.check(L.pstd_spectral_plan(ctypes.byref(cc.c), None, None, None, None, sizes))
    nr, nw, nrec = sizes[0], sizes[1], sizes[2]
    rows = np.zeros((nr, 8), np.int32)
    yw = np.zeros(nr, np.float32)
    w = np.zeros(nw, np.float32)
    first = np.zeros(nrec + 1, np.int32)
    _lib.check(L.pstd_spectral_plan(ctypes.byref(cc.c), rows.ctypes.data, yw.ctypes.data, w.ctypes.data,
                                    first.ctypes.data, sizes))
    return rows, yw, w, first


@pytest.mark.parametrize("case", ["square", "l_shape"])
def test_device_plan_reproduces_oracle(pstd_lib, oracle_mod, case):
    """The stencil the device evaluates (pstd_spectral_plan, built on the
    host), applied to the FP64 oracle's p0 fields after some steps, gives the
    oracle's own spectral samples of that step; every index stays inside
    its domain's p0."""
    from openpstd_gb300 import scenes
    if case == "square":
        conf = _spectral(scenes.plain_square(4, n=120, steps=30, pml=40), [(70.3, 95.6), (60.9, 60.1), (3.5, 117.25)])
    else:
        conf = _spectral(scenes.l_shape(3, scale=0.2, steps=30), _l_shape_points())
    rows, yw, w, first = _plan(conf)
    assert first[0] == 0 and first[-1] == len(rows) and np.all(np.diff(first) > 0)
    s = oracle_mod.OracleScene(conf, 64)
    s.run(30, threads=16)
    p0 = [s.snapshot(i, "p0") for i in range(s.n_domains)]
    got = []
    for r in range(len(first) - 1):
        acc = 0.0
        for i in range(first[r], first[r + 1]):
            dom, row, d1, d2, r1, r2, W, wo = (int(v) for v in rows[i])
            ny, nx = p0[dom].shape
            assert 0 <= row < ny and 0 <= wo and wo + 2 * W + nx <= len(w)
            x = np.dot(w[wo + W:wo + W + nx].astype(np.float64), p0[dom][row])
            if d1 >= 0:
                assert 0 <= r1 < p0[d1].shape[0] and W <= p0[d1].shape[1]
                x += np.dot(w[wo:wo + W].astype(np.float64), p0[d1][r1, -W:])
            if d2 >= 0:
                assert 0 <= r2 < p0[d2].shape[0] and W <= p0[d2].shape[1]
                x += np.dot(w[wo + W + nx:wo + 2 * W + nx].astype(np.float64), p0[d2][r2, :W])
            acc += float(yw[i]) * x
        got.append(acc)
    want = s.receivers()[-1]
    assert np.abs(want).max() > 1e-3
    assert rel(got, want) < 1e-6, (got, want)
