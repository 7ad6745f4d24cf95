"""GPU solve against the CPU oracle (float = the reference's CPU PSTDKernel
restated, double = FP64 build), through the C ABI.

Tolerances:
* receiver time series: relative L2 <= 1e-5 against the FP64 oracle wherever
  the float oracle is itself within 1e-5 of FP64, and <= 1e-5 against the
  float oracle where that is within 1e-5/3 of FP64; receivers the wave has
  not reached carry only round-off, and there the GPU must stay within 3x
  the float oracle's distance to FP64;
* final p0/px/py/vx/vy over the whole scene: the GPU's distance to the FP64
  oracle must stay within 2x the float oracle's own distance to FP64 (+1e-6).
  A fixed 1e-5 is not attainable by any FP32 build on absorbing scenes
  (px - py is an undamped round-off walk in the split-field formulation; the
  float oracle itself is ~1e-4 from FP64 on the 500-step square), so the
  bar is the reference-float noise floor measured on the same inputs.
  (Measured: reached receivers 0.5-2e-6 from FP64, fields 0.6-1.55x the
  float oracle's distance.)
"""
import json
import os

import numpy as np
import pytest

from parity import FIELDS, rel, scene_fields

pytestmark = pytest.mark.gpu


def gpu_solve(conf, steps):
    from openpstd_gb300 import kernel
    k = kernel.PSTDKernel()
    k.initialize_kernel(conf)
    k.advance(steps)
    k.synchronize()
    return k


def check_parity(oracle_mod, conf, steps, rec_tol=1e-5, threads=8):
    k = gpu_solve(conf, steps)
    n = k.domain_count()
    rg = k.receivers().astype(np.float64)
    fg = scene_fields(n, lambda i, f: k.snapshot(i, f))
    s32 = oracle_mod.OracleScene(conf, 32)
    s32.run(steps, threads=threads)
    s64 = oracle_mod.OracleScene(conf, 64)
    s64.run(steps, threads=threads)
    r32, r64 = s32.receivers(), s64.receivers()
    f32_, f64_ = scene_fields(n, s32.snapshot), scene_fields(n, s64.snapshot)
    report = {"rec_vs_f32": rel(rg, r32), "rec_vs_f64": rel(rg, r64), "rec_floor": rel(r32, r64)}
    if r64.size:
        # rec_tol against FP64 wherever the float reference itself meets it;
        # receivers the wave has not reached yet carry only round-off (the
        # float reference is then far from FP64 too)
        if report["rec_floor"] <= rec_tol:
            assert report["rec_vs_f64"] <= rec_tol, report
        else:
            assert report["rec_vs_f64"] <= 3 * report["rec_floor"], report
        if report["rec_floor"] <= rec_tol / 3:
            assert report["rec_vs_f32"] <= rec_tol, report
    for f in FIELDS:
        report[f] = (rel(fg[f], f64_[f]), rel(f32_[f], f64_[f]))
    path = os.environ.get("PSTD_PARITY_REPORT")
    if path:   # measured errors, one JSON line per case
        with open(path, "a") as fh:
            fh.write(json.dumps({"case": f"{conf.Settings.framecount()}-frame scene, {steps} steps, "
                                         f"{len(conf.Domains)} domains", **report}) + "\n")
    for f in FIELDS:   # px - py is an undamped round-off walk: within 2x the float reference's own error
        err, floor = report[f]
        assert err <= 2 * floor + 1e-6, (f, err, floor)
    return k, report


def test_plain_square_full(oracle_mod):
    """200x200 cells + 50-cell PML, 500 steps (the CPU-runnable workload)."""
    from openpstd_gb300 import scenes
    _, rep = check_parity(oracle_mod, scenes.plain_square(0), 500, threads=16)
    print(rep)


@pytest.mark.parametrize("seed,scale,steps", [(0, 0.2, 400), (1, 0.25, 300), (3, 0.15, 200)])
def test_l_shape(oracle_mod, seed, scale, steps):
    from openpstd_gb300 import scenes
    _, rep = check_parity(oracle_mod, scenes.l_shape(seed, scale=scale, steps=steps), steps, threads=16)
    print(rep)


@pytest.mark.parametrize("seed", [5, 11, 17])
def test_batch_like_scenes(oracle_mod, seed):
    from openpstd_gb300 import scenes
    conf = scenes.batch_scenes(seed, n=1, steps=120, max_cells=(320, 256))[0]
    _, rep = check_parity(oracle_mod, conf, 120, threads=16)
    print(rep)


def test_reference_domain_test_scene(oracle_mod):
    """The scene of test/Kernel/Domain.cpp (alpha 0 / 0.25 / 0.35 LR / 0.7 edges)."""
    from openpstd_gb300 import config as C
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Domains = [C.DomainConf((0, 0), (50, 60), T=C.DomainConfEdge(0, False), L=C.DomainConfEdge(0.35, True),
                                 B=C.DomainConfEdge(0.25, False), R=C.DomainConfEdge(0.7, False))]
    conf.Speakers = [(4.1, 5.1, 0)]
    conf.Receivers = [(10.0, 12.0, 0), (30.0, 20.0, 0)]
    conf.Settings.SetRenderTime(float(60.5 * conf.Settings.GetTimeStep()))
    check_parity(oracle_mod, conf, 60, threads=16)


def test_no_speakers_stays_zero():
    from openpstd_gb300 import scenes
    conf = scenes.plain_square(0, n=60, steps=5, pml=40)
    conf.Speakers = []
    k = gpu_solve(conf, 5)
    for i in range(k.domain_count()):
        for f in FIELDS:
            assert not np.any(k.snapshot(i, f))


def test_reset_is_bitwise_reproducible():
    from openpstd_gb300 import scenes
    conf = scenes.l_shape(1, scale=0.15, steps=50)
    k = gpu_solve(conf, 37)
    a = k.receivers().copy()
    snap = k.snapshot(0, "p0").copy()
    k.reset()
    k.advance(37)
    k.synchronize()
    assert np.array_equal(a, k.receivers())
    assert np.array_equal(snap, k.snapshot(0, "p0"))


class Collector:
    def __init__(self):
        from openpstd_gb300 import kernel
        self.frames, self.samples, self.info = [], [], []
        self.kernel = kernel

    def WriteFrame(self, frame, domain, data):
        self.frames.append((frame, domain, data))

    def WriteSample(self, start, receiver, data):
        self.samples.append((start, receiver, list(data)))

    def Info(self, m):
        self.info.append(m)

    def Debug(self, m):
        pass

    Fatal = Error = Warning = Debug


@pytest.mark.parametrize("save_nth", [1, 3])
def test_run_callbacks_match_reference_order(oracle_mod, save_nth):
    """PSTDKernel::run: frames of every non-PML domain, then every receiver's
    sample, for frame % SaveNth == 0, in frame order (kernel/Solver.cpp:71-93)."""
    from openpstd_gb300 import kernel, scenes
    conf = scenes.l_shape(2, scale=0.15, steps=12)
    conf.Settings.SetSaveNth(save_nth)
    k = kernel.PSTDKernel()
    k.initialize_kernel(conf, kernel.KernelCallbackLog())
    md = k.get_metadata()
    assert md.Framecount == 12
    cb = Collector()
    k.run(cb)
    o = oracle_mod.OracleScene(conf, 32)
    oframes = []
    o.run(on_frame=lambda f, d, a: oframes.append((f, d, a)))
    want_frames = [f for f in range(12) if f % save_nth == 0]
    assert [(f, d) for f, d, _ in cb.frames] == [(f, d) for f, d, _ in oframes]
    assert sorted({f for f, _, _ in cb.frames}) == want_frames
    # domain ids 0..n-1 in configuration order, row-major Nx*Ny frames
    ids = sorted({d for _, d, _ in cb.frames})
    assert ids == list(range(len(conf.Domains)))
    for (f, d, a), (_, _, b) in zip(cb.frames, oframes):
        nx, ny = md.DomainMetadata[d][:2]
        assert a.shape == (nx * ny,)
        assert rel(a, b) < 1e-5 or np.linalg.norm(b) < 1e-20
    nrec = len(conf.Receivers)
    assert [(s, r) for s, r, _ in cb.samples] == [(f, r) for f in want_frames for r in range(nrec)]
    rec = o.receivers()
    got = np.array([v[0] for _, _, v in cb.samples]).reshape(len(want_frames), nrec)
    assert rel(got, rec[want_frames]) < 1e-5
    assert cb.info[0] == "Starting simulation" and cb.info[-1] == "Succesfully finished simulation"
    assert sum(m.startswith("Finished frame") for m in cb.info) == 12


def test_callback_exception_stops_run():
    from openpstd_gb300 import kernel, scenes

    class Boom(Collector):
        def WriteFrame(self, frame, domain, data):
            if frame == 2:
                raise RuntimeError("stop here")
            super().WriteFrame(frame, domain, data)

    k = kernel.PSTDKernel()
    k.initialize_kernel(scenes.plain_square(0, n=60, steps=8, pml=40))
    cb = Boom()
    with pytest.raises(RuntimeError, match="stop here"):
        k.run(cb)
    assert max(f for f, _, _ in cb.frames) == 1
    k.advance(1)   # the context stays usable
    k.synchronize()


def test_metadata_lists_all_domains():
    from openpstd_gb300 import kernel, scenes
    conf = scenes.l_shape(0, scale=0.2, steps=7)
    k = kernel.PSTDKernel()
    k.initialize_kernel(conf)
    md = k.get_metadata()
    assert md.Framecount == 7
    assert len(md.DomainMetadata) == k.domain_count() > 3
    assert md.DomainMetadata[0] == [240, 120, 0]
    assert md.DomainPositions == []


def test_full_size_l_shape_first_steps(oracle_mod):
    """1200x600 + 600x600 + 600x1200 L-shape at full size: the first steps
    against the oracle (16 threads), then superposition over a longer run."""
    from openpstd_gb300 import scenes
    conf = scenes.l_shape(0, steps=4000)
    k = gpu_solve(conf, 2)
    n = k.domain_count()
    s = oracle_mod.OracleScene(conf, 32)
    s.run(2, threads=16)
    fg = scene_fields(n, lambda i, f: k.snapshot(i, f))
    fo = scene_fields(n, s.snapshot)
    for f in FIELDS:
        assert rel(fg[f], fo[f]) < 2e-6, f
    # after two steps the receivers hold only round-off: compare on the field scale
    scale = np.abs(fo["p0"]).max()
    assert np.abs(k.receivers() - s.receivers()).max() < 1e-6 * scale


def test_full_size_l_shape_superposition():
    """The solve is linear in the initial condition: the field of speakers
    {a, b} is the sum of the fields of {a} and {b}."""
    from openpstd_gb300 import scenes
    conf = scenes.l_shape(4, steps=4000)
    steps = 300
    both = gpu_solve(conf, steps)
    ca, cb = conf.copy(), conf.copy()
    ca.Speakers, cb.Speakers = conf.Speakers[:2], conf.Speakers[2:]
    ka, kb = gpu_solve(ca, steps), gpu_solve(cb, steps)
    rsum = ka.receivers().astype(np.float64) + kb.receivers()
    assert rel(rsum, both.receivers()) < 1e-5
    for f in ("p0", "vx", "vy"):
        a = scene_fields(both.domain_count(), lambda i, g: both.snapshot(i, g))[f]
        b = scene_fields(ka.domain_count(), lambda i, g: ka.snapshot(i, g))[f] + \
            scene_fields(kb.domain_count(), lambda i, g: kb.snapshot(i, g))[f]
        assert rel(b, a) < 1e-5, f


@pytest.mark.parametrize("variant", list(range(26)))
def test_every_stage_variant(oracle_mod, variant, monkeypatch):
    """Each compiled stage-kernel variant (strips per CTA, threads, radix
    plan) must reproduce the oracle: the autotuner may pick any of them."""
    from openpstd_gb300 import scenes
    monkeypatch.setenv("PSTD_VARIANT", str(variant))
    conf = scenes.l_shape(2, scale=0.5, steps=60)      # transform lengths 128, 512, 1024
    _, rep = check_parity(oracle_mod, conf, 60, threads=16)
    print(variant, rep)
    conf = scenes.plain_square(1, n=180, steps=40)     # 128, 256
    check_parity(oracle_mod, conf, 40, threads=16)
    conf = scenes.rect(4, nx=1200, ny=90, steps=30)    # 2048 (x strips), 256, 128
    check_parity(oracle_mod, conf, 30, threads=16)
    conf = scenes.rect(5, nx=2000, ny=60, steps=20)    # 4096 (x strips), 128
    check_parity(oracle_mod, conf, 20, threads=16)
    conf = scenes.rect(7, nx=4100, ny=40, steps=12)    # 8192 (x strips), 128
    check_parity(oracle_mod, conf, 12, threads=16)


def test_merged_launch(oracle_mod, monkeypatch):
    """The merged form -- one persistent launch per RK stage over the strips
    of every transform length, jobs taken from a per-stage counter --
    reproduces the oracle."""
    from openpstd_gb300 import scenes
    from openpstd_gb300.kernel import PSTDKernel
    monkeypatch.setenv("PSTD_MERGED", "1")
    conf = scenes.l_shape(2, scale=0.5, steps=60)      # transform lengths 128, 512, 1024
    k = PSTDKernel()
    k.initialize_kernel(conf)
    assert "merged launch" in k.plan_info()
    k.close()
    check_parity(oracle_mod, conf, 60, threads=16)
    check_parity(oracle_mod, scenes.rect(4, nx=1200, ny=90, steps=30), 30, threads=16)   # 2048, 256, 128


def test_plan_cache_and_pinning(monkeypatch):
    """A scene created a second time takes its autotuned plan from the
    per-process cache (same variants, no timing); PSTD_PLAN pins one
    variant per strip length; both give the oracle-checked results of the
    variants they name (bit-identical to a solo run of those variants)."""
    from openpstd_gb300 import scenes
    from openpstd_gb300.kernel import PSTDKernel
    monkeypatch.delenv("PSTD_VARIANT", raising=False)
    conf = scenes.plain_square(8, n=150, steps=20)
    a = PSTDKernel()
    a.initialize_kernel(conf)
    a.advance(20)
    a.synchronize()
    b = PSTDKernel()
    b.initialize_kernel(conf)
    assert "(plan cache)" in b.plan_info()     # (the first create may itself hit a scene of equal structure)
    b.advance(20)
    b.synchronize()
    assert np.array_equal(a.receivers(), b.receivers())
    monkeypatch.setenv("PSTD_PLAN", "128:1,256:0")
    c = PSTDKernel()
    c.initialize_kernel(conf)
    info = c.plan_info()
    assert info.count("pinned by PSTD_PLAN") == 2 and "(plan cache)" not in info
