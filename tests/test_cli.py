"""Scene files (PSTDConfiguration as JSON) and the command line
(``python -m openpstd_gb300``), mirroring CLI/main.cpp's create / run -g."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cli(*args, cwd=None):
    env = dict(os.environ, PYTHONPATH=ROOT)
    return subprocess.run([sys.executable, "-m", "openpstd_gb300", *args], capture_output=True, text=True, env=env,
                          cwd=cwd)


def test_scene_json_round_trip(tmp_path):
    from openpstd_gb300 import scenes
    from openpstd_gb300.config import CConfig, PSTDConfiguration
    for conf in [PSTDConfiguration.CreateDefaultConf(), scenes.l_shape(3, steps=10), scenes.batch_scenes(2, n=1)[0]]:
        p = tmp_path / "s.json"
        conf.save(str(p))
        back = PSTDConfiguration.load(str(p))
        assert back.to_dict() == conf.to_dict()
        a, b = CConfig(conf), CConfig(back)       # identical C structures
        assert bytes(a.c.settings) == bytes(b.c.settings)
        assert [bytes(a.c.domains[i]) for i in range(a.c.n_domains)] == \
               [bytes(b.c.domains[i]) for i in range(b.c.n_domains)]


def test_cli_create_and_gpu_only(tmp_path):
    from openpstd_gb300.config import PSTDConfiguration
    p = tmp_path / "scene.json"
    r = _cli("create", str(p))
    assert r.returncode == 0, r.stderr
    assert PSTDConfiguration.load(str(p)).to_dict() == PSTDConfiguration.CreateDefaultConf().to_dict()
    r = _cli("run", str(p))                       # without -g: the reference's CPU solvers are not provided
    assert r.returncode == 1 and "-g" in r.stderr


@pytest.mark.gpu
def test_cli_run_gpu_and_device_subsampling(tmp_path, monkeypatch):
    from openpstd_gb300 import scenes
    from openpstd_gb300.kernel import KernelCallback, PSTDKernel
    # both processes run the same variants (each would autotune on its own)
    monkeypatch.setenv("PSTD_VARIANT", "0")
    conf = scenes.plain_square(4, n=90, steps=12, pml=40)
    p = tmp_path / "scene.json"
    conf.save(str(p))
    out = tmp_path / "res.npz"
    r = _cli("run", "-g", str(p), "-o", str(out))
    assert r.returncode == 0, r.stderr
    res = np.load(out)
    # the same run through the API
    got_f, got_s = {}, {}

    class Cb(KernelCallback):
        def WriteFrame(self, frame, domain, data):
            got_f[(domain, frame)] = data

        def WriteSample(self, start, receiver, data):
            got_s.setdefault(receiver, []).extend(data)

    k = PSTDKernel()
    k.initialize_kernel(conf)
    md = k.get_metadata()
    k.run(Cb())
    assert len([x for x in res.files if x.startswith("frame/")]) == len(got_f) == 12
    for (d, f), data in got_f.items():
        nx, ny = md.DomainMetadata[d][:2]
        a = res[f"frame/{d}/{f}"]
        assert a.shape == (nx, ny) and np.array_equal(a.ravel(), data)
    for rr, v in got_s.items():
        assert np.array_equal(res[f"receiver/{rr}"], np.asarray(v, np.float32))
    # device subsampling: every 3rd frame, every 2nd row and column
    sub = {}

    class Sub(KernelCallback):
        def WriteFrame(self, frame, domain, data):
            sub[(domain, frame)] = data

        def WriteSample(self, start, receiver, data):
            pass

    k2 = PSTDKernel()
    k2.initialize_kernel(conf)
    k2.run(Sub(), save_nth=3, stride=2)
    assert sorted(f for _, f in sub) == [0, 3, 6, 9]
    for (d, f), data in sub.items():
        nx, ny = md.DomainMetadata[d][:2]
        full = got_f[(d, f)].reshape(ny, nx)        # row-major, x fastest
        assert np.array_equal(data, full[::2, ::2].ravel())


@pytest.fixture(scope="module")
def kv_standin(tmp_path_factory):
    """A key/value store with unqlite's entry points (tests/cxx/kv_standin.cpp),
    for machines without the reference's unqlite source."""
    so = str(tmp_path_factory.mktemp("kv") / "libkv_standin.so")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", "-o", so,
                           os.path.join(ROOT, "tests", "cxx", "kv_standin.cpp")])
    return so


def _cxx_cli(*args, unq=None):
    exe = os.path.join(ROOT, "openpstd_gb300", "pstd-cli")
    env = dict(os.environ)
    if unq:
        env["PSTD_UNQLITE_LIB"] = unq
    return subprocess.run([exe, *args], capture_output=True, text=True, env=env)


def test_cxx_cli_create_and_run_stand_in(pstd_lib, kv_standin, tmp_path):
    """The C++ command line (pstd-cli, CLI/main.cpp's create and RunCommand)
    on a .pstd scene file: `create` writes the default scene; `run -M` runs
    RunCommand's sequence with the stand-in kernel and the frames and samples
    land in the file; `run` without -g is refused (no CPU solver).  The file
    is unqlite's where the reference's unqlite source is at hand, else the
    test key/value store's."""
    from oracle import oracle
    from openpstd_gb300.config import PSTDConfiguration
    from openpstd_gb300.pstdfile import PSTDFile
    unq = oracle.unqlite_lib() or kv_standin
    p = str(tmp_path / "scene.pstd")
    r = _cxx_cli("create", p, unq=unq)
    assert r.returncode == 0, r.stderr
    conf = PSTDConfiguration.CreateDefaultConf()
    conf.Settings.SetRenderTime(float(np.float32(3.5 * conf.Settings.GetTimeStep())))   # 3 frames
    with PSTDFile.Open(p, unq) as f:
        f.SetSceneConf(conf)
        f.Commit()
    r = _cxx_cli("run", p, unq=unq)
    assert r.returncode == 1 and "-g" in r.stderr
    r = _cxx_cli("run", "-f", p, "-M", unq=unq)
    assert r.returncode == 0, r.stderr
    assert "Delete old results" in r.stdout and "Finished the stand-in kernel" in r.stdout
    with PSTDFile.Open(p, unq) as f:
        assert f.GetResultsDomainCount() == 2
        assert f.GetResultsFrameCount(0) == 3 and f.GetResultsFrameCount(1) == 3
        assert np.array_equal(f.GetResultsFrame(2, 1), np.full(100 * 75, 2.0, np.float32))   # 20 m x 15 m at 0.2 m
        assert np.array_equal(f.GetReceiverData(0), [0.0, 1.0, 2.0])


def _large_scene(frames):
    from openpstd_gb300 import config as C
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Domains = [C.DomainConf((0, 0), (200.0, 120.0), *(C.DomainConfEdge(1.0, False) for _ in range(4)))]
    conf.Settings.SetPMLCells(40)
    conf.Speakers = [(100.05, 60.05, 0)]
    conf.Receivers = [(30.05, 20.05, 0)]
    conf.Settings.SetRenderTime(float(np.float32((frames + 0.5) * float(conf.Settings.GetTimeStep()))))
    return conf


def test_scene_file_on_standin_store(pstd_lib, kv_standin, tmp_path):
    """The scene-file code over the stand-in store: scene and results round trip."""
    from openpstd_gb300.pstdfile import PSTDFile
    conf = _large_scene(3)
    p = str(tmp_path / "s.pstd")
    with PSTDFile.New(p, kv_standin) as f:
        f.SetSceneConf(conf)
        f.InitializeResults()
        f.SaveNextResultsFrame(0, np.arange(5, dtype=np.float32))
        f.SaveReceiverData(0, [1.5, 2.5])
        f.Commit()
    with PSTDFile.Open(p, kv_standin) as g:
        assert len(g.GetSceneConf().Domains) == 1
        assert g.GetResultsFrameCount(0) == 1 and np.array_equal(g.GetResultsFrame(0, 0), np.arange(5, dtype=np.float32))
        assert np.array_equal(g.GetReceiverData(0), [1.5, 2.5])


@pytest.mark.gpu
def test_cxx_cli_run_gpu_on_scene_file(pstd_lib, kv_standin, tmp_path, monkeypatch):
    """`pstd-cli run -f scene.pstd -g`: RunCommand on the GB300 solver.  The
    frames of a 1000 x 600-cell domain (large enough for the device to copy
    them straight into the vectors CLIOutput stores) and the receiver samples
    land in the scene file and equal the Python API's run of the same scene
    with the same variants.  (The file's key/value store is the test stand-in
    with unqlite's entry points.)"""
    from openpstd_gb300.kernel import KernelCallback, PSTDKernel
    from openpstd_gb300.pstdfile import PSTDFile
    monkeypatch.setenv("PSTD_VARIANT", "0")
    frames = 4
    conf = _large_scene(frames)
    p = str(tmp_path / "scene.pstd")
    with PSTDFile.New(p, kv_standin) as f:
        f.SetSceneConf(conf)
        f.Commit()
    r = _cxx_cli("run", "-f", p, "-g", unq=kv_standin)
    assert r.returncode == 0, r.stderr
    assert "Delete old results" in r.stdout
    got_f, got_s = [], []

    class Keep(KernelCallback):
        def WriteFrame(self, frame, domain, data):
            got_f.append(np.array(data))

        def WriteSample(self, start, receiver, data):
            got_s.extend(data)

    k = PSTDKernel()
    k.initialize_kernel(conf)
    k.run(Keep())
    k.close()
    assert len(got_f) == frames and got_f[0].size == 1000 * 600
    with PSTDFile.Open(p, kv_standin) as f:
        assert f.GetResultsDomainCount() == 1 and f.GetResultsFrameCount(0) == frames
        for i in range(frames):
            assert np.array_equal(f.GetResultsFrame(i, 0), got_f[i]), i
        assert np.array_equal(f.GetReceiverData(0), np.asarray(got_s, np.float32))
