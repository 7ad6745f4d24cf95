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
def test_cli_run_gpu_and_device_subsampling(tmp_path):
    from openpstd_gb300 import scenes
    from openpstd_gb300.kernel import KernelCallback, PSTDKernel
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
