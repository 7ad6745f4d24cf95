"""The C++ kernel API (include/pstd_kernel.hpp): a program written against
it links against libpstd_gb300.so and behaves like openPSTD's PSTDKernel."""
import json
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "kernel_api_driver.cpp")


@pytest.fixture(scope="module")
def driver(pstd_lib, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("cxx") / "kernel_api_driver")
    libdir = os.path.join(ROOT, "openpstd_gb300")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-o", exe, SRC, "-I" + os.path.join(ROOT, "include"),
                           "-L" + libdir, "-lpstd_gb300", "-Wl,-rpath," + libdir])
    return exe


def test_cxx_api_errors_without_gpu(driver):
    out = json.loads(subprocess.check_output([driver, "check"]))
    assert out["not_configured"] and out["run_not_configured"]
    assert out["window"] == 32 and out["domains"] == 2


@pytest.mark.gpu
def test_cxx_api_run_matches_oracle(driver, oracle_mod):
    frames = 30
    out = json.loads(subprocess.check_output([driver, "run", str(frames)]))
    assert out["framecount"] == frames and out["frames"] == frames
    assert out["info"] >= frames
    # the same scene through the oracle
    from openpstd_gb300 import config as C
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Domains = [C.DomainConf((0, 0), (12.0, 12.0), *(C.DomainConfEdge(1.0, False) for _ in range(4)))]
    conf.Settings.SetPMLCells(40)
    conf.Speakers = [(5.05, 6.05, 0)]
    conf.Receivers = [(7.05, 6.05, 0), (3.05, 8.05, 0)]
    conf.Settings.SetRenderTime(float(np.float32((frames + 0.5) * float(conf.Settings.GetTimeStep()))))
    s = oracle_mod.OracleScene(conf, 32)
    s.run()
    got = np.array(out["receivers"]).T
    want = s.receivers()
    assert got.shape == want.shape
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-5


@pytest.mark.gpu
def test_cxx_api_large_frames_owned(driver, monkeypatch):
    """Frames of a 1000 x 600-cell domain: the device copies them straight
    into pooled vectors handed to WriteFrame.  Every kept frame is intact
    after the run, and the frames equal the Python API's (same variants)."""
    monkeypatch.setenv("PSTD_VARIANT", "0")
    frames = 6
    out = json.loads(subprocess.check_output([driver, "big", str(frames)]))
    assert out["frames"] == frames and out["size"] == 1000 * 600
    assert out["sums"] == out["resums"]
    from openpstd_gb300 import config as C
    from openpstd_gb300.kernel import KernelCallback, PSTDKernel
    conf = C.PSTDConfiguration.CreateDefaultConf()
    conf.Domains = [C.DomainConf((0, 0), (200.0, 120.0), *(C.DomainConfEdge(1.0, False) for _ in range(4)))]
    conf.Settings.SetPMLCells(40)
    conf.Speakers = [(100.05, 60.05, 0)]
    conf.Receivers = [(30.05, 20.05, 0)]
    conf.Settings.SetRenderTime(float(np.float32((frames + 0.5) * float(conf.Settings.GetTimeStep()))))
    kept = []

    class Keep(KernelCallback):
        def WriteFrame(self, frame, domain, data):
            kept.append(data)

        def WriteSample(self, start, receiver, data):
            pass

    k = PSTDKernel()
    k.initialize_kernel(conf)
    k.run(Keep())
    k.close()
    assert len(kept) == frames
    assert [float(np.sum(f, dtype=np.float64)) for f in kept] == pytest.approx(out["sums"], rel=1e-12, abs=1e-12)


def test_cxx_pstdfile(pstd_lib, tmp_path):
    """pstd_gb300::PSTDFile (the reference's PSTDFile class on the C ABI),
    used from C++ over the reference's unqlite store."""
    from oracle import oracle
    unq = oracle.unqlite_lib()
    if unq is None:
        pytest.skip("the reference's unqlite source is not available")
    exe = str(tmp_path / "pstdfile_driver")
    libdir = os.path.join(ROOT, "openpstd_gb300")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-o", exe, os.path.join(ROOT, "tests", "cxx", "pstdfile_driver.cpp"),
                           "-I" + os.path.join(ROOT, "include"), "-L" + libdir, "-lpstd_gb300", "-Wl,-rpath," + libdir])
    out = json.loads(subprocess.check_output([exe, str(tmp_path / "scene.pstd"), unq]))
    assert out == {"domains": 2, "receivers": 2, "results_domains": 2, "frames": 3, "frame2": 1.0, "samples": 2,
                   "sample0": 1.25, "open_missing_throws": True, "pml": 50, "window": 32}
