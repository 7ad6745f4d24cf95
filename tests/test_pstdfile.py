"""Scene files (.pstd): the reference's PSTDFile store (shared/PSTDFile.cpp)
restated over its unqlite key/value engine.

The engine is the reference's vendored unqlite/unqlite.c compiled into
oracle/_ref by oracle/Makefile (these tests skip where the reference tree is
absent).  Keys and values are also read back here through unqlite's own API
(ctypes), independently of the library's file code, to pin the record layout:
int32 keys {prefix, indices...}, prefixes 1 / 100 / 102 / 103 / 104 / 10000,
version 4 (shared/PSTDFile.cpp:50-60).

The scene record is a Boost text archive of PSTDConfiguration.  Boost is not
available here, so the expected text of CreateDefaultConf below is written
from Boost.Serialization's text-archive rules (header, "tracking version" on
the first object of each class, vector = count, element version, elements)
and the member order of the reference's serialize functions
(kernel/KernelInterface.h:80-97,170-175,196-205,233-240,
shared/PSTDFile.h:63-111); it is not checked against Boost itself.
"""
import ctypes
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def unq(pstd_lib):
    from oracle import oracle
    path = oracle.unqlite_lib()
    if path is None:
        pytest.skip("the reference's unqlite source is not available")
    return path


class RawStore:
    """unqlite's own key/value API, for reading records without the library."""

    def __init__(self, lib_path, file_path):
        self.L = ctypes.CDLL(lib_path)
        self.L.unqlite_kv_fetch.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.POINTER(ctypes.c_int64)]
        self.L.unqlite_kv_store.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                            ctypes.c_int64]
        self.L.unqlite_open.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p, ctypes.c_uint]
        self.L.unqlite_close.argtypes = [ctypes.c_void_p]
        self.db = ctypes.c_void_p()
        assert self.L.unqlite_open(ctypes.byref(self.db), file_path.encode(), 0x4) == 0

    def get(self, *key):
        k = struct.pack(f"<{len(key)}I", *key)
        n = ctypes.c_int64()
        if self.L.unqlite_kv_fetch(self.db, k, len(k), None, ctypes.byref(n)) != 0:
            return None
        buf = ctypes.create_string_buffer(n.value)
        assert self.L.unqlite_kv_fetch(self.db, k, len(k), buf, ctypes.byref(n)) == 0
        return buf.raw[:n.value]

    def put(self, value: bytes, *key):
        k = struct.pack(f"<{len(key)}I", *key)
        assert self.L.unqlite_kv_store(self.db, k, len(k), value, len(value)) == 0

    def close(self):
        self.L.unqlite_close(self.db)


DEFAULT_ARCHIVE = (
    "22 serialization::archive 12 "
    # PSTDConfiguration, PSTDSettings class preambles
    "0 0 0 0 "
    # calctime c1 ampMax freqMax rho patcherror tfactRK gridSpacing band_width wave_length
    "1 340 20000 0 1.20000005 70 0.5 0.200000003 8.67000008 0 "
    # rk_coefficients: count, element version, values
    "6 0 0.117979899 0.184646964 0.246623605 0.331839532 0.5 1 "
    # spectral_interpolation PMLCells SaveNth
    "1 50 1 "
    # Speakers: count, element version, QVector3D preamble, x y z
    "1 0 0 0 4 5 0 "
    # Receivers
    "1 0 6 5 0 "
    # Domains: count, element version, DomainConf preamble, QVector2D preamble, TopLeft, Size,
    # DomainConfEdge preamble, T, L, B, R (Absorption LR)
    "2 0 0 0 0 0 0 0 10 15 0 0 1 0 0.300000012 0 0 0 1 0 "
    "10 4 20 15 1 0 1 0 0 0 1 0\n")


def test_default_scene_archive_text():
    from openpstd_gb300.config import PSTDConfiguration
    from openpstd_gb300.pstdfile import archive_text
    assert archive_text(PSTDConfiguration.CreateDefaultConf()) == DEFAULT_ARCHIVE


def _f32(conf):
    """The configuration as the reference's float members hold it."""
    d = conf.to_dict()

    def walk(x):
        if isinstance(x, float):
            return float(np.float32(x))
        if isinstance(x, list):
            return [walk(v) for v in x]
        if isinstance(x, dict):
            return {k: walk(v) for k, v in x.items()}
        return x
    return walk(d)


def test_new_file_records(unq, tmp_path):
    """PSTDFile::New: version 4 under {10000}, the default scene under {1}, an
    empty results scene under {100}."""
    from openpstd_gb300.config import PSTDConfiguration
    from openpstd_gb300.pstdfile import PSTDFile
    p = str(tmp_path / "new.pstd")
    f = PSTDFile.New(p, unq)
    assert _f32(f.GetSceneConf()) == _f32(PSTDConfiguration.CreateDefaultConf())
    assert f.GetResultsSceneConf().Domains == []
    f.close()
    raw = RawStore(unq, p)
    assert struct.unpack("<i", raw.get(10000))[0] == 4
    assert raw.get(1).decode() == DEFAULT_ARCHIVE
    rs = raw.get(100).decode()
    assert rs.startswith("22 serialization::archive 12 0 0 0 0 0 0 0 0 0 0 0 0 0 0 0 0 0 0 ") and rs.rstrip().endswith("0 0 0 0 0 0")
    raw.close()


@pytest.mark.parametrize("which", ["lshape", "batch", "empty"])
def test_scene_round_trip(unq, tmp_path, which):
    from openpstd_gb300 import scenes
    from openpstd_gb300.config import PSTDConfiguration
    from openpstd_gb300.pstdfile import PSTDFile
    conf = {"lshape": lambda: scenes.l_shape(1, scale=0.2, steps=20),
            "batch": lambda: scenes.batch_scenes(4, n=1, steps=30)[0],
            "empty": PSTDConfiguration.CreateEmptyConf}[which]()
    p = str(tmp_path / "s.pstd")
    with PSTDFile.New(p, unq) as f:
        f.SetSceneConf(conf)
        f.Commit()
    with PSTDFile.Open(p, unq) as g:
        assert _f32(g.GetSceneConf()) == _f32(conf)


def test_results_records(unq, tmp_path):
    """InitializeResults / SaveNextResultsFrame / SaveReceiverData /
    DeleteResults with the reference's keys {102,d}, {103,d,f}, {104,r}."""
    from openpstd_gb300 import scenes
    from openpstd_gb300.pstdfile import PSTDFile
    conf = scenes.l_shape(0, scale=0.1, steps=5)
    p = str(tmp_path / "r.pstd")
    with PSTDFile.New(p, unq) as f:
        f.SetSceneConf(conf)
        f.InitializeResults()
        assert f.GetResultsDomainCount() == len(conf.Domains)
        assert [f.GetResultsFrameCount(d) for d in range(len(conf.Domains))] == [0] * len(conf.Domains)
        for k in range(3):
            f.SaveNextResultsFrame(1, np.arange(6, dtype=np.float32) + k)
        f.SaveReceiverData(2, [1.5])
        f.SaveReceiverData(2, [2.5, 3.5])
        f.Commit()
    raw = RawStore(unq, p)
    assert struct.unpack("<i", raw.get(102, 1))[0] == 3
    assert np.array_equal(np.frombuffer(raw.get(103, 1, 2), np.float32), np.arange(6, dtype=np.float32) + 2)
    assert np.array_equal(np.frombuffer(raw.get(104, 2), np.float32), [1.5, 2.5, 3.5])
    assert raw.get(104, 0) == b""                      # InitializeResults leaves empty receiver records
    raw.close()
    with PSTDFile.Open(p, unq) as g:
        assert g.GetResultsFrameCount(1) == 3
        assert np.array_equal(g.GetResultsFrame(1, 1), np.arange(6, dtype=np.float32) + 1)
        assert np.array_equal(g.GetReceiverData(2), [1.5, 2.5, 3.5])
        g.DeleteResults()
        g.Commit()
    raw = RawStore(unq, p)
    assert raw.get(103, 1, 0) is None and raw.get(102, 1) is None
    raw.close()
    with PSTDFile.Open(p, unq) as g:
        assert g.GetResultsDomainCount() == 0


def test_wrong_version_and_bad_files(unq, tmp_path):
    from openpstd_gb300.pstdfile import PSTDFile, PSTDFileError, PSTDFileVersionError
    p = str(tmp_path / "v.pstd")
    PSTDFile.New(p, unq).close()
    raw = RawStore(unq, p)
    raw.put(struct.pack("<i", 3), 10000)
    raw.close()
    with pytest.raises(PSTDFileVersionError, match=r"Wrong version: 3\(expected: 4\)"):
        PSTDFile.Open(p, unq)
    with pytest.raises(PSTDFileError, match="not a PSTD file"):
        PSTDFile.Open(str(tmp_path / "empty.pstd"), unq)
    with pytest.raises(PSTDFileError, match="cannot load the unqlite library"):
        PSTDFile.New(str(tmp_path / "x.pstd"), str(tmp_path / "no-such-lib.so"))


def test_archive_of_library_version_3(unq, tmp_path):
    """Archives of Boost library versions <= 3 carry no element version in
    collections; they are read as well."""
    from openpstd_gb300.pstdfile import PSTDFile
    text = ("22 serialization::archive 3 0 0 0 0 1 340 20000 0 1.2 70 0.5 0.2 8.67 0 "
            "6 0.1 0.2 0.3 0.4 0.5 1 0 50 1 0 1 0 0 6 5 0 "
            "1 0 0 0 0 0 0 10 15 0 0 1 0 0.3 0 0 0 1 0\n")
    p = str(tmp_path / "old.pstd")
    PSTDFile.New(p, unq).close()
    raw = RawStore(unq, p)
    raw.put(text.encode() + b"\0", 1)
    raw.close()
    with PSTDFile.Open(p, unq) as f:
        c = f.GetSceneConf()
    assert c.Speakers == [] and c.Receivers == [(6.0, 5.0, 0.0)] and len(c.Domains) == 1
    assert c.Settings.rk_coefficients == [float(np.float32(v)) for v in (0.1, 0.2, 0.3, 0.4, 0.5, 1)]
    assert c.Domains[0].L.Absorption == float(np.float32(0.3))


def test_run_command_flow_stores_results(unq, tmp_path):
    """RunCommand's sequence on a .pstd file (CLI/main.cpp:419-449) with a
    stand-in kernel that emits known frames and samples: results land under
    the reference's keys, old results are deleted first."""
    from openpstd_gb300 import scenes
    from openpstd_gb300.__main__ import run_into_file
    from openpstd_gb300.pstdfile import PSTDFile

    class FakeKernel:
        def initialize_kernel(self, conf, log):
            self.conf = conf

        def run(self, cb):
            for frame in range(4):
                for d in range(2):
                    cb.WriteFrame(frame, d, np.full(3, 10 * frame + d, np.float32))
                for r in range(len(self.conf.Receivers)):
                    cb.WriteSample(frame, r, [float(frame + r)])

    conf = scenes.l_shape(2, scale=0.1, steps=4)
    p = str(tmp_path / "run.pstd")
    with PSTDFile.New(p, unq) as f:
        f.SetSceneConf(conf)
        f.InitializeResults()
        for _ in range(7):
            f.SaveNextResultsFrame(0, np.zeros(2, np.float32))   # stale results of an earlier run
        f.Commit()
    n = run_into_file(p, FakeKernel(), unqlite_lib=unq, log=lambda m: None)
    assert n == 8
    with PSTDFile.Open(p, unq) as g:
        assert g.GetResultsFrameCount(0) == 4 and g.GetResultsFrameCount(1) == 4
        assert np.array_equal(g.GetResultsFrame(3, 1), np.full(3, 31, np.float32))
        assert np.array_equal(g.GetReceiverData(1), [1.0, 2.0, 3.0, 4.0])
        assert _f32(g.GetResultsSceneConf()) == _f32(conf)
