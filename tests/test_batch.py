"""Batched solves: each scene of a batch gets exactly the result it gets
alone (same kernel variant), and matches the oracle."""
import numpy as np
import pytest

from parity import rel

pytestmark = pytest.mark.gpu


def _scenes(n, steps, seed=7):
    from openpstd_gb300 import scenes
    return scenes.batch_scenes(seed, n=n, steps=steps, max_cells=(384, 320))


def test_batch_equals_alone_bitwise(monkeypatch):
    from openpstd_gb300 import kernel
    from openpstd_gb300.batch import BatchKernel
    monkeypatch.setenv("PSTD_VARIANT", "0")
    confs = _scenes(6, 40)
    b = BatchKernel(confs)
    b.advance(40)
    b.synchronize()
    for i, c in enumerate(confs):
        k = kernel.PSTDKernel()
        k.initialize_kernel(c)
        k.advance(40)
        k.synchronize()
        assert np.array_equal(b.receivers(scene=i), k.receivers()), i
        for d in range(b.info[i]["domains"]):
            for f in ("px", "vy"):
                assert np.array_equal(b.scene_snapshot(i, d, f), k.snapshot(d, f)), (i, d, f)


def test_batch_equals_alone_merged(monkeypatch):
    """With the merged launch a scene's jobs are the same alone and in a
    batch: results are bit-identical."""
    from openpstd_gb300 import kernel
    from openpstd_gb300.batch import BatchKernel
    monkeypatch.setenv("PSTD_MERGED", "1")
    confs = _scenes(4, 30, seed=12)
    b = BatchKernel(confs)
    b.advance(30)
    b.synchronize()
    for i, c in enumerate(confs):
        k = kernel.PSTDKernel()
        k.initialize_kernel(c)
        k.advance(30)
        k.synchronize()
        assert np.array_equal(b.receivers(scene=i), k.receivers()), i
        for d in range(b.info[i]["domains"]):
            assert np.array_equal(b.scene_snapshot(i, d, "px"), k.snapshot(d, "px")), (i, d)


def test_batch_matches_oracle(oracle_mod):
    from openpstd_gb300.batch import BatchKernel
    confs = _scenes(4, 150, seed=3)
    b = BatchKernel(confs)
    b.advance(150)
    b.synchronize()
    for i, c in enumerate(confs):
        s32, s64 = oracle_mod.OracleScene(c, 32), oracle_mod.OracleScene(c, 64)
        s32.run(150, threads=16)
        s64.run(150, threads=16)
        got = b.receivers(scene=i).astype(np.float64)
        floor = rel(s32.receivers(), s64.receivers())
        assert rel(got, s64.receivers()) <= max(1e-5, 3 * floor + 1e-6), i
        for d in range(b.info[i]["domains"]):
            want = s64.snapshot(d, "vx")
            if np.linalg.norm(want) > 1e-3:
                f32 = s32.snapshot(d, "vx")
                assert rel(b.scene_snapshot(i, d, "vx"), want) <= 3 * rel(f32, want) + 1e-6, (i, d)


def test_batch_bookkeeping():
    from openpstd_gb300.batch import BatchKernel
    confs = _scenes(3, 10, seed=9)
    b = BatchKernel(confs)
    assert len(b) == 3
    assert b.info[0]["domain_base"] == 0
    assert b.info[1]["domain_base"] == b.info[0]["domains"]
    assert sum(i["receivers"] for i in b.info) == b.n_receivers == sum(len(c.Receivers) for c in confs)
    md = b.get_metadata()
    assert len(md.DomainMetadata) == sum(i["domains"] for i in b.info)
