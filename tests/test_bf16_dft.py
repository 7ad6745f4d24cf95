"""Precision study: split-BF16 tensor-core DFT stages (PSTD_DFT=bf16x3) for
the long strips against the FP32 CUDA-core FFT, both measured against the
FP64 oracle.  The split form keeps the state in FP32 and accumulates in FP32;
its error budget is relative L2 <= 1e-4 (FP32: <= 1e-5)."""
import numpy as np
import pytest

from parity import rel

pytestmark = pytest.mark.gpu


def _gpu(conf, steps, monkeypatch, bf16):
    from openpstd_gb300.kernel import PSTDKernel
    if bf16:
        monkeypatch.setenv("PSTD_DFT", "bf16x3")
    else:
        monkeypatch.delenv("PSTD_DFT", raising=False)
    k = PSTDKernel()
    k.initialize_kernel(conf)
    k.advance(steps)
    k.synchronize()
    plan = k.plan_info()
    out = {f: k.snapshot(0, f) for f in ("p0", "vx", "vy")}
    rec = k.receivers()
    k.close()
    monkeypatch.delenv("PSTD_DFT", raising=False)
    return out, rec, plan


@pytest.mark.parametrize("nx,ny,steps", [(4100, 120, 40), (2000, 140, 40)])   # transform lengths 8192, 4096
def test_split_bf16_dft_vs_fp64(oracle_mod, monkeypatch, nx, ny, steps):
    from openpstd_gb300 import scenes
    conf = scenes.rect(6, nx=nx, ny=ny, steps=steps)
    o64 = oracle_mod.OracleScene(conf, 64)
    o64.run(steps, threads=oracle_mod.max_threads())
    want = {f: o64.snapshot(0, f) for f in ("p0", "vx", "vy")}
    f32, _, plan32 = _gpu(conf, steps, monkeypatch, False)
    b16, _, plan16 = _gpu(conf, steps, monkeypatch, True)
    assert "bf16x3" in plan16 and "bf16x3" not in plan32
    for f in want:
        e32, e16 = rel(f32[f], want[f]), rel(b16[f], want[f])
        print(f"L({nx}) {f}: fp32 vs fp64 {e32:.3e}   split-bf16 vs fp64 {e16:.3e}")
        assert e32 <= 1e-5
        assert e16 <= 1e-4
