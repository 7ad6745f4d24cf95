"""Precision study: tensor-core DFT stages for the long strips against the
FP32 CUDA-core FFT, all measured against the FP64 oracle:
* PSTD_DFT=bf16x3 -- split BF16 (hi + lo, three products) on mma.sync;
* PSTD_DFT=tf32x3 -- split TF32 (three products) on tcgen05 with the
  accumulator in TMEM (L = 8192 strips).
The split forms keep the state in FP32 and accumulate in FP32.  Error budgets
(relative L2): FP32 <= 1e-5, split-TF32 <= 1e-5, split-BF16 <= 1e-4."""
import numpy as np
import pytest

from parity import rel

pytestmark = pytest.mark.gpu


def _gpu(conf, steps, monkeypatch, bf16):
    from openpstd_gb300.kernel import PSTDKernel
    if bf16:
        monkeypatch.setenv("PSTD_DFT", bf16 if isinstance(bf16, str) else "bf16x3")
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


def test_split_tf32_tcgen05_dft_vs_fp64(oracle_mod, monkeypatch):
    """L = 8192 strips with every radix-16 pass as tcgen05 TF32x3 GEMMs."""
    from openpstd_gb300 import scenes
    nx, ny, steps = 4100, 120, 40
    conf = scenes.rect(6, nx=nx, ny=ny, steps=steps)
    o64 = oracle_mod.OracleScene(conf, 64)
    o64.run(steps, threads=oracle_mod.max_threads())
    want = {f: o64.snapshot(0, f) for f in ("p0", "vx", "vy")}
    tf, rec, plan = _gpu(conf, steps, monkeypatch, "tf32x3")
    assert "tcgen05 tf32x3" in plan, plan
    for f in want:
        e = rel(tf[f], want[f])
        print(f"L(8192) {f}: split-tf32 tcgen05 vs fp64 {e:.3e}")
        assert e <= 1e-5
