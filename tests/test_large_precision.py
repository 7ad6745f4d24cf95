"""Large-scene precision (the 2x2-domain square of the precision workload at
half size: 4096x4096 cells, strips of transform length 4096): FP32 GPU
against the FP64 oracle, next to the float oracle's own distance from FP64."""
import numpy as np
import pytest

from parity import rel

pytestmark = pytest.mark.gpu


def test_large_square_fp32_vs_fp64(oracle_mod):
    from openpstd_gb300 import scenes
    from openpstd_gb300.kernel import PSTDKernel
    steps = 3
    conf = scenes.large_square(1, half=2048, steps=steps, n_receivers=16)
    k = PSTDKernel()
    k.initialize_kernel(conf)
    k.advance(steps)
    k.synchronize()
    o64 = oracle_mod.OracleScene(conf, 64)
    o64.run(steps, threads=oracle_mod.max_threads())
    o32 = oracle_mod.OracleScene(conf, 32)
    o32.run(steps, threads=oracle_mod.max_threads())
    # after a few steps the pulse has not reached the receivers (their series
    # are round-off), so the whole fields are compared
    for d in range(4):                               # the four air domains
        for f in ("p0", "vx", "vy"):
            w = o64.snapshot(d, f)
            e, fl = rel(k.snapshot(d, f), w), rel(o32.snapshot(d, f), w)
            print(d, f, "gpu vs f64", e, "f32 oracle vs f64", fl)
            assert e <= max(1e-5, 3 * fl + 1e-6), (d, f, e, fl)
