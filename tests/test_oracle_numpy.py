"""Independent numpy (pocketfft) restatement of the strip derivative
(kernel/core/kernel_functions.cpp:123-318) checked against the oracle, so
that the oracle's own FFT and band logic are not the only witness."""
import numpy as np
import pytest


def numpy_spatderp3(p1, p2, p3, derfact, window, W, rho1, rho, rho2, velocity):
    zn1, izn1, zn2, izn2 = rho1 / rho, rho / rho1, rho2 / rho, rho / rho2
    rlw1, tlw1, tlw2 = (zn1 - 1) / (zn1 + 1), 2 * zn1 / (zn1 + 1), 2 * izn1 / (izn1 + 1)
    rrw1, trw1, trw2 = (zn2 - 1) / (zn2 + 1), 2 * zn2 / (zn2 + 1), 2 * izn2 / (izn2 + 1)
    n = len(p2)
    L = 1 << int(np.ceil(np.log2(n + 2 * W)))
    if not velocity:
        dom1 = (p1[-W:] * tlw2 + p2[:W][::-1] * rlw1) * window[:W]
        dom3 = (p3[:W] * trw2 + p2[-W:][::-1] * rrw1) * window[-W:]
    else:
        dom1 = (p1[-W - 1:-1] * tlw1 + p2[1:W + 1][::-1] * -rlw1) * window[:W]
        dom3 = (p3[1:W + 1] * trw1 + p2[-W - 1:-1][::-1] * -rrw1) * window[-W:]
    x = np.zeros(L)
    x[:W], x[W:W + n], x[W + n:2 * W + n] = dom1, p2, dom3
    X = np.fft.rfft(x) * derfact[:L // 2 + 1]
    y = np.fft.irfft(X, L)          # numpy normalises by 1/L like result / fft_length
    return y[W:W + n + 1] if not velocity else y[W:W + n - 1]


@pytest.mark.parametrize("n,W,velocity,rhos", [
    (50, 32, False, (1.2, 1.2, 1.2)), (51, 32, True, (1.2, 1.2, 1.2)),
    (200, 32, False, (13.49, 1.2, 1e30)), (201, 32, True, (13.49, 1.2, 1e30)),
    (600, 32, False, (1.2, 13.49, 1.2)), (601, 32, True, (1.2, 13.49, 1.2)),
    (20, 16, False, (1.2, 1.2, 1.2)), (21, 16, True, (1.2, 1.2, 1.2)),
])
def test_oracle_strip_derivative_matches_numpy(oracle_mod, n, W, velocity, rhos):
    rng = np.random.default_rng(n + W)
    p1, p2, p3 = rng.standard_normal(n + 7), rng.standard_normal(n), rng.standard_normal(n + 3)
    L = 1 << int(np.ceil(np.log2(n + 2 * W)))
    disc = oracle_mod.discretization(0.2, L, 64)
    der = disc["velocity" if velocity else "pressure"]
    w = oracle_mod.window(W, 70, 64)
    want = numpy_spatderp3(p1, p2, p3, der, w, W, *rhos, velocity)
    got64 = oracle_mod.spatderp3(p1, p2, p3, der, w, W, *rhos, velocity=velocity, precision=64)
    got32 = oracle_mod.spatderp3(p1, p2, p3, der, w, W, *rhos, velocity=velocity, precision=32)
    scale = np.linalg.norm(want)
    assert np.linalg.norm(got64 - want) / scale < 1e-12
    assert np.linalg.norm(got32 - want) / scale < 2e-6
