"""Exact emulation of the stage kernel's strip transform (csrc/stage_kernel.cuh:
DFT<R>, fwd_pass / mid_pass / inv_pass) with the device's float constants and
twiddle tables and exact complex128 arithmetic, for checking the per-bin
round-trip gain model (csrc/transform_gain.hpp) that the derivative filters
are divided by.  Test infrastructure only."""
import numpy as np

f32 = lambda v: float(np.float32(v))
C8, S8, R2 = f32(0.92387953251128674), f32(0.38268343236508978), f32(0.70710678118654752)
C16, S16 = f32(0.98078528040323044913), f32(0.19509032201612826785)
C316, S316 = f32(0.83146961230254523708), f32(0.55557023301960222474)


def _rot32(K, inv, a):
    """a * exp(-/+ 2 pi i K / 32) as tw16 / tw32 do it."""
    sg = 1.0 if inv else -1.0
    if K == 0:
        return a
    if K == 8:
        return a * (1j if inv else -1j)
    if K % 2 == 0:
        c, s = {2: (R2, R2), 6: (-R2, R2), 1: (C8, S8), 3: (S8, C8), 5: (-S8, C8), 7: (-C8, S8)}[K // 2]
    else:
        c, s = {1: (C16, S16), 3: (C316, S316), 5: (S316, C316), 7: (S16, C16), 9: (-S16, C16), 11: (-S316, C316),
                13: (-C316, S316), 15: (-C16, S16)}[K]
    return a * complex(c, sg * s)


def dft(x, inv):
    """DFT<R> along the last axis."""
    R = x.shape[-1]
    if R == 2:
        return np.stack([x[..., 0] + x[..., 1], x[..., 0] - x[..., 1]], -1)
    if R == 4:
        a, b = x[..., 0] + x[..., 2], x[..., 0] - x[..., 2]
        c, d = x[..., 1] + x[..., 3], (x[..., 1] - x[..., 3]) * (1j if inv else -1j)
        return np.stack([a + c, b + d, a - c, b - d], -1)
    e, o = dft(x[..., 0::2], inv), dft(x[..., 1::2], inv).copy()
    for k in range(1, R // 2):
        o[..., k] = _rot32(k * (32 // R), inv, o[..., k])
    return np.concatenate([e + o, e - o], -1)


def _p(m, M):
    a = -2 * np.pi * m / M
    return np.cos(a).astype(np.float32) + 1j * np.sin(a).astype(np.float32)


def _mul32(a, b):
    """cmul on the device: per component one rounded product and one fused
    multiply-add, in float32."""
    a, b = np.asarray(a, complex), np.asarray(b, complex)
    p = np.float32(a.imag * b.imag).astype(float)
    q = np.float32(a.imag * b.real).astype(float)
    return np.float32(a.real * b.real - p).astype(float) + 1j * np.float32(a.real * b.imag + q).astype(float)


def table(M, R, ctw):
    """w[n1][k] of a pass as the device forms them (computed twiddles: float
    products of the stored float powers, make_twiddles)."""
    n1 = np.arange(M // R)[:, None].astype(float)
    if not ctw or R == 2:
        return _p(n1 * np.arange(R)[None, :], M).astype(complex)
    w1 = _p(n1, M).astype(complex)
    one = np.ones_like(w1)
    if R == 4:
        wb = _p(2 * n1, M).astype(complex)
        cols = [one, w1, wb, _mul32(wb, w1)]
    elif R == 8:
        wb = _p(4 * n1, M).astype(complex)
        w2 = _mul32(w1, w1)
        w3 = _mul32(w2, w1)
        cols = [one, w1, w2, w3, wb, _mul32(wb, w1), _mul32(wb, w2), _mul32(wb, w3)]
    else:
        w2, w4, w8 = (_p(m * n1, M).astype(complex) for m in (2, 4, 8))
        lo, hi = [one, w1, w2, _mul32(w2, w1)], [one, w4, w8, _mul32(w8, w4)]
        cols = [(_mul32(hi[k >> 2], lo[k & 3]) if k >> 2 else lo[k & 3]) if k & 3 else hi[k >> 2] for k in range(16)]
    return np.concatenate(cols, 1)


def _passes(radices, lane_pair):
    rad = list(radices)
    if lane_pair:   # the lane-pair mid pass is a radix-2 pass with a table, then radix R/2
        rad = rad[:-1] + [2, rad[-1] // 2]
    return rad


def round_trip_gain(L, radices, ctw=False, lane_pair=False):
    """<inv(fwd(e_k)), e_k> / L^2 for every bin k (no filter)."""
    rad = _passes(radices, lane_pair)
    modes = np.arange(L)
    x = np.exp(2j * np.pi * modes[:, None] * np.arange(L)[None, :] / L)
    M, plan = L, []
    for i, R in enumerate(rad[:-1]):
        ctw_p = ctw and not (lane_pair and i == len(rad) - 2)
        Q = M // R
        y = np.moveaxis(x.reshape(L, L // M, R, Q), 2, -1)
        x = np.moveaxis(dft(y, False) * table(M, R, ctw_p)[None, None], -1, 2).reshape(L, L)
        plan.append((M, R, ctw_p))
        M = Q
    R = rad[-1]
    x = dft(dft(x.reshape(L, L // R, R), False), True).reshape(L, L)
    for M, R, ctw_p in reversed(plan):
        Q = M // R
        y = np.moveaxis(x.reshape(L, L // M, R, Q), 2, -1)
        x = np.moveaxis(dft(y * np.conj(table(M, R, ctw_p))[None, None], True), -1, 2).reshape(L, L)
    e = np.exp(2j * np.pi * modes[:, None] * np.arange(L)[None, :] / L)
    return (x * np.conj(e)).sum(-1) / (L * L)
