"""Seeded synthetic scenes for the five PSTD workloads.

The reference publishes no benchmark scenes; these generators build
``PSTDConfiguration`` objects with the shapes, sizes and value distributions of
the workloads:

* ``plain_square``   -- 200x200 cells, dx=0.2 m, 50-cell PML on all edges
  (alpha=1), window 32, CFL 0.5, 1 speaker, 4 receivers, 500 steps.
* ``l_shape``        -- 1200x600 + 600x600 + 600x1200 cells sharing windowed
  interfaces, outer edges a seeded mix of rigid (alpha=0) and alpha=0.3 with
  a 50-cell PML, 4 speakers, 16 receivers, 4000 steps.
* ``batch_scenes``   -- independent scenes whose total size is log-uniform in
  64x64 ... 1024x768 cells, 1-6 rectangles in a seeded grid layout with
  exactly aligned shared edges, edge alpha ~ U[0,1], 1-4 speakers, 1-8
  receivers, 2000 steps.
* ``large_square``   -- 8192x8192 cells as 2x2 domains of 4096^2, PML on the
  outer edges, 2 speakers, 64 receivers, 1000 steps.
* serving arrivals  -- ``batch_scenes``-like draws with step counts
  log-uniform in 200 ... 8000 (see ``serving_requests``).

Every generator places domains on exact grid coordinates (world / dx in
float32 truncates to the intended integer), keeps speakers and receivers at
least 1 m inside the edges, and rejects layouts that make the reference read
undefined memory: a transform length N+2W equal to a power of two, a receiver
whose transposed index (row = x offset) falls outside p0, domains narrower
than the window.  ``scale`` shrinks a layout for tests.
"""
from __future__ import annotations

import math
from typing import List, Optional, Tuple

import numpy as np

from .config import DomainConf, DomainConfEdge, PSTDConfiguration

f32 = np.float32


def _grid_world(cells: int, dx: float) -> float:
    """World coordinate whose float32 division by dx truncates to `cells`."""
    dxf = f32(dx)
    v = f32(cells * float(dxf))
    for _ in range(8):
        if int(f32(v / dxf)) == cells:
            return float(v)
        v = np.nextafter(v, f32(np.inf))
    raise ValueError(f"no float32 world coordinate maps to {cells} cells at dx={dx}")


def base_settings(conf: PSTDConfiguration, steps: int, dx: float = 0.2, pml: int = 50, save_nth: int = 1):
    s = conf.Settings
    s.SetSoundSpeed(340.0)
    s.SetAttenuationOfPMLCells(20000.0)
    s.SetDensityOfAir(1.2)
    s.SetPatchError(70.0)
    s.SetFactRK(0.5)
    s.SetGridSpacing(dx)
    s.SetPMLCells(pml)
    s.SetSaveNth(save_nth)
    s.SetMaxFrequency(1000.0)
    q = float(f32(340.0) / f32(dx))
    s.SetBandWidth(3e-6 * q * q)
    s.SetSpectralInterpolation(False)
    dt = s.GetTimeStep()
    s.SetRenderTime(float(f32((steps + 0.5) * float(dt))))
    assert s.framecount() == steps, (s.framecount(), steps)


def _domain(x0, y0, nx, ny, dx, edges):
    """edges: dict with geometric 'left','right','top'(small y),'bottom'(large y) -> alpha.

    DomainConf's T/B are swapped by the reference (kernel/PSTDKernel.cpp:184-188):
    DomainConf.B is the edge at small y, DomainConf.T the edge at large y."""
    return DomainConf((_grid_world(x0, dx), _grid_world(y0, dx)), (_grid_world(nx, dx), _grid_world(ny, dx)),
                      T=DomainConfEdge(edges["bottom"], False), L=DomainConfEdge(edges["left"], False),
                      B=DomainConfEdge(edges["top"], False), R=DomainConfEdge(edges["right"], False))


def _ok_length(n: int, W: int = 32) -> bool:
    w = W
    while w > n:
        w //= 2
    m = n + 2 * w
    return m & (m - 1) != 0


def _point_in(rng, x0, y0, nx, ny, dx, margin_m=1.0):
    m = int(math.ceil(margin_m / dx))
    gx = rng.integers(x0 + m, x0 + nx - m)
    gy = rng.integers(y0 + m, y0 + ny - m)
    # a fractional offset inside the cell, kept on a float32-exact lattice
    return (float(f32((gx + 0.25) * f32(dx))), float(f32((gy + 0.25) * f32(dx))), 0.0)


def _receiver_in(rng, rect, dx, margin_m=1.0):
    """Receiver position inside rect=(x0,y0,nx,ny) with the transposed lookup in range."""
    x0, y0, nx, ny = rect
    for _ in range(1000):
        p = _point_in(rng, x0, y0, nx, ny, dx, margin_m)
        gx, gy = int(f32(p[0]) / f32(dx)), int(f32(p[1]) / f32(dx))
        if 0 <= gx - x0 < ny and 0 <= gy - y0 < nx:
            return p
    raise ValueError("no receiver position satisfies the transposed index")


# --------------------------------------------------------------------------
def plain_square(seed: int = 0, n: int = 200, steps: int = 500, pml: int = 50, n_receivers: int = 4,
                 dx: float = 0.2) -> PSTDConfiguration:
    """Single square domain with absorbing PML on all four edges."""
    rng = np.random.default_rng(seed)
    conf = PSTDConfiguration()
    base_settings(conf, steps, dx=dx, pml=pml)
    conf.Domains = [_domain(0, 0, n, n, dx, dict(left=1.0, right=1.0, top=1.0, bottom=1.0))]
    conf.Speakers = [_point_in(rng, 0, 0, n, n, dx)]
    conf.Receivers = [_receiver_in(rng, (0, 0, n, n), dx) for _ in range(n_receivers)]
    return conf


def rect(seed: int = 0, nx: int = 1200, ny: int = 100, steps: int = 50, pml: int = 50, n_receivers: int = 2,
         dx: float = 0.2) -> PSTDConfiguration:
    """Single nx x ny domain with absorbing PML on all four edges (long x strips)."""
    rng = np.random.default_rng(seed)
    conf = PSTDConfiguration()
    base_settings(conf, steps, dx=dx, pml=pml)
    conf.Domains = [_domain(0, 0, nx, ny, dx, dict(left=1.0, right=1.0, top=1.0, bottom=1.0))]
    conf.Speakers = [_point_in(rng, 0, 0, nx, ny, dx)]
    conf.Receivers = [_receiver_in(rng, (0, 0, nx, ny), dx) for _ in range(n_receivers)]
    return conf


def l_shape(seed: int = 0, scale: float = 1.0, steps: int = 4000, pml: int = 50, n_speakers: int = 4,
            n_receivers: int = 16, dx: float = 0.2) -> PSTDConfiguration:
    """A (2a x a) + B (a x a) + C (a x 2a), a = 600*scale cells, as an L."""
    rng = np.random.default_rng(seed)
    a = int(round(600 * scale))
    while not (_ok_length(a) and _ok_length(2 * a)):
        a += 1
    conf = PSTDConfiguration()
    base_settings(conf, steps, dx=dx, pml=pml)
    # outer edges: seeded mix of rigid and alpha=0.3; the two edges meeting at
    # the concave corner are rigid so that no PML overlaps an air domain.
    outer = ["A.left", "A.top", "B.top", "B.right", "C.right", "C.bottom"]
    while True:
        alphas = {k: float(rng.choice([0.0, 0.3])) for k in outer}
        if 0.0 in alphas.values() and 0.3 in alphas.values():
            break
    A = dict(left=alphas["A.left"], top=alphas["A.top"], right=1.0, bottom=0.0)
    B = dict(left=1.0, top=alphas["B.top"], right=alphas["B.right"], bottom=1.0)
    C = dict(left=0.0, top=1.0, right=alphas["C.right"], bottom=alphas["C.bottom"])
    rects = [(0, 0, 2 * a, a), (2 * a, 0, a, a), (2 * a, a, a, 2 * a)]
    conf.Domains = [_domain(*rects[0], dx, A), _domain(*rects[1], dx, B), _domain(*rects[2], dx, C)]
    for _ in range(n_speakers):
        r = rects[rng.integers(0, 3)]
        conf.Speakers.append(_point_in(rng, *r, dx))
    for _ in range(n_receivers):
        r = rects[rng.integers(0, 3)]
        conf.Receivers.append(_receiver_in(rng, r, dx))
    return conf


def _split(total: int, parts: int, rng, min_size: int) -> Optional[List[int]]:
    for _ in range(200):
        if parts == 1:
            sizes = [total]
        else:
            cuts = np.sort(rng.choice(np.arange(min_size, total - min_size + 1), size=parts - 1, replace=False))
            sizes = list(np.diff(np.concatenate([[0], cuts, [total]])))
        if all(s >= min_size and _ok_length(int(s)) for s in sizes):
            return [int(s) for s in sizes]
    return None


def batch_scene(rng, steps: int = 2000, min_cells=(64, 64), max_cells=(1024, 768), dx: float = 0.2,
                pml: int = 50, min_domain: int = 40) -> PSTDConfiguration:
    """One scene: total size log-uniform, a rows x cols grid of 1-6 rectangles."""
    lo = math.log(min_cells[0] * min_cells[1])
    hi = math.log(max_cells[0] * max_cells[1])
    for _ in range(1000):
        area = math.exp(rng.uniform(lo, hi))
        aspect = math.exp(rng.uniform(math.log(0.5), math.log(2.0)))
        nx = int(round(math.sqrt(area * aspect)))
        ny = int(round(area / max(nx, 1)))
        nx = min(max(nx, min_cells[0]), max_cells[0])
        ny = min(max(ny, min_cells[1]), max_cells[1])
        n_dom = int(rng.integers(1, 7))
        shapes = [(r, c) for r in range(1, 7) for c in range(1, 7) if r * c == n_dom]
        r, c = shapes[rng.integers(0, len(shapes))]
        if nx < c * min_domain or ny < r * min_domain:
            continue
        ws = _split(nx, c, rng, min_domain)
        hs = _split(ny, r, rng, min_domain)
        if ws is None or hs is None:
            continue
        break
    else:
        raise RuntimeError("could not draw a batch scene")
    conf = PSTDConfiguration()
    base_settings(conf, steps, dx=dx, pml=pml)
    xs = np.concatenate([[0], np.cumsum(ws)]).astype(int)
    ys = np.concatenate([[0], np.cumsum(hs)]).astype(int)
    outer_alpha = {}
    rects = []
    for i in range(r):
        for j in range(c):
            e = {}
            for side, cond in (("left", j == 0), ("right", j == c - 1), ("top", i == 0), ("bottom", i == r - 1)):
                e[side] = float(f32(rng.uniform(0.0, 1.0))) if cond else 1.0
                if e[side] < 1e-3 and cond:
                    e[side] = 1e-3
            rect = (int(xs[j]), int(ys[i]), int(ws[j]), int(hs[i]))
            rects.append(rect)
            conf.Domains.append(_domain(*rect, dx, e))
    del outer_alpha
    for _ in range(int(rng.integers(1, 5))):
        conf.Speakers.append(_point_in(rng, *rects[rng.integers(0, len(rects))], dx, margin_m=1.0))
    for _ in range(int(rng.integers(1, 9))):
        conf.Receivers.append(_receiver_in(rng, rects[rng.integers(0, len(rects))], dx, margin_m=1.0))
    return conf


def batch_scenes(seed: int = 0, n: int = 256, steps: int = 2000, **kw) -> List[PSTDConfiguration]:
    rng = np.random.default_rng(seed)
    return [batch_scene(rng, steps=steps, **kw) for _ in range(n)]


def large_square(seed: int = 0, half: int = 4096, steps: int = 1000, pml: int = 50, n_speakers: int = 2,
                 n_receivers: int = 64, dx: float = 0.2,
                 receivers_near: Optional[Tuple[float, float]] = None) -> PSTDConfiguration:
    """2x2 domains of half x half cells with PML (alpha=1) on the outer edges.

    ``receivers_near=(r0, r1)`` places every receiver so that the cell it
    samples lies at a seeded distance between r0 and r1 metres from a seeded
    speaker (same speakers as without it), so that a solve of a few dozen
    steps -- the pulse travels c*dt = 0.1 m per step at CFL 0.5 -- already
    records the pulse."""
    rng = np.random.default_rng(seed)
    conf = PSTDConfiguration()
    base_settings(conf, steps, dx=dx, pml=pml)
    rects = []
    for i in range(2):
        for j in range(2):
            e = dict(left=1.0 if j == 0 else 1.0, right=1.0, top=1.0, bottom=1.0)
            rect = (j * half, i * half, half, half)
            rects.append(rect)
            conf.Domains.append(_domain(*rect, dx, e))
    for _ in range(n_speakers):
        conf.Speakers.append(_point_in(rng, *rects[rng.integers(0, 4)], dx))
    for _ in range(n_receivers):
        if receivers_near is None:
            conf.Receivers.append(_receiver_in(rng, rects[rng.integers(0, 4)], dx))
            continue
        sx, sy, _ = conf.Speakers[int(rng.integers(0, n_speakers))]
        for _ in range(1000):
            r = rng.uniform(*receivers_near)
            a = rng.uniform(0.0, 2.0 * math.pi)
            # the cell the receiver samples; the reference reads p0(rel.x, rel.y)
            # with rows = y (kernel/core/Receiver.cpp:82), so a receiver at
            # domain offset (u, v) samples the cell at offset (v, u)
            tx = math.floor((sx + r * math.cos(a)) / dx)
            ty = math.floor((sy + r * math.sin(a)) / dx)
            dom = [(x0, y0, nx, ny) for x0, y0, nx, ny in rects if x0 <= tx < x0 + nx and y0 <= ty < y0 + ny]
            if not dom:
                continue
            x0, y0, nx, ny = dom[0]
            gx, gy = x0 + (ty - y0), y0 + (tx - x0)
            p = (float(f32((gx + 0.25) * f32(dx))), float(f32((gy + 0.25) * f32(dx))), 0.0)
            qx, qy = int(f32(p[0]) / f32(dx)), int(f32(p[1]) / f32(dx))
            if (qx, qy) == (gx, gy) and x0 <= qx < x0 + nx and y0 <= qy < y0 + ny and qx - x0 < ny and qy - y0 < nx:
                conf.Receivers.append(p)
                break
        else:
            raise ValueError("no receiver position near the speaker")
    return conf


def serving_requests(seed: int = 0, rate_hz: float = 50.0, duration_s: float = 600.0,
                     min_steps: int = 200, max_steps: int = 8000, **kw) -> List[Tuple[float, PSTDConfiguration]]:
    """Poisson arrivals (mean rate_hz) of batch-like scenes, steps log-uniform."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > duration_s:
            break
        steps = int(round(math.exp(rng.uniform(math.log(min_steps), math.log(max_steps)))))
        out.append((t, batch_scene(rng, steps=steps, **kw)))
    return out


def count_cells(conf: PSTDConfiguration) -> int:
    """Air cells of the configured domains (PML excluded)."""
    dx = f32(conf.Settings.GetGridSpacing())
    return sum(int(f32(d.Size[0]) / dx) * int(f32(d.Size[1]) / dx) for d in conf.Domains)
