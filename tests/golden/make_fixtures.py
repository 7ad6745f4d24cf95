"""Generate the full-size parity fixtures from the CPU oracle.

The oracle (``oracle/pstd_oracle.cpp``) restates the reference's CPU
PSTDKernel (kernel/Solver.cpp:62-117 and kernel/core/*); it is run here in
float (the reference's own precision) and in double (the FP64 oracle) on the
three large workloads, at their stated sizes:

* ``lshape``: the L-shaped 3-domain scene (1200x600 + 600x600 + 600x1200
  cells, 4 speakers, 16 receivers), all 4000 steps;
* ``batch``: 8 scenes of the 256-scene batched workload (seeded choice that
  always includes the largest scene), at full size, 2000 steps each;
* ``large``: the 8192x8192 scene in 2x2 domains of 4096^2 with its 64
  receivers placed 1-3 m from the speakers, 60 steps (the pulse moves 0.1 m
  per step, so every receiver records it).

Each fixture ``<name>.npz`` holds, per scene ``s``:

* ``s/rec32``, ``s/rec64``: receiver series (steps x receivers), float / FP64
  oracle;
* ``s/win``: the sampled window per domain, rows (r0, r1, rs) x columns
  (c0, c1, cs) of the p0-shaped field (vx / vy take the same slices);
* ``s/<dom>/<field>/32``, ``.../64``: the final fields on that window, as
  float32;
* ``s/floor``: whole-scene relative L2 of the float oracle against FP64 per
  field (p0, px, py, vx, vy), computed here on the full fields.

Run (8 host threads, about two and a half hours on 8 cores):

    python tests/golden/make_fixtures.py [--only batch,lshape,large] [--threads 8]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from openpstd_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402

FIELDS = ("p0", "px", "py", "vx", "vy")


def batch_subset():
    """Indices (into batch_scenes(0, n=256)) of the 8 fixture scenes."""
    confs = scenes.batch_scenes(0, n=256, steps=2000)
    cells = [scenes.count_cells(c) for c in confs]
    pick = [int(np.argmax(cells))]
    rng = np.random.default_rng(2026)
    for i in rng.permutation(256):
        if len(pick) == 8:
            break
        if int(i) not in pick:
            pick.append(int(i))
    return pick, confs


def cases(only):
    out = []
    for name in only:
        out += _case(name)
    return out


def _case(name):
    out = []
    if name == "lshape":
        out.append(("lshape", [("lshape", scenes.l_shape(0, steps=4000), 4000, 8)]))
    if name == "batch":
        pick, confs = batch_subset()
        out.append(("batch", [(f"b{i}", confs[i], 2000, 8) for i in pick]))
    if name == "large":
        conf = scenes.large_square(0, half=4096, steps=60, receivers_near=(1.0, 3.0))
        out.append(("large", [("large", conf, 60, 0)]))
    return out


def windows(o: oracle.OracleScene, stride: int, conf):
    """Per domain: a strided sample of the whole domain (stride > 0), or, for
    the large scene (stride 0), a 256x256-cell crop around each speaker at
    stride 2 in the domain holding it (other domains get no window)."""
    out = {}
    dx = float(np.float32(conf.Settings.GetGridSpacing()))
    for i in range(o.n_domains):
        d = o.domain_info(i)
        nx, ny = d["size"]
        if stride > 0:
            out[i] = (0, ny, stride, 0, nx, stride)
            continue
        x0, y0 = d["top_left"]
        for sx, sy, _ in conf.Speakers:
            gx, gy = int(sx / dx) - x0, int(sy / dx) - y0
            if 0 <= gx < nx and 0 <= gy < ny:
                r0, c0 = max(0, gy - 128), max(0, gx - 128)
                out[i] = (r0, min(ny, r0 + 256), 2, c0, min(nx, c0 + 256), 2)
    return out


def sample(a, w):
    r0, r1, rs, c0, c1, cs = w
    return np.ascontiguousarray(a[r0:r1:rs, c0:c1:cs]).astype(np.float32)


def run_scene(key, conf, steps, stride, threads, arrays, meta):
    t0 = time.time()
    runs = {}
    for prec in (32, 64):
        s = oracle.OracleScene(conf, prec)
        s.run(steps, threads=threads)
        runs[prec] = s
        print(f"  {key} fp{prec}: {steps} steps in {time.time() - t0:.0f} s", flush=True)
    s32, s64 = runs[32], runs[64]
    arrays[f"{key}/rec32"] = s32.receivers().astype(np.float32)
    arrays[f"{key}/rec64"] = s64.receivers()
    win = windows(s64, stride, conf)
    arrays[f"{key}/win"] = np.array([[i, *w] for i, w in sorted(win.items())], dtype=np.int64)
    floor = {}
    for f in FIELDS:
        num = den = 0.0
        for i in range(s64.n_domains):
            a32, a64 = s32.snapshot(i, f), s64.snapshot(i, f)
            num += float(np.sum((a32 - a64) ** 2))
            den += float(np.sum(a64 ** 2))
            if i in win:
                arrays[f"{key}/{i}/{f}/32"] = sample(a32, win[i])
                arrays[f"{key}/{i}/{f}/64"] = sample(a64, win[i])
        floor[f] = float(np.sqrt(num / den)) if den > 0 else 0.0
    arrays[f"{key}/floor"] = np.array([floor[f] for f in FIELDS])
    r32, r64 = arrays[f"{key}/rec32"].astype(np.float64), arrays[f"{key}/rec64"]
    rec_floor = float(np.linalg.norm(r32 - r64) / max(np.linalg.norm(r64), 1e-300))
    meta[key] = {"steps": steps, "domains": s64.n_domains, "receivers": s64.n_receivers,
                 "rec_f32_vs_f64": rec_floor, "field_f32_vs_f64": floor,
                 "oracle_seconds": round(time.time() - t0, 1)}
    print(f"  {key}: receivers f32 vs f64 {rec_floor:.3e}; fields {floor}", flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="batch,lshape,large")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 8)
    args = ap.parse_args()
    oracle.build()
    for name, items in cases(args.only.split(",")):
        arrays, meta = {}, {}
        print(f"{name}: {len(items)} scene(s)", flush=True)
        for key, conf, steps, stride in items:
            run_scene(key, conf, steps, stride, args.threads, arrays, meta)
        arrays["meta"] = np.frombuffer(json.dumps(meta, sort_keys=True).encode(), dtype=np.uint8)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **arrays)
        print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB)", flush=True)


if __name__ == "__main__":
    main()
