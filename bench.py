"""Throughput of the GB300 PSTD solve (Gcell-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                   [--workload lshape|square|square1200|rect8192|large|batch|serve]

Workload (default ``lshape``): the multi-domain L-shaped scene -- 1200x600,
600x600 and 600x1200 air cells (dx = 0.2 m) with a seeded mix of rigid and
alpha = 0.3 + 50-cell-PML outer edges, 4 speakers, 16 receivers (seeded
synthetic scene; the reference publishes no scenes).  A step is one full PSTD
time step (6 RK stages) of the whole scene; the unit of work is one pressure
cell of a non-rigid domain advanced one step.

* ``value``: device-resident throughput: K timed steps launched with
  ``pstd_advance`` on a CUDA stream, each timed with CUDA events on it and
  preceded by a 256 MiB write that evicts L2 (the L-shape's state is about the
  size of L2), so every timed step reads its fields from HBM.
* ``receiver_err``: the same scene solved for all 4000 steps on the GPU and
  compared with the committed oracle fixture (float = the reference's CPU
  path restated, and FP64), relative L2 of the 16 receiver series.
* ``e2e``: the same metric through the reference-facing API: a 1000-step
  scene through ``PSTDKernel.run`` with every frame of p0 and every receiver
  sample delivered to host callbacks (SaveNth = 1), host<->device copies in
  the timed region; ``initialize_kernel`` (scene build, upload, plan) is timed
  apart and reported as ``init_s``.
* ``roofline``: the stage kernels (every strip-length bucket of an RK stage),
  48 algorithmic bytes per cell and RK stage (read px,py,vx,vy + the
  stage-start px,py,vx,vy, write px,py,vx,vy), over their CUDA-event time
  measured in a second timed region with events around every stage launch.
* ``batched``: the batched workload -- 256 scenes (total size log-uniform
  64x64..1024x768 cells, 1-6 rectangles) advanced together -- against the
  plain path solving the same scenes one at a time, with its receiver error on
  the 8 fixture scenes of that workload (2000 steps).
* ``cpu_baseline``: the CPU restatement of the reference solver (oracle/),
  OpenMP over all host cores, on a bounded sample of the same scene, with the
  speed of its own FFT set beside scipy's pocketfft on the same strip shapes
  (the reference links FFTW, which is absent here).

``--impl reference`` times the reference's CPU algorithm (the oracle port; the
reference itself cannot be built: Eigen, FFTW3f, Boost and Qt5 are absent) on
the same scene with all host threads; under torchrun only rank 0 runs it.
Multi-GPU runs are replicas: every rank solves its own scene (seed = rank),
no collective on the data path; value = all ranks' cells x steps / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 126 * 1024 * 1024
FLUSH_BYTES = 256 * 1024 * 1024     # written before every timed step: evicts L2
BYTES_PER_CELL_STAGE = 48
METRIC = "Gcell-steps/s"


def workload(name: str, seed: int):
    from openpstd_gb300 import scenes
    if name == "lshape":
        return scenes.l_shape(seed, steps=4000), ("L-shape 1200x600+600x600+600x1200 cells, dx 0.2 m, mixed rigid / "
                                                  "alpha 0.3 + 50-cell PML edges, 4 speakers, 16 receivers")
    if name == "square":
        return scenes.plain_square(seed), "square 200x200 cells + 50-cell PML, 1 speaker, 4 receivers"
    if name == "square1200":
        from openpstd_gb300.config import PSTDConfiguration
        conf = PSTDConfiguration()
        scenes.base_settings(conf, 1000, dx=0.2, pml=50)
        conf.Domains = [scenes._domain(0, 0, 1200, 1200, 0.2, dict(left=0.0, right=0.0, top=0.0, bottom=0.0))]
        conf.Speakers = [(120.05, 130.05, 0.0)]
        conf.Receivers = [(200.05, 150.05, 0.0)]
        return conf, "square 1200x1200 cells, rigid edges (transform length 2048 only), 1 speaker, 1 receiver"
    if name == "rect8192":
        return scenes.rect(6 + seed, nx=4100, ny=1200, steps=1000), (
            "rectangle 4100x1200 cells + 50-cell PML (transform length 8192 along x), 1 speaker, 2 receivers")
    if name == "large":
        return scenes.large_square(seed, half=4096, steps=1000), (
            "8192x8192 cells as 2x2 domains of 4096x4096 with windowed interfaces, 50-cell PML (alpha 1) on the "
            "outer edges, 2 speakers, 64 receivers")
    raise SystemExit(f"unknown workload {name}")


def replica_totals(ms: float, cells: float, dist, device: str = "cuda"):
    """Whole-job numbers of a replicas run: the slowest rank's time and the
    cells of all ranks (every rank solves its own scene; no data-path
    collective)."""
    if dist is None:
        return ms, float(cells)
    import torch
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(cells)], device=device, dtype=torch.float64)
    dist.all_reduce(c)
    return float(t.item()), float(c.item())


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    backend = "nccl"
    dist.init_process_group(backend=backend)
    return rank, ws, dist


class ClockSampler:
    """nvidia-smi samples (200 ms) over the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9 and p[1].replace(".", "").isdigit():
                    rows.append(p)
        finally:
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit())}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_cell_stage():
    """DRAM bytes per cell and RK stage of the stage kernels from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")
    if not os.path.exists(path):
        return None, None
    d = json.load(open(path))
    return d.get("dram_bytes_per_cell_stage"), d.get("case")


def rel(a, b):
    import numpy as np
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    n = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b) / (n if n > 0 else 1.0))


def fixture(name):
    """Committed oracle fixture tests/golden/<name>.npz (float and FP64 oracle), or None."""
    import numpy as np
    path = os.path.join(ROOT, "tests", "golden", f"{name}.npz")
    return np.load(path) if os.path.exists(path) else None


def parity_case(workload: str):
    """(fixture key, scene factory, description) of the full-size oracle
    fixture that belongs to a workload, or None."""
    from openpstd_gb300 import scenes
    if workload == "lshape":
        return "lshape", lambda: scenes.l_shape(0, steps=4000), "the benchmarked scene, all 4000 steps"
    if workload == "large":
        return ("large", lambda: scenes.large_square(0, half=4096, steps=60, receivers_near=(1.0, 3.0)),
                "the 8192^2 scene with its 64 receivers 1-3 m from the speakers, 60 steps")
    return None


def dft_form():
    return {"tf32x3": "split-TF32 tcgen05 DFT (precision study, L=8192 strips)",
            "bf16x3": "split-BF16 mma.sync DFT (precision study, L=4096/8192 strips)"}.get(
        os.environ.get("PSTD_DFT", ""), "FP32 FFT")


def receiver_error(got, fx, key):
    """Relative L2 of GPU receiver series against the fixture's float and FP64 oracle."""
    r32, r64 = fx[f"{key}/rec32"], fx[f"{key}/rec64"]
    return {"vs_f32_oracle": rel(got, r32), "vs_f64_oracle": rel(got, r64), "f32_oracle_vs_f64": rel(r32, r64)}


def fft_speed(threads: int):
    """The oracle's strip transform (r2c, multiply, c2r) against scipy's
    pocketfft on the same shapes: 2048-point strips, as the L-shape's
    1200-cell strips use."""
    import numpy as np
    from oracle import oracle
    try:
        import scipy.fft as sf
    except ImportError:
        return None
    L, n = 2048, 2048
    t_or = oracle.fft_seconds(L, n, threads, 3)
    x = np.random.default_rng(0).random((n, L), dtype=np.float32)
    f = np.full(L // 2 + 1, 0.5 + 0.25j, dtype=np.complex64)
    best = 1e30
    for _ in range(3):
        t0 = time.perf_counter()
        sf.irfft(sf.rfft(x, axis=1, workers=threads) * f, n=L, axis=1, workers=threads)
        best = min(best, time.perf_counter() - t0)
    return {"shape": f"{n} strips x {L} points, r2c + multiply + c2r", "threads": threads,
            "oracle_ms": t_or * 1e3, "pocketfft_ms": best * 1e3, "oracle_over_pocketfft": t_or / best}


def cpu_rate(conf, seconds: float, threads: int):
    """Gcell-steps/s of the oracle port on a bounded sample (whole steps, >= 1)."""
    from oracle import oracle
    oracle.build()
    s = oracle.OracleScene(conf, 32)
    cells = sum(s.domain_info(i)["size"][0] * s.domain_info(i)["size"][1]
                for i in range(s.n_domains) if not s.domain_info(i)["is_rigid"])
    s.run(1, threads=threads)   # warm-up (plans, caches)
    steps, t0 = 0, time.perf_counter()
    while True:
        s.run(1, threads=threads)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return cells * steps / el / 1e9, steps, el, cells


def batch_leg(args, stream):
    """Batched workload: n independent scenes (total size log-uniform in
    64x64 .. 1024x768 cells, 1-6 rectangles, edge alpha ~ U[0,1]) advanced
    together, against the plain path solving the same scenes one at a time,
    plus the receiver error of the 8 fixture scenes of this workload advanced
    together for 2000 steps."""
    import numpy as np
    import torch
    from openpstd_gb300 import scenes
    from openpstd_gb300.batch import BatchKernel
    from openpstd_gb300 import kernel
    confs = scenes.batch_scenes(0, n=args.batch_scenes, steps=2000)
    t0 = time.perf_counter()
    b = BatchKernel(confs)
    t_create = time.perf_counter() - t0
    cells = b.work_counts()["cells"]
    sh = stream.cuda_stream
    b.advance(args.warmup, sh)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    bsteps = max(3, min(args.steps, args.batch_steps))
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        b.advance(bsteps, sh)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    batched = cells * bsteps / (ms / 1e3) / 1e9
    plan = b.plan_info().strip().splitlines()
    b.close()
    # plain path: one scene at a time (device-resident, same step count each)
    plain_steps = max(3, min(bsteps, args.plain_steps))
    tot_ms, tot_cells = 0.0, 0
    t0 = time.perf_counter()
    for c in confs:
        k = kernel.PSTDKernel()
        k.initialize_kernel(c)
        k.advance(args.warmup, sh)
        torch.cuda.synchronize()
        e0.record(stream)
        k.advance(plain_steps, sh)
        e1.record(stream)
        torch.cuda.synchronize()
        tot_ms += e0.elapsed_time(e1)
        tot_cells += k.work_counts()["cells"] * plain_steps
        k.close()
    t_plain = time.perf_counter() - t0
    plain = tot_cells / (tot_ms / 1e3) / 1e9
    out = {"value": batched, "unit": METRIC, "steps": bsteps, "ms_per_step": ms / bsteps,
           "workload": f"batch of {len(confs)} scenes, total size log-uniform 64x64..1024x768 cells, 1-6 rectangles "
                       "each, edge alpha U[0,1], 1-4 speakers, 1-8 receivers",
           "cells_per_step": cells, "create_s": t_create,
           "plain_serial": {"value": plain, "unit": METRIC, "steps_per_scene": plain_steps, "wall_s": t_plain,
                            "note": "the same scenes solved one at a time with the plain path"},
           "batched_over_plain": batched / plain, "plan": plan, "clocks": clk.summary()}
    fx = fixture("batch")
    if fx is not None:
        keys = sorted({k.split("/")[0] for k in fx.files if k.startswith("b") and k.endswith("/rec64")},
                      key=lambda x: int(x[1:]))
        bf = BatchKernel([confs[int(k[1:])] for k in keys])
        bf.advance(2000, sh)
        bf.synchronize()
        got = np.concatenate([bf.receivers(scene=i).astype(np.float64) for i in range(len(keys))], axis=1)
        bf.close()
        r32 = np.concatenate([fx[f"{k}/rec32"] for k in keys], axis=1)
        r64 = np.concatenate([fx[f"{k}/rec64"] for k in keys], axis=1)
        out["receiver_err"] = {"scenes": [int(k[1:]) for k in keys], "steps": 2000, "vs_f32_oracle": rel(got, r32),
                               "vs_f64_oracle": rel(got, r64), "f32_oracle_vs_f64": rel(r32, r64),
                               "tolerance": 1e-5}
    return out


def run_batch(args):
    import torch
    from openpstd_gb300 import build as _b
    _b.build()
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    bl = batch_leg(args, stream)
    line = {"metric": METRIC, "value": bl["value"], "unit": METRIC, "n_gpus": 1, "steps": bl["steps"],
            "warmup": args.warmup, "ms_per_step": bl["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes)",
            "config": {"workload": bl["workload"], "cells_per_step": bl["cells_per_step"], "create_s": bl["create_s"],
                       "l2": "no flush: 256 scenes of state (several GB) exceed L2"},
            "plain_serial": bl["plain_serial"], "batched_over_plain": bl["batched_over_plain"],
            "receiver_err": bl.get("receiver_err"), "plan": bl["plan"], "clocks": bl["clocks"]}
    print(json.dumps(line), flush=True)


def request_cells(conf) -> int:
    """Non-rigid cells of a scene, PML domains included: the work of one of
    its steps in the unit the server counts (scene built on the host)."""
    import ctypes
    from openpstd_gb300 import _lib
    from openpstd_gb300.config import CConfig, c_domain_info
    cc, h = CConfig(conf), ctypes.c_void_p()
    _lib.check(_lib.lib().pstd_scene_build(ctypes.byref(cc.c), ctypes.byref(h)))
    try:
        n, total = ctypes.c_int32(), 0
        _lib.check(_lib.lib().pstd_scene_domain_count(h, ctypes.byref(n)))
        for i in range(n.value):
            d = c_domain_info()
            _lib.check(_lib.lib().pstd_scene_domain_info(h, i, ctypes.byref(d)))
            if not d.is_rigid:
                total += d.size[0] * d.size[1]
        return total
    finally:
        _lib.lib().pstd_destroy(h)


TICK_SECONDS = 0.25


def serve_leg(reqs, duration, budget, tick_steps):
    """Feed a request stream (arrival time, scene) to a fresh server for
    `duration` seconds of wall clock; latency = completion - arrival.  Ticks
    are sized to about TICK_SECONDS of wall clock (at most tick_steps steps),
    so that arrivals are admitted within that time however large the batch."""
    from openpstd_gb300.serving import Server
    work = [request_cells(c) * c.Settings.framecount() for _, c in reqs]   # built before the clock starts
    srv = Server(budget, max_scenes=4096)
    pending, live, offered, steps = 0, {}, 0, tick_steps
    lat, occ = [], []
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        if now >= duration:
            break
        while pending < len(reqs) and reqs[pending][0] <= now:
            at, conf = reqs[pending]
            rid = srv.submit(conf, conf.Settings.framecount())
            offered += work[pending]
            live[rid] = at
            pending += 1
        t_tick = time.perf_counter()
        info = srv.tick(steps)
        if info["steps"]:
            # next tick: about TICK_SECONDS of wall clock, at most tick_steps steps
            per_step = (time.perf_counter() - t_tick) / info["steps"]
            steps = max(1, min(tick_steps, int(TICK_SECONDS / max(per_step, 1e-6))))
        occ.append(srv.stats()["bytes_in_use"])
        if info["finished"]:
            t_done = time.perf_counter() - t0
            for rid in list(live):
                if srv.poll(rid)["state"] == 2:
                    lat.append(t_done - live.pop(rid))
                    srv.result(rid)
        if info["active"] == 0 and info["queued"] == 0 and pending < len(reqs):
            time.sleep(max(0.0, min(reqs[pending][0] - (time.perf_counter() - t0), 0.01)))
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat_s = sorted(lat)
    pct = (lambda q: lat_s[min(len(lat_s) - 1, int(q * len(lat_s)))] if lat_s else None)
    return {"served": st["cell_steps"] / wall / 1e9, "offered": offered / wall / 1e9,
            "latency_s": {"p50": pct(0.5), "p99": pct(0.99), "completed": len(lat)},
            "requests": {"arrived": pending, "completed": st["done"], "active_at_end": st["active"],
                         "queued_at_end": st["queued"]},
            "hbm": {"budget_bytes": budget, "peak_bytes_in_use": st["peak_bytes"],
                    "mean_occupancy": (sum(occ) / len(occ) / budget) if occ else 0.0},
            "launch_form": {"persistent": st["persistent"], "graph_captures": st["graph_captures"],
                            "in_place_table_updates": st["table_updates"], "launches_per_step": st["launches_per_step"],
                            "membership_changes": st["rebuilds"]}}


def run_serve(args):
    """Serving workload: Poisson arrivals (mean --rate per second) of
    batch-like scenes with step counts log-uniform 200..8000, served by the
    continuous-batching loop under an HBM budget for --duration seconds of
    wall clock.  When that stream is more than the GPU sustains, the served
    throughput is the server's capacity; capacity / mean work per request is
    the highest sustainable arrival rate, and a second leg at 80 % of it
    (--sustain-duration seconds) reports the latency of a stream the server
    keeps up with.  Beside them, the plain path solving a sample of the same
    requests one at a time (create + steps)."""
    import torch
    from openpstd_gb300 import build as _b, scenes
    from openpstd_gb300 import kernel
    _b.build()
    torch.cuda.set_device(0)
    budget = int(args.budget_gb * (1 << 30))
    reqs = scenes.serving_requests(0, rate_hz=args.rate, duration_s=args.duration)
    with ClockSampler(0) as clk:
        main = serve_leg(reqs, args.duration, budget, args.tick_steps)
    # mean work of a request of this mix (cell-steps), from a large sample of the generator
    sample = scenes.serving_requests(7, rate_hz=100.0, duration_s=20.0)
    mean_work = sum(request_cells(c) * c.Settings.framecount() for _, c in sample) / len(sample)
    saturated = main["offered"] > 1.05 * main["served"]
    sustain = None
    if saturated and args.sustain_duration > 0:
        r_max = main["served"] * 1e9 / mean_work
        r = 0.8 * r_max
        leg = serve_leg(scenes.serving_requests(1, rate_hz=r, duration_s=args.sustain_duration),
                        args.sustain_duration, budget, args.tick_steps)
        sustain = {"max_sustainable_rate_hz": r_max, "rate_hz": r, **leg}
    # plain path, one request at a time (create + all its steps), on a sample
    t_plain, cs_plain, n_plain = 0.0, 0, 0
    for at, conf in reqs[: args.plain_requests]:
        t1 = time.perf_counter()
        k = kernel.PSTDKernel()
        k.initialize_kernel(conf)
        n = conf.Settings.framecount()
        k.advance(n)
        k.synchronize()
        t_plain += time.perf_counter() - t1
        cs_plain += k.work_counts()["cells"] * n
        n_plain += 1
        k.close()
        if t_plain > args.plain_seconds:
            break
    plain = cs_plain / t_plain / 1e9
    served = main["served"]
    line = {"metric": METRIC, "value": served, "unit": METRIC, "n_gpus": 1, "steps": None, "warmup": 0,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Poisson request stream)",
            "config": {"workload": f"serving: Poisson {args.rate}/s of batch-like scenes (64x64..1024x768 cells, "
                                   "1-6 rectangles), steps log-uniform 200..8000, HBM budget "
                                   f"{args.budget_gb} GB, {args.duration} s wall clock",
                       "tick_steps": args.tick_steps},
            "offered": main["offered"], "saturated": saturated,
            "latency_s": main["latency_s"], "requests": main["requests"], "hbm": main["hbm"],
            "launch_form": main["launch_form"], "mean_request_cell_steps": mean_work,
            "sustained": sustain,
            "plain_serial": {"value": plain, "unit": METRIC, "requests": n_plain,
                             "note": "the first requests solved one at a time with the plain path (create + steps)"},
            "served_over_plain": served / plain if plain else None, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_reference(args):
    # the reference's CPU path runs once, on rank 0; other ranks leave at once
    # (no process group: nothing is exchanged)
    rank, ws = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from oracle import oracle
    conf, desc = workload(args.workload, 0)
    threads = os.cpu_count() or 1
    # W warm-up steps are folded into one untimed step; K steps are timed,
    # capped at ~90 s of host time (the rate is per step, so the cap only
    # bounds the sample)
    oracle.build()
    s = oracle.OracleScene(conf, 32)
    cells = sum(s.domain_info(i)["size"][0] * s.domain_info(i)["size"][1]
                for i in range(s.n_domains) if not s.domain_info(i)["is_rigid"])
    for _ in range(min(args.warmup, 1)):
        s.run(1, threads=threads)
    done, t0 = 0, time.perf_counter()
    while done < args.steps:
        s.run(1, threads=threads)
        done += 1
        if time.perf_counter() - t0 > 90:
            break
    el = time.perf_counter() - t0
    v = cells * done / el / 1e9
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": ws, "steps": done, "warmup": args.warmup,
            "ms_per_step": el * 1e3 / done, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded scene)", "impl": "reference",
            "config": {"workload": desc, "cells_per_step": cells, "steps_requested": args.steps},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{done} time steps of the workload (capped at 90 s)",
                             "fft_speed": fft_speed(threads)},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes
    import numpy as np
    import torch
    rank, ws, dist = dist_setup()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from openpstd_gb300 import build as _b
    _b.build()
    from openpstd_gb300 import kernel
    conf, desc = workload(args.workload, rank)
    k = kernel.PSTDKernel()
    k.initialize_kernel(conf)
    wc = k.work_counts()
    cells = wc["cells"]
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def barrier():
        if dist:
            dist.barrier()

    # ---- device-resident timed region: every timed step follows a write of
    # FLUSH_BYTES on the same stream (outside its events) that evicts L2
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    k.advance(args.warmup, sh)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for i, (a, b) in enumerate(evs):
                flush.fill_(float(i & 7))
                a.record(stream)
                k.advance(1, sh)
                b.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    clocks = clk.summary()
    del flush
    ms, total_cells = replica_totals(ms, cells, dist)
    value = total_cells * args.steps / (ms / 1e3) / 1e9

    # ---- pass-kernel timing (events around every pass launch)
    prof_steps = max(3, min(args.steps, 200))
    torch.cuda.synchronize()
    prof = k.profile_passes(prof_steps, sh)
    stage_ms = prof["ms_stage"]
    launches = prof["stage_launches"]
    alg_bytes = cells * BYTES_PER_CELL_STAGE * 6 * prof_steps
    peak, peak_kind = peaks()
    achieved = alg_bytes / (stage_ms / 1e3) / 1e9
    tpcs, tcase = traffic_per_cell_stage()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (tpcs * cells * 6 * prof_steps / launches) if tpcs else None,
                "kernel": "stage_kernel<L,...> (all strip-length buckets of an RK stage)",
                "algorithmic_bytes_per_launch": alg_bytes / launches, "launches": launches,
                "avg_launch_us": stage_ms * 1e3 / launches, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic_source": tcase, "stage_share_of_step": stage_ms / prof["ms_total"],
                "plan": k.plan_info().strip().splitlines()}

    # ---- receiver error: the workload's full-size solve against its committed oracle fixture
    rec_err = None
    parity = parity_case(args.workload)
    fx = fixture(parity[0]) if parity and rank == 0 and not args.no_parity else None
    if fx is not None:
        kp = kernel.PSTDKernel()
        kp.initialize_kernel(parity[1]())
        nsteps = int(fx[f"{parity[0]}/rec64"].shape[0])
        kp.advance(nsteps, sh)
        kp.synchronize()
        rec_err = dict(receiver_error(kp.receivers(), fx, parity[0]), steps=nsteps, tolerance=1e-5,
                       scene=parity[2])
        kp.close()

    # ---- end-to-end through the reference-facing API (host callbacks)
    e2e_steps = max(5, min(args.e2e_steps, int(2e9 // cells)))   # every frame goes to the host
    ce = conf.copy()
    dt = ce.Settings.GetTimeStep()
    ce.Settings.SetRenderTime(float(np.float32((e2e_steps + 0.5) * float(dt))))
    assert ce.Settings.framecount() == e2e_steps
    sizes = {"frame_bytes": 0, "sample_bytes": 0}

    class Sink(kernel.KernelCallback):
        def WriteFrame(self, frame, domain, data):
            sizes["frame_bytes"] += data.nbytes

        def WriteSample(self, start, receiver, data):
            sizes["sample_bytes"] += 4 * len(data)

    # untimed warm-up of the same path (first frame buffers, callback bridge)
    cw = conf.copy()
    cw.Settings.SetRenderTime(float(np.float32(10.5 * float(dt))))
    kw = kernel.PSTDKernel()
    kw.initialize_kernel(cw)
    class Drop(kernel.KernelCallback):
        def WriteFrame(self, frame, domain, data):
            pass

        def WriteSample(self, start, receiver, data):
            pass

    kw.run(Drop())
    kw.close()
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ke = kernel.PSTDKernel()
    ke.initialize_kernel(ce)
    torch.cuda.synchronize()
    init_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ke.run(Sink())
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    cfg_bytes = sum(ctypes.sizeof(x) for x in (ke._cc.c,)) + 40 * len(ce.Domains) + 12 * (len(ce.Speakers) + len(ce.Receivers))
    ke.close()
    e2e_s, _ = replica_totals(e2e_s, 0.0, dist)
    e2e = {"value": total_cells * e2e_steps / e2e_s / 1e9, "unit": METRIC,
           "h2d_bytes_per_step": cfg_bytes / e2e_steps,
           "d2h_bytes_per_step": (sizes["frame_bytes"] + sizes["sample_bytes"]) / e2e_steps,
           "steps": e2e_steps, "init_s": init_s,
           "with_init": total_cells * e2e_steps / (e2e_s + init_s) / 1e9,
           "path": "PSTDKernel.run(WriteFrame every frame, WriteSample), after initialize_kernel (timed apart: init_s)"}

    batched = batch_leg(args, stream) if (args.workload == "lshape" and ws == 1 and not args.no_batch) else None
    if rank != 0:
        return
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene, no published scene exists)",
            "config": {"workload": desc, "cells_per_step_per_gpu": cells, "air_cells": wc["air_cells"],
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                       "l2": f"flushed: a {FLUSH_BYTES >> 20} MiB write before every timed step (outside its events)",
                       "cuda_graphs": "one graph per time step (3-phase set rotation)", "dft": dft_form()},
            "receiver_err": rec_err, "roofline": roofline, "e2e": e2e, "clocks": clocks,
            "gpu_launches": wc["launches_per_step"] * args.steps}
    if batched is not None:
        line["batched"] = batched
    if ws == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, steps, el, ccells = cpu_rate(conf, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": v, "unit": METRIC, "cores": threads, "kind": "port",
                                "sample": f"{steps} time steps of the same scene in {el:.1f} s (oracle, OpenMP)",
                                "fft_speed": fft_speed(threads)}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="lshape")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--batch-steps", type=int, default=200, help="timed steps of the batched leg")
    ap.add_argument("--e2e-steps", type=int, default=1000, help="steps of the end-to-end leg")
    ap.add_argument("--no-batch", action="store_true", help="leave the batched leg out of the default line")
    ap.add_argument("--no-parity", action="store_true", help="leave the 4000-step receiver check out")
    ap.add_argument("--rate", type=float, default=50.0, help="serve: mean request arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of wall clock")
    ap.add_argument("--budget-gb", type=float, default=80.0, help="serve: HBM budget")
    ap.add_argument("--tick-steps", type=int, default=64, help="serve: most steps per tick")
    ap.add_argument("--sustain-duration", type=float, default=60.0,
                    help="serve: seconds of the leg at 80 %% of the highest sustainable rate (0: skip)")
    ap.add_argument("--plain-requests", type=int, default=40)
    ap.add_argument("--plain-seconds", type=float, default=20.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
