"""Benchmark: uniform-grid rebuild + 3D-DDA trace on one GB300.

Default run (one JSON line, rank 0):

* headline -- deforming-mesh per-frame rebuild.  One "step" = one frame: a
  160 x 320 x 2 = 102,400-triangle UV sphere (pole caps open) whose 51,520
  vertices are displaced on the device by 0.05*sin(3*p.x + 0.3*frame) along
  their normals; full uniform-grid rebuild at k = 4 cells per triangle (k = 2
  and 8 in `per_k`); 1024 x 1024 primary camera rays and one shadow ray per
  lit-facing hit, traced as any-hit.  Frames cycle through 20 phases.
  `value` = (primary + shadow rays) / frame time, device-timed with CUDA
  events on the scene's stream, inputs resident.  Two frames are in flight:
  frames 2j and 2j + 1 each deform, rebuild and trace their own scene (two
  scenes of the mesh) on their own streams, replayed from one CUDA graph a
  pair, the L2 flushed before each pair; `one_frame_in_flight` is the same
  frames one graph a frame on one scene.  `e2e` = the same frames through
  the public C ABI with host buffers (keyframes from pinned host memory,
  hits and occlusion copied back every frame, frames alternating over the
  two scenes), host-clocked.  `cpu_baseline` = the oracle restatement
  of the reference's CPU path on the host cores (single-thread build, every
  ray in 16 x 16 tiles).
* `cfg0_plain` -- 65,536-triangle plane + debris scene, 512 x 512 rays and
  their shadow rays, build + trace per step, with the CPU path timed beside it.
* `cfg2_skewed` -- 1,048,576 triangles of skewed density, 1024 x 1024 primary
  rays + one diffuse secondary ray per hit, build included; FP64 errors.
* `cfg3_batched` -- 64 uneven scenes built and traced in one graph-captured
  batch vs 64 sequential per-scene calls.
* `cfg4_serving` -- 16 resident scenes, requests served by continuous
  batching vs one at a time: saturation throughput and p50/p99 latency, and
  latency at 1,000 requests/s.

`--workload X` runs one workload alone and prints its full result (also
`instances`: two-level instancing; `render`: the shading wavefront;
`ingest`: OBJ and binary PLY read with the reference loaders' rules, then
uploaded and built); `--detail PATH` writes every workload's full result to
PATH.

--impl reference times the reference's CPU path (the oracle restatement of
UniformGridAccStructBuilder + UniformGridAccStruct, compiled here) on the
host cores, every ray of the headline workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "grid-rt_gb300"))

from gridrt import scenes  # noqa: E402

FRAMES = 20
LAMBDAS = (2, 4, 8)
HEADLINE_K = 4          # cells per triangle of the headline line (and of the CPU arms)
WIDTH = HEIGHT = 1024
METRIC = "Mrays/s (primary + shadow, per-frame rebuild included)"
WORKLOAD = "deforming_sphere_102400tri_1024x1024_shadow"


def _peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while the
    timed regions run; only samples whose timestamp falls inside a timed
    window (mark()/unmark()) are summarised."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.windows = []
        self._t0 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t_end = time.time() + 5.0
            while not self.lines and time.time() < t_end:   # wait for the first sample
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        import datetime
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except Exception:
                ts = time.time()
            self.lines.append((ts, parts))

    def mark(self):
        self._t0 = time.time()

    def unmark(self):
        if self._t0 is not None:
            self.windows.append((self._t0, time.time()))
            self._t0 = None

    def stop(self):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons, n = [], 0.0, set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, parts in self.lines:
            if len(parts) < 9 or not any(a - 0.05 <= ts <= b + 0.05 for a, b in self.windows):
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            n += 1
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": n}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl"
    try:
        import torch
        if not torch.cuda.is_available():
            backend = "gloo"
        else:
            torch.cuda.set_device(local)
    except Exception:
        backend = "gloo"
    dist.init_process_group(backend=backend)
    return rank, ws, local, dist


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(x: float, dist) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _sum_over_ranks(x: float, dist) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement of the reference path), bounded sample
# ---------------------------------------------------------------------------
def cpu_frame_sample(k: int, frame: int, sample_stride: int, nthreads: int = 0):
    """Build the frame's grid single-threaded (the reference's build is), trace
    every `sample_stride`-th primary ray (in 16 x 16 pixel tiles) plus the
    shadow rays of those hits on all host threads; extrapolate to the full
    frame."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    sc = scenes.deforming_sphere(frame)
    t0 = time.perf_counter()
    g = pyoracle.Grid(sc.verts, sc.idx, k)
    t_build = time.perf_counter() - t0
    cam = scenes.deforming_sphere_camera(WIDTH, HEIGHT)
    # 16 x 16 pixel tiles, one per OpenMP chunk (TiledRenderer's schedule,
    # src/rtplugins/TiledRenderer.cpp:19-27)
    rays = scenes.camera_rays(cam)[_tile_order(WIDTH, HEIGHT)][::sample_stride]
    t0 = time.perf_counter()
    h = g.trace_closest(rays, nthreads=nthreads)
    t_prim = time.perf_counter() - t0
    sr = _host_shadow_rays(sc, rays, h, scenes.SPHERE_LIGHT)
    t0 = time.perf_counter()
    g.trace_any(sr, nthreads=nthreads)
    t_shadow = time.perf_counter() - t0
    n_prim = WIDTH * HEIGHT
    n_shadow = sr.shape[0] * sample_stride
    t_frame = t_build + (t_prim + t_shadow) * sample_stride
    return dict(t_build=t_build, t_frame=t_frame, rays=n_prim + n_shadow, sampled=rays.shape[0] + sr.shape[0],
                threads=pyoracle.max_threads() if nthreads <= 0 else nthreads)


def _host_shadow_rays(sc, rays, h, light):
    ok = h["id"] >= 0
    tid = h["id"][ok]
    v0 = sc.verts[sc.idx[tid, 0]].astype(np.float64)
    e1 = sc.verts[sc.idx[tid, 1]] - v0
    e2 = sc.verts[sc.idx[tid, 2]] - v0
    n = np.cross(e1, e2)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    d = rays[ok, 4:7].astype(np.float64)
    flip = (n * d).sum(1) > 0
    n[flip] = -n[flip]
    p = rays[ok, 0:3] + d * h["t"][ok, None] + n * 2e-4
    L = light[None].astype(np.float64) - p
    keep = (n * L).sum(1) > 0
    sr = np.zeros((int(keep.sum()), 8), np.float32)
    sr[:, 0:3] = p[keep]
    sr[:, 3] = 2e-4
    sr[:, 4:7] = L[keep]
    sr[:, 7] = 1.0
    return sr


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    pyoracle.build()
    k = HEADLINE_K
    stride = 1
    for w in range(args.warmup):
        cpu_frame_sample(k, w % FRAMES, stride)
    res = [cpu_frame_sample(k, s % FRAMES, stride) for s in range(args.steps)]
    t = sum(r["t_frame"] for r in res)
    rays = sum(r["rays"] for r in res)
    value = rays / t / 1e6
    cores = res[0]["threads"]
    sample = (f"per frame: single-thread grid build (k={k}) + every 1024^2 primary ray and its shadow ray "
              f"traced on {cores} threads")
    return ({
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * t / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "k": k, "frames": FRAMES},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": sample, "build_ms": round(1e3 * statistics.median(r["t_build"] for r in res), 3)},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
def _pair_ms(torch, stream, stream2, enqueue):
    """Device time of the work `enqueue` puts on two streams: the second
    stream forked from the first before it and joined back after it, CUDA
    events on the first around both."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fork, join = torch.cuda.Event(), torch.cuda.Event()
    e0.record(stream)
    fork.record(stream)
    stream2.wait_event(fork)
    enqueue()
    join.record(stream2)
    stream.wait_event(join)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def run_gpu(args, rank, ws, local, dist):
    import torch
    from gridrt import lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    v, idx, nrm = scenes.sphere_mesh()
    nverts, ntris = v.shape[0], idx.shape[0]
    cam = scenes.deforming_sphere_camera(WIDTH, HEIGHT)
    npix = WIDTH * HEIGHT
    light = scenes.SPHERE_LIGHT

    s = lib.Scene(local)
    s.set_geometry(v, idx)
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    d_base = torch.from_numpy(v).to(dev)
    d_nrm = torch.from_numpy(nrm).to(dev)
    d_hits = torch.empty((npix, 4), dtype=torch.int32, device=dev)
    d_occ = torch.empty(npix, dtype=torch.uint8, device=dev)
    d_sr = torch.empty((npix, 8), dtype=torch.float32, device=dev)
    # a second scene of the same mesh holds the other frame in flight: frames
    # 2j and 2j + 1 each deform, rebuild and trace their own scene, on their
    # own streams, so one frame's launch chain runs beside the other's work
    s2 = lib.Scene(local)
    s2.set_geometry(v, idx)
    stream2 = torch.cuda.ExternalStream(s2.stream, device=dev)
    d_hits2 = torch.empty_like(d_hits)
    d_occ2 = torch.empty_like(d_occ)
    d_sr2 = torch.empty_like(d_sr)
    scene_a = (s, stream, d_hits, d_occ, d_sr)
    scene_b = (s2, stream2, d_hits2, d_occ2, d_sr2)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    fixed = _parse_tuning(args.fixed_tuning)
    if args.profile_frames:
        # profiling run: the fixed tuning's k, a capacity build, then
        # `profile_frames` frames launched call by call (deform, build, frame
        # trace) -- no tuning search, graphs, end-to-end leg or CPU legs, so
        # a profiler's capture ends quickly
        k = fixed["k"] if fixed else HEADLINE_K
        if fixed:
            _apply_tuning(s, fixed)
        s.deform(d_base, d_nrm, 0.05, 3.0, 0.0)
        s.build(k)
        order = fixed["order"] if fixed else "morton8"
        with torch.cuda.stream(stream):
            for f in range(args.profile_frames):
                s.deform(d_base, d_nrm, 0.05, 3.0, 0.3 * f)
                s.build_async(k)
                s.trace_frame_device(cam, light, d_hits, d_occ, d_sr, order=order)
        torch.cuda.synchronize()
        if s.build_check() != 0:
            raise RuntimeError("profiled build failed: " + lib.load().rtg_last_error().decode())
        return None

    # capacities for every frame at every k (synchronous builds, untimed)
    for sc in (s, s2):
        for k in LAMBDAS:
            for f in range(FRAMES):
                sc.deform(d_base, d_nrm, 0.05, 3.0, 0.3 * f)
                sc.build(k)

    def frame(k, f, order, ev=None, on=scene_a):
        sc, st, hits, occ, sr = on
        with torch.cuda.stream(st):
            if ev:
                ev[0].record(st)
            sc.deform(d_base, d_nrm, 0.05, 3.0, 0.3 * f)
            sc.build_async(k)
            if ev:
                ev[1].record(st)
            # primary rays, then each hit's shadow ray (any-hit)
            sc.trace_frame_device(cam, light, hits, occ, sr, order=order)
            if ev:
                ev[2].record(st)
                ev[3].record(st)

    def pair_ms(enqueue):
        return _pair_ms(torch, stream, stream2, enqueue)

    # autotune the trace launch shape and ray order per k (results do not
    # depend on them); each candidate is timed as the headline runs: a pair
    # of frames in flight on the two scenes, after one untimed frame
    from gridrt import autotune

    def tune_k(k):
        def measure(cfg):
            _apply_tuning(s, cfg)
            _apply_tuning(s2, cfg)
            frame(k, 0, cfg["order"])
            return pair_ms(lambda: (frame(k, 1, cfg["order"]), frame(k, 2, cfg["order"], on=scene_b)))
        return autotune.search(measure, reps=3)

    tuned = {}
    per_k = {}
    sampler = ClockSampler(local).start() if rank == 0 else None
    for k in ([fixed["k"]] if fixed else LAMBDAS):
        if fixed:
            best, allres, source = {x: fixed[x] for x in fixed if x != "k"}, [], "fixed"
        else:
            best, allres = tune_k(k)
            source = autotune.search.last_source
        tuned[k] = dict(best=best, all=[(c, round(m, 4)) for c, m in allres], source=source)
        _save_autotune(f"deforming_k{k}", allres)
        order = best["order"]
        _apply_tuning(s, best)
        _apply_tuning(s2, best)
        for w in range(args.warmup):
            frame(k, w % FRAMES, order)
            frame(k, (w + 1) % FRAMES, order, on=scene_b)
        torch.cuda.synchronize()
        if s.build_check() != 0 or s2.build_check() != 0:
            raise RuntimeError("warm-up build failed: " + lib.load().rtg_last_error().decode())
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
        shadow_count = torch.zeros((), dtype=torch.int64, device=dev)
        _barrier(dist)
        torch.cuda.synchronize()
        if sampler:
            sampler.mark()
        lc0 = lib.kernel_launches()
        for st in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()                      # L2 flush between frames (outside the events)
            frame(k, st % FRAMES, order, evs[st])
            with torch.cuda.stream(stream):
                shadow_count += (d_occ != 2).sum()
        lc1 = lib.kernel_launches()
        torch.cuda.synchronize()
        _barrier(dist)
        if sampler:
            sampler.unmark()
        if s.build_check() != 0:
            raise RuntimeError("timed build failed: " + lib.load().rtg_last_error().decode())
        build_ms = [e[0].elapsed_time(e[1]) for e in evs]
        prim_ms = [e[1].elapsed_time(e[2]) for e in evs]   # primary + shadow launches
        shad_ms = [0.0 for e in evs]
        frame_ms = [e[0].elapsed_time(e[3]) for e in evs]
        total_s = _max_over_ranks(sum(frame_ms) / 1e3, dist)
        rays = npix * args.steps + int(shadow_count.item())
        rays_all = _sum_over_ranks(rays, dist)
        # the same frames replayed from CUDA graphs (one per deformation
        # phase, captured on the scene's stream): the library's launches
        # without the host's per-launch cost between the frame's 15 kernels
        graphs = []
        lg0 = lib.kernel_launches()
        for f in range(FRAMES):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                frame(k, f, order)
            graphs.append(g)
        per_frame = (lib.kernel_launches() - lg0) / FRAMES
        torch.cuda.synchronize()
        gevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
        gshadow = torch.zeros((), dtype=torch.int64, device=dev)
        _barrier(dist)
        torch.cuda.synchronize()
        if sampler:
            sampler.mark()
        for st in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                gevs[st][0].record(stream)
                graphs[st % FRAMES].replay()
                gevs[st][1].record(stream)
                gshadow += (d_occ != 2).sum()
        torch.cuda.synchronize()
        _barrier(dist)
        if sampler:
            sampler.unmark()
        if s.build_check() != 0:
            raise RuntimeError("graph-replayed build failed: " + lib.load().rtg_last_error().decode())
        g_s = _max_over_ranks(sum(e[0].elapsed_time(e[1]) for e in gevs) / 1e3, dist)
        g_rays = _sum_over_ranks(npix * args.steps + int(gshadow.item()), dist)
        # two frames in flight: frames 2j and 2j + 1 on the two scenes, forked
        # and joined inside one graph; the K timed frames are K // 2 such
        # pairs (and one single frame when K is odd), the L2 flushed before
        # each
        pairs = []
        for j in range(FRAMES // 2):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                fork = torch.cuda.Event()
                fork.record(stream)
                stream2.wait_event(fork)
                frame(k, 2 * j, order)
                frame(k, 2 * j + 1, order, on=scene_b)
                join = torch.cuda.Event()
                join.record(stream2)
                stream.wait_event(join)
            pairs.append(g)
        torch.cuda.synchronize()
        n_pair = args.steps // 2
        pevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(n_pair + args.steps % 2)]
        pshadow = torch.zeros((), dtype=torch.int64, device=dev)
        _barrier(dist)
        torch.cuda.synchronize()
        if sampler:
            sampler.mark()
        for st in range(len(pevs)):
            with torch.cuda.stream(stream):
                flush.zero_()
                pevs[st][0].record(stream)
                if st < n_pair:
                    pairs[st % (FRAMES // 2)].replay()
                else:
                    graphs[(2 * st) % FRAMES].replay()
                pevs[st][1].record(stream)
                pshadow += (d_occ != 2).sum()
                if st < n_pair:
                    pshadow += (d_occ2 != 2).sum()
        torch.cuda.synchronize()
        _barrier(dist)
        if sampler:
            sampler.unmark()
        if s.build_check() != 0 or s2.build_check() != 0:
            raise RuntimeError("paired build failed: " + lib.load().rtg_last_error().decode())
        p_s = _max_over_ranks(sum(e[0].elapsed_time(e[1]) for e in pevs) / 1e3, dist)
        p_rays = _sum_over_ranks(npix * args.steps + int(pshadow.item()), dist)
        del graphs, pairs
        per_k[k] = dict(tuning=best, value=p_rays / p_s / 1e6, ms_per_step=1e3 * p_s / args.steps,
                        one_in_flight_value=g_rays / g_s / 1e6, one_in_flight_ms=1e3 * g_s / args.steps,
                        launches=int(round(per_frame * args.steps)),
                        stream_value=rays_all / total_s / 1e6, stream_ms_per_step=1e3 * total_s / args.steps,
                        build_ms=statistics.median(build_ms), trace_ms=statistics.median(prim_ms),
                        rays_per_step=rays / args.steps,
                        trace_mrays_s=rays / (sum(prim_ms) + sum(shad_ms)) / 1e3,
                        stream_launches=lc1 - lc0)
    if sampler:
        sampler.stop()

    best_k = HEADLINE_K if HEADLINE_K in per_k else max(per_k, key=lambda kk: per_k[kk]["value"])
    head = per_k[best_k]
    order = head["tuning"]["order"]
    _apply_tuning(s, head["tuning"])

    # roofline of the dominant kernel (primary camera trace): algorithmic bytes
    # from the traversal counters (16 B hit + 8 B per visited cell + 52 B per
    # triangle test: 4 B list entry + 48 B record), camera rays read 0 B
    s.deform(d_base, d_nrm, 0.05, 3.0, 0.0)
    s.build(best_k)
    # counters of the frame's two ray generations: primary rays (camera
    # kernel) and their shadow rays (any-hit over the same shadow rays)
    s.counters(reset=True)
    s.trace_camera_device(cam, d_hits, light=light, d_shadow_rays=d_sr, order=order, counters=True)
    c1 = s.counters(reset=True)
    s.trace_any_device(d_sr, npix, d_occ, counters=True)
    c2 = s.counters(reset=True)
    n_shadow = int((d_sr[:, 7] >= 0).sum().item())
    c = {"rays": c1["rays"] + n_shadow, "cells": c1["cells"] + c2["cells"], "tests": c1["tests"] + c2["tests"]}
    # per camera ray a 16 B hit (the ray itself is generated: 0 B); per
    # shadow ray 24 B in (origin, direction) and 4 B out; 8 B per visited
    # cell (list bounds), 52 B per triangle test (4 B id + 48 B record)
    alg_bytes = 16 * npix + (24 + 4) * n_shadow + 8 * c["cells"] + 52 * c["tests"]
    # the frame's trace launches, averaged (events around the launches alone)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(reps):
            s.trace_frame_device(cam, light, d_hits, d_occ, d_sr, order=order)
        ev1.record(stream)
    torch.cuda.synchronize()
    kern_s = ev0.elapsed_time(ev1) / 1e3 / reps
    peak, peak_kind = _peaks()
    achieved = alg_bytes / kern_s / 1e9
    traffic = _traffic_from_profiles("trace_frame", best_k)
    l2_peak = _l2_read_gbs(dev)
    # build roofline: 12 N index bytes + 12 V vertex bytes + 4 (C + 1) offsets
    # + 4 R ids per build, over the median device-timed build
    gi = s.info()
    build_bytes = 12 * ntris + 12 * nverts + 4 * (gi["ncells"] + 1) + 4 * gi["nrefs"]
    build_s = head["build_ms"] / 1e3

    # e2e through the public C ABI with host buffers
    e2e = run_e2e(args, (s, s2), v, idx, nrm, cam, light, best_k, order, dist)

    if rank != 0:
        return None
    cpu_frames = [cpu_frame_sample(best_k, f, 1) for f in range(0, FRAMES, 2)]   # 10 frames, every ray
    cpu = dict(t_build=statistics.median(c["t_build"] for c in cpu_frames),
               t_frame=sum(c["t_frame"] for c in cpu_frames), rays=sum(c["rays"] for c in cpu_frames),
               threads=cpu_frames[0]["threads"])
    clocks = sampler.summary() if sampler else {}
    out = {
        "metric": METRIC, "value": round(head["value"], 3), "unit": "Mrays/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(head["ms_per_step"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "k": best_k, "ray_order": order, "tuning": head["tuning"], "frames": FRAMES,
                   "triangles": ntris,
                   "rays_primary": npix, "frames_in_flight": 2,
                   "l2": "flushed before every pair of frames in flight (256 MiB write, outside the timed events)",
                   "parallelism": f"replicas x{ws}"},
        "one_frame_in_flight": {"value": round(head["one_in_flight_value"], 3),
                                "ms_per_step": round(head["one_in_flight_ms"], 4),
                                "how": "the same frames replayed one graph a frame on one scene, the L2 flushed "
                                       "before each"},
        "build_ms": round(head["build_ms"], 4), "trace_mrays_s": round(head["trace_mrays_s"], 2),
        "per_k": {str(kk): {x: (round(y, 4) if isinstance(y, float) else y) for x, y in d.items() if x != "tuning"}
                  for kk, d in per_k.items()},
        "autotune": {str(kk): {"candidates": len(v["all"]), "source": v["source"],
                               "best_ms": min((m for _, m in v["all"]), default=None),
                               "worst_ms": max((m for _, m in v["all"]), default=None)} for kk, v in tuned.items()},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "frame trace_kernel (camera rays, then each hit's shadow ray in the same lane) "
                               "with its deferred-ray pass (one frame's trace launches)",
                     "alg_bytes_per_launch": int(alg_bytes),
                     "kernel_ms": round(kern_s * 1e3, 4), "cells": int(c["cells"]), "tests": int(c["tests"]),
                     "l2": {"peak": round(l2_peak, 1), "frac": round(achieved / l2_peak, 4),
                            "peak_source": "measured in this run: rtg_probe_read_gbs over a 32 MiB "
                                           "L2-resident buffer (16-byte loads bypassing L1)"}},
        "build_roofline": {"bound": "hbm", "achieved": round(build_bytes / build_s / 1e9, 1), "peak": peak,
                           "unit": "GB/s", "frac": round(build_bytes / build_s / 1e9 / peak, 4),
                           "alg_bytes": int(build_bytes), "ms": head["build_ms"],
                           "cells": int(gi["ncells"]), "refs": int(gi["nrefs"])},
        "cpu_baseline": {"value": round(cpu["rays"] / cpu["t_frame"] / 1e6, 4), "unit": "Mrays/s",
                         "cores": cpu["threads"], "kind": "port", "nproc": os.cpu_count(),
                         "cpu_model": _cpu_model(),
                         "sample": f"10 of the 20 frames, k={best_k}: single-thread grid build (as the reference "
                                   f"builds) + all 1024^2 primary rays and their shadow rays on {cpu['threads']} "
                                   f"threads; value = rays / (build + trace) time",
                         "build_ms": round(cpu["t_build"] * 1e3, 3)},
        "e2e": e2e,
        "gpu_launches": int(head["launches"]),
        "clocks": {"sm_mhz": clocks.get("sm_mhz"), "sm_max_mhz": clocks.get("sm_max_mhz"),
                   "reasons": clocks.get("reasons", []), "samples": clocks.get("samples", 0)},
    }
    return out


def _l2_read_gbs(dev) -> float:
    """Achievable L2 read bandwidth: the library's read probe over a 32 MiB
    buffer (inside the 126 MiB L2), 16-byte loads that bypass L1."""
    from gridrt import lib
    return lib.probe_read_gbs(dev.index or 0, 32 << 20, 20)


def _cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def _traffic_from_profiles(kernel: str, k: int):
    """DRAM bytes per launch of `kernel` at cells-per-triangle k, from the
    committed ncu summary (profiles/traffic.json), or None when that k was
    not captured."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        e = d.get(kernel, {})
        if int(e.get("k", -1)) != int(k):
            return None
        return e.get("dram_bytes_per_launch")
    except Exception:
        return None


def _save_autotune(name: str, results):
    """The full candidate table of one search, written as
    autotune_<name>.json into the directory GRIDRT_BENCH_OUT names (when it
    is set and exists) instead of into the result line."""
    out_dir = os.environ.get("GRIDRT_BENCH_OUT")
    if not results or not out_dir or not os.path.isdir(out_dir):
        return
    try:
        with open(os.path.join(out_dir, f"autotune_{name}.json"), "w") as f:
            json.dump([{"cfg": c, "ms": round(m, 4)} for c, m in results], f)
    except OSError:
        pass


def run_e2e(args, scs, v, idx, nrm, cam, light, k, order, dist):
    import torch
    from gridrt import lib
    npix = cam.width * cam.height
    host_verts = [torch.from_numpy(scenes.deform(v, nrm, f)).pin_memory() for f in range(FRAMES)]
    hits = [torch.empty((npix, 4), dtype=torch.int32).pin_memory() for _ in range(2)]
    occ = [torch.empty(npix, dtype=torch.uint8).pin_memory() for _ in range(2)]
    nverts = v.shape[0]
    copies = [torch.cuda.Stream() for _ in scs]

    # frame f runs on scene f % 2 (two scenes, the same mesh: two frames in
    # flight on the device, each on its own streams).  A frame builds its
    # keyframe (staged during that scene's previous frame), uploads the
    # scene's next keyframe (f + 2) on a copy stream while it traces, and its
    # hits + occlusion are copied back on the scene's copy stream while the
    # next frame builds and traces; the host waits for frame f's results
    # after enqueuing frame f + 1 (host buffers alternate with the scenes)
    def enqueue(f):
        sc = scs[f % 2]
        sc.build_async(k)
        sc.stage_vertices(host_verts[(f + 2) % FRAMES], nverts, copies[f % 2].cuda_stream)
        return sc, sc.trace_frame_async(cam, light, hits[f % 2], occ[f % 2], order=order)

    def run(first, count):
        prev = None
        for i in range(count):
            t = enqueue((first + i) % FRAMES)
            if prev is not None:
                prev[0].trace_frame_wait(prev[1])
            prev = t
        if prev is not None:
            prev[0].trace_frame_wait(prev[1])

    # shadow rays per frame (deterministic per frame), counted outside the timed loop
    shadow_of = []
    for j, sc in enumerate(scs):
        sc.stage_vertices(host_verts[j], nverts, copies[j].cuda_stream)
    for f in range(FRAMES):
        sc, t = enqueue(f)
        sc.trace_frame_wait(t)
        shadow_of.append(int((occ[f % 2].numpy() != 2).sum()))
    run(0, args.warmup)           # frames 0 and 1's keyframes were staged by the last counted frames
    _barrier(dist)
    t0 = time.perf_counter()
    run(args.warmup, args.steps)
    t = _max_over_ranks(time.perf_counter() - t0, dist)
    if any(sc.build_check() != 0 for sc in scs):
        raise RuntimeError("e2e build failed: " + lib.load().rtg_last_error().decode())
    shadow = sum(shadow_of[(args.warmup + st) % FRAMES] for st in range(args.steps))
    rays = _sum_over_ranks(npix * args.steps + shadow, dist)
    return {"value": round(rays / t / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": int(nverts * 12),
            "d2h_bytes_per_step": int(npix * 17), "ms_per_step": round(1e3 * t / args.steps, 3),
            "how": "host clock over the frame loop, frames alternating over two scenes of the mesh: per frame "
                   "rtg_scene_build_async + rtg_scene_stage_vertices (that scene's next keyframe from pinned host "
                   "memory on a copy stream) + rtg_trace_frame_async (hits and occlusion copied to pinned host "
                   "memory on the scene's copy stream), and rtg_trace_frame_wait for the previous frame's results; "
                   "the clock stops after the last frame's results are on the host"}


# ---------------------------------------------------------------------------
# plain small scene, the case the reference's CPU path runs: 65,536 triangles
# (a 128 x 128-quad ground plane and 32,768 small random triangles), k = 4,
# 512 x 512 primary rays and one shadow ray per lit-facing hit; a step is one
# grid build and the frame trace.  The CPU side is the oracle restatement of
# the reference's path: a single-thread build, then the camera rays in 16 x 16
# pixel tiles, one tile per OpenMP chunk (TiledRenderer's schedule), and the
# shadow rays of their hits.
# ---------------------------------------------------------------------------
def _tile_order(width: int, height: int, tile: int = 16) -> np.ndarray:
    """Scanline ray indices regrouped into tile x tile pixel tiles, row of
    tiles after row of tiles."""
    i = np.arange(width * height).reshape(height // tile, tile, width // tile, tile)
    return i.transpose(0, 2, 1, 3).reshape(-1)


def run_plain_small(args, rank, ws, local, dist):
    import torch
    from gridrt import lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sc = scenes.plane_and_debris()
    cam = scenes.plane_and_debris_camera(512, 512)
    light = scenes.PLANE_LIGHT
    npix = cam.width * cam.height
    k = 4
    s = lib.Scene(local)
    s.set_geometry(sc.verts, sc.idx)
    s.build(k)
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    d_hits = torch.empty((npix, 4), dtype=torch.int32, device=dev)
    d_occ = torch.empty(npix, dtype=torch.uint8, device=dev)
    d_sr = torch.empty((npix, 8), dtype=torch.float32, device=dev)
    # a second scene of the same triangles holds the other step in flight
    s2 = lib.Scene(local)
    s2.set_geometry(sc.verts, sc.idx)
    s2.build(k)
    stream2 = torch.cuda.ExternalStream(s2.stream, device=dev)
    d_occ2 = torch.empty_like(d_occ)
    scene_a = (s, stream, d_hits, d_occ, d_sr)
    scene_b = (s2, stream2, torch.empty_like(d_hits), d_occ2, torch.empty_like(d_sr))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    order = ["morton8"]

    def step(ev=None, on=scene_a):
        g, st, hits, occ, sr = on
        with torch.cuda.stream(st):
            if ev:
                ev[0].record(st)
            g.build_async(k)
            if ev:
                ev[1].record(st)
            g.trace_frame_device(cam, light, hits, occ, sr, order=order[0])
            if ev:
                ev[2].record(st)

    # the autotuner's launch shape and ray order for this step (results do
    # not depend on them), each candidate timed on a pair of steps in flight
    # on the two scenes, after one untimed step
    from gridrt import autotune

    def measure(cfg):
        _apply_tuning(s, cfg)
        _apply_tuning(s2, cfg)
        order[0] = cfg["order"]
        step()
        return _pair_ms(torch, stream, stream2, lambda: (step(), step(on=scene_b)))

    fixed = _parse_tuning(args.fixed_tuning)
    if fixed:
        best, allres, source = {x: fixed[x] for x in fixed if x != "k"}, [], "fixed"
    else:
        best, allres = autotune.search(measure, reps=3)
        source = autotune.search.last_source
    _save_autotune("plain_small", allres)
    _apply_tuning(s, best)
    _apply_tuning(s2, best)
    order[0] = best["order"]
    for _ in range(args.warmup):
        step()
        step(on=scene_b)
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for st in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        step(evs[st])
    torch.cuda.synchronize()
    build_ms = statistics.median(e[0].elapsed_time(e[1]) for e in evs)
    trace_ms = statistics.median(e[1].elapsed_time(e[2]) for e in evs)
    # the same step replayed from a CUDA graph (the headline's form)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        step()
    g.replay()
    torch.cuda.synchronize()
    gevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    for st in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            gevs[st][0].record(stream)
            g.replay()
            gevs[st][1].record(stream)
    torch.cuda.synchronize()
    one_ms = sum(e[0].elapsed_time(e[1]) for e in gevs) / args.steps
    # two steps in flight: one graph holds a step on each scene, forked from
    # and joined back to the first scene's stream; the same K steps as K // 2
    # pairs (and one single step when K is odd), the L2 flushed before each
    gp = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gp, stream=stream):
        fork = torch.cuda.Event()
        fork.record(stream)
        stream2.wait_event(fork)
        step()
        step(on=scene_b)
        join = torch.cuda.Event()
        join.record(stream2)
        stream.wait_event(join)
    gp.replay()
    torch.cuda.synchronize()
    n_pair = args.steps // 2
    pevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(n_pair + args.steps % 2)]
    for st in range(len(pevs)):
        with torch.cuda.stream(stream):
            flush.zero_()
            pevs[st][0].record(stream)
            (gp if st < n_pair else g).replay()
            pevs[st][1].record(stream)
    torch.cuda.synchronize()
    if s.build_check() != 0 or s2.build_check() != 0:
        raise RuntimeError("plain-scene build failed: " + lib.load().rtg_last_error().decode())
    g_ms = sum(e[0].elapsed_time(e[1]) for e in pevs) / args.steps
    nshadow = int((d_occ != 2).sum().item())
    if int((d_occ2 != 2).sum().item()) != nshadow:
        raise RuntimeError("the two scenes' steps disagree")
    rays = npix + nshadow
    del g, gp
    if rank != 0:
        return None
    # CPU: the oracle restatement of the reference's build and trace
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle
    tiles = scenes.camera_rays(cam)[_tile_order(cam.width, cam.height)]
    cpu = []
    for rep in range(4):
        t0 = time.perf_counter()
        grid = pyoracle.Grid(sc.verts, sc.idx, k)
        t1 = time.perf_counter()
        h = grid.trace_closest(tiles)
        t2 = time.perf_counter()
        sr = _host_shadow_rays(sc, tiles, h, light)
        t3 = time.perf_counter()
        grid.trace_any(sr)
        t4 = time.perf_counter()
        if rep:                                   # the first repetition warms the caches
            cpu.append((t1 - t0, (t2 - t1) + (t4 - t3), npix + sr.shape[0]))
    cpu_s = sum(b + t for b, t, _ in cpu) / len(cpu)
    cpu_rays = cpu[0][2]
    return {"workload": "plane_debris_65536tri_512x512_shadow", "k": k, "value": round(rays / g_ms / 1e3, 2),
            "tuning": _tune_str(best), "tuned_by": source,
            "ms_per_step": round(g_ms, 4), "steps_in_flight": 2,
            "one_in_flight": {"value": round(rays / one_ms / 1e3, 2), "ms_per_step": round(one_ms, 4)},
            "build_ms": round(build_ms, 4),
            "trace_ms": round(trace_ms, 4), "rays_per_step": rays, "steps": args.steps,
            "cpu": {"value": round(cpu_rays / cpu_s / 1e6, 3), "ms_per_step": round(1e3 * cpu_s, 3),
                    "build_ms": round(1e3 * statistics.median(b for b, _, _ in cpu), 3),
                    "cores": pyoracle.max_threads(), "kind": "port", "steps": len(cpu)},
            "vs_cpu": round((rays / g_ms / 1e3) / (cpu_rays / cpu_s / 1e6), 1)}


# ---------------------------------------------------------------------------
# batched uneven workload: 64 scenes built + traced in one graph-captured
# batch (build kernels for all scenes, one persistent trace launch) versus 64
# sequential plain per-scene calls (synchronous build + trace launch)
# ---------------------------------------------------------------------------
def run_batched(args, rank, ws, local, dist):
    import torch
    from gridrt import autotune, lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    items = {o: scenes.batched_workload(order=o) for o in ("scanline", "morton8")}
    base = items["scanline"]
    nscenes = len(base)
    tris = sum(it.scene.ntris for it in base)
    d_rays = {o: [torch.from_numpy(it.rays).to(dev) for it in items[o]] for o in items}
    d_hits = [torch.empty((it.rays.shape[0], 4), dtype=torch.int32, device=dev) for it in base]
    rays_total = sum(it.rays.shape[0] for it in base)
    scs = []
    for it in base:
        sc = lib.Scene(local)
        sc.set_geometry(it.scene.verts, it.scene.idx)
        scs.append(sc)
    stream = torch.cuda.Stream(device=dev)
    batches = {}

    def batch_for(k, order):
        key = (k, order)
        if key not in batches:
            tasks = [(i, lib.RTG_MODE_NEAREST, d_rays[order][i], base[i].rays.shape[0], d_hits[i])
                     for i in range(nscenes)]
            batches[key] = lib.Batch(scs, [k] * nscenes, tasks)
        return batches[key]

    def time_batch(b, reps):
        b.build_async(stream.cuda_stream)
        b.trace_async(stream.cuda_stream)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            b.build_async(stream.cuda_stream)
            b.trace_async(stream.cuda_stream)
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                g.replay()
            e1.record(stream)
        torch.cuda.synchronize()
        if b.check(stream.cuda_stream) != 0:
            raise RuntimeError("batched build failed: " + lib.load().rtg_last_error().decode())
        return e0.elapsed_time(e1) / reps, g

    def measure(cfg):
        b = batch_for(cfg["k"], cfg["order"])
        b.set_tuning(empty_run=cfg["empty_run"], persistent=True, refill=cfg["refill"])
        ms, _ = time_batch(b, 2)
        return ms

    space = {"k": (2, 4, 8), "order": ("scanline", "morton8"), "empty_run": (2, 4, 8), "refill": (0, 8)}
    best, allres = autotune.search(measure, space=space, reps=1)
    _save_autotune("batched", allres)
    b = batch_for(best["k"], best["order"])
    b.set_tuning(empty_run=best["empty_run"], persistent=True, refill=best["refill"])
    _barrier(dist)
    batched_ms, graph = time_batch(b, max(3, args.steps // 10))
    batched_ms = _max_over_ranks(batched_ms, dist)

    # plain: per scene, synchronous build then one trace launch, in sequence
    for sc in scs:
        sc.set_tuning(empty_run=best["empty_run"], persistent=True, refill=best["refill"])

    def plain_pass():
        for i, sc in enumerate(scs):
            sc.build(best["k"])
            sc.trace_nearest_device(d_rays[best["order"]][i], base[i].rays.shape[0], d_hits[i])
        torch.cuda.synchronize()

    # breakdown: batched build alone, batched trace alone, plain builds alone,
    # plain traces alone (each timed separately, outside the headline numbers)
    def graph_ms(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        g2 = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g2, stream=stream):
            fn()
        g2.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                g2.replay()
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    breakdown = {"batched_build_ms": graph_ms(lambda: b.build_async(stream.cuda_stream)),
                 "batched_trace_ms": graph_ms(lambda: b.trace_async(stream.cuda_stream))}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for sc in scs:
        sc.build(best["k"])
    breakdown["plain_build_ms"] = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    for i, sc in enumerate(scs):
        sc.trace_nearest_device(d_rays[best["order"]][i], base[i].rays.shape[0], d_hits[i])
    torch.cuda.synchronize()
    breakdown["plain_trace_ms"] = (time.perf_counter() - t0) * 1e3

    for _ in range(args.warmup):
        plain_pass()
    reps = max(3, args.steps // 10)
    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(reps):
        plain_pass()
    plain_ms = _max_over_ranks((time.perf_counter() - t0) * 1e3 / reps, dist)
    if rank != 0:
        return None
    rays_all = rays_total * ws
    return ({
        "metric": "Mrays/s (64-scene batch: build + trace)", "value": round(rays_all / batched_ms / 1e3, 3),
        "unit": "Mrays/s", "n_gpus": ws, "steps": reps, "warmup": args.warmup, "ms_per_step": round(batched_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched_64_scenes", "scenes": nscenes, "triangles": tris, "rays": rays_total,
                   "tuning": best, "l2": "inputs resident; total grid + ray data larger than L2"},
        "plain": {"value": round(rays_all / plain_ms / 1e3, 3), "unit": "Mrays/s", "ms_per_step": round(plain_ms, 4),
                  "how": "per scene: rtg_scene_build (synchronous) + rtg_trace_nearest_device, 64 in sequence"},
        "batched_over_plain": round(plain_ms / batched_ms, 3),
        "breakdown_ms": {k_: round(v_, 4) for k_, v_ in breakdown.items()},
    })


# ---------------------------------------------------------------------------
# skewed density: 1,048,576 triangles (90% small in a 0.1^3 box, 10% large in
# [-4,4]^3); per step a grid build, 1024^2 primary camera rays and one
# cosine-weighted diffuse secondary ray per primary hit (generated on the
# device, seeded per step), both traced closest-hit; t / u / v errors of the
# reported hits against a float64 Moller-Trumbore recomputation
# ---------------------------------------------------------------------------
def _fp64_errors(verts, idx, rays, hits):
    """Max / mean error of the reported t (relative) and u, v (absolute) of
    every hit against float64 Moller-Trumbore on the same ray and triangle."""
    ok = hits["id"] >= 0
    tri = hits["id"][ok]
    r = rays[ok].astype(np.float64)
    o, d = r[:, 0:3], r[:, 4:7]
    v0 = verts[idx[tri, 0]].astype(np.float64)
    e1 = verts[idx[tri, 1]].astype(np.float64) - v0
    e2 = verts[idx[tri, 2]].astype(np.float64) - v0
    p = np.cross(d, e2)
    inv = 1.0 / (e1 * p).sum(1)
    tv = o - v0
    q = np.cross(tv, e1)
    u = (tv * p).sum(1) * inv
    v = (d * q).sum(1) * inv
    t = (e2 * q).sum(1) * inv
    et = np.abs(hits["t"][ok] - t) / np.maximum(np.abs(t), 1e-30)
    eu = np.abs(hits["u"][ok] - u)
    ev = np.abs(hits["v"][ok] - v)
    out = {"hits": int(ok.sum())}
    for name, e in (("t_rel", et), ("u_abs", eu), ("v_abs", ev)):
        out[name] = {"max": float(e.max()) if e.size else 0.0, "mean": float(e.mean()) if e.size else 0.0,
                     "above_1e-5": int((e > 1e-5).sum())}
    return out


def run_skewed(args, rank, ws, local, dist):
    import torch
    from gridrt import autotune, lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sc = scenes.skewed_density()
    cam = scenes.skewed_density_camera(WIDTH, HEIGHT)
    npix = WIDTH * HEIGHT
    s = lib.Scene(local)
    s.set_geometry(sc.verts, sc.idx)
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    d_hits = torch.empty((npix, 4), dtype=torch.int32, device=dev)
    d_sec = torch.empty((npix, 8), dtype=torch.float32, device=dev)
    d_hits2 = torch.empty((npix, 4), dtype=torch.int32, device=dev)
    # a second scene of the same triangles holds the other step in flight
    s2 = lib.Scene(local)
    s2.set_geometry(sc.verts, sc.idx)
    stream2 = torch.cuda.ExternalStream(s2.stream, device=dev)
    d_sec_b = torch.empty_like(d_sec)
    scene_a = (s, stream, d_hits, d_sec, d_hits2)
    scene_b = (s2, stream2, torch.empty_like(d_hits), d_sec_b, torch.empty_like(d_hits2))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for k in LAMBDAS:
        s.build(k)          # capacities for every k (untimed)
        s2.build(k)

    def step(k, seed, order, ev=None, on=scene_a):
        g, st, hits, sec, hits2 = on
        with torch.cuda.stream(st):
            if ev:
                ev[0].record(st)
            g.build_async(k)
            if ev:
                ev[1].record(st)
            g.trace_camera_diffuse_device(cam, seed, hits, sec, order=order)
            g.trace_nearest_device(sec, npix, hits2)
            if ev:
                ev[2].record(st)

    # each candidate timed as the workload runs: a pair of steps in flight on
    # the two scenes (after one untimed step)
    def measure(cfg):
        _apply_tuning(s, cfg)
        _apply_tuning(s2, cfg)
        k = cfg["k"]
        step(k, 1, cfg["order"])
        return _pair_ms(torch, stream, stream2,
                        lambda: (step(k, 2, cfg["order"]), step(k, 3, cfg["order"], on=scene_b)))

    fixed = _parse_tuning(args.fixed_tuning)
    if fixed:
        best, allres = dict(fixed), []
    else:
        space = {"k": LAMBDAS, "order": ("scanline", "morton8"), "empty_run": (2, 4, 8), "persistent": (True,),
                 "heavy_cell": (0, 24, 48), "heavy_lanes": (16, 32), "cell_records": (False, True),
                 "refill": (0, 16), "block": (128, 64, 256), "lanes": (1, 2)}
        best, allres = autotune.search(measure, space=space, reps=2)
        _save_autotune("skewed", allres)
    _apply_tuning(s, best)
    _apply_tuning(s2, best)
    k, order = best["k"], best["order"]
    for w in range(args.warmup):
        step(k, 100 + w, order)
        step(k, 200 + w, order, on=scene_b)
    torch.cuda.synchronize()
    if s.build_check() != 0 or s2.build_check() != 0:
        raise RuntimeError("warm-up build failed: " + lib.load().rtg_last_error().decode())
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    nsec = torch.zeros((), dtype=torch.int64, device=dev)
    sampler = ClockSampler(local).start() if rank == 0 else None
    _barrier(dist)
    torch.cuda.synchronize()
    if sampler:
        sampler.mark()
    lc0 = lib.kernel_launches()
    for st in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()                      # L2 flush between steps (outside the events)
        step(k, 1000 + st, order, evs[st])
        with torch.cuda.stream(stream):
            nsec += (d_sec[:, 7] > 0).sum()    # secondary rays traced (outside the events)
    lc1 = lib.kernel_launches()
    torch.cuda.synchronize()
    if sampler:
        sampler.unmark()
    build_ms = [e[0].elapsed_time(e[1]) for e in evs]
    step_ms = [e[0].elapsed_time(e[2]) for e in evs]
    one_ms = _max_over_ranks(sum(step_ms), dist)
    one_rays = _sum_over_ranks(npix * args.steps + int(nsec.item()), dist)

    # two steps in flight: steps 2j and 2j + 1 on the two scenes, each on its
    # own streams (forked from and joined back to the first scene's stream),
    # so one step's build runs beside the other's trace; the same K steps,
    # the L2 flushed before each pair
    n_pair = args.steps // 2
    pevs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(n_pair + args.steps % 2)]
    fork = [torch.cuda.Event() for _ in pevs]
    join = [torch.cuda.Event() for _ in pevs]
    nsec2 = torch.zeros((), dtype=torch.int64, device=dev)
    _barrier(dist)
    torch.cuda.synchronize()
    if sampler:
        sampler.mark()
    for st in range(len(pevs)):
        with torch.cuda.stream(stream):
            flush.zero_()
            pevs[st][0].record(stream)
        if st < n_pair:
            fork[st].record(stream)
            stream2.wait_event(fork[st])
            step(k, 1000 + 2 * st, order)
            step(k, 1000 + 2 * st + 1, order, on=scene_b)
            join[st].record(stream2)
            stream.wait_event(join[st])
        else:
            step(k, 1000 + 2 * st, order)
        with torch.cuda.stream(stream):
            pevs[st][1].record(stream)
            nsec2 += (d_sec[:, 7] > 0).sum()
            if st < n_pair:
                nsec2 += (d_sec_b[:, 7] > 0).sum()
    torch.cuda.synchronize()
    if sampler:
        sampler.unmark()
        sampler.stop()
    if s.build_check() != 0 or s2.build_check() != 0:
        raise RuntimeError("paired build failed: " + lib.load().rtg_last_error().decode())
    t_ms = _max_over_ranks(sum(e[0].elapsed_time(e[1]) for e in pevs), dist)
    rays = _sum_over_ranks(npix * args.steps + int(nsec2.item()), dist)

    # traversal counters of one step (primary, then secondary rays) for the
    # algorithmic bytes: 16 B hit + 32 B secondary ray written per primary
    # ray, 32 B read + 16 B hit per secondary ray, 8 B per visited cell,
    # 52 B per triangle test
    s.counters(reset=True)
    with torch.cuda.stream(stream):
        s.trace_camera_diffuse_device(cam, 1000, d_hits, d_sec, order=order, counters=True)
    torch.cuda.synchronize()
    c1 = s.counters(reset=True)
    with torch.cuda.stream(stream):
        s.trace_nearest_device(d_sec, npix, d_hits2, counters=True)
    torch.cuda.synchronize()
    c2 = s.counters(reset=True)
    alg_bytes = (48 * npix + 48 * npix + 8 * (c1["cells"] + c2["cells"]) + 52 * (c1["tests"] + c2["tests"]))
    trace_ms = statistics.median(e[1].elapsed_time(e[2]) for e in evs)
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (trace_ms / 1e3) / 1e9

    # errors of the last step's hits (primary rays regenerated on the host
    # bit-identically; secondary rays as the device wrote them)
    prim_rays = scenes.camera_rays(cam, order)
    prim = lib.split_hits(d_hits.cpu().numpy())
    sec_rays = d_sec.cpu().numpy()
    sec = lib.split_hits(d_hits2.cpu().numpy())
    err = {"primary": _fp64_errors(sc.verts, sc.idx, prim_rays, prim),
           "secondary": _fp64_errors(sc.verts, sc.idx, sec_rays, sec)}
    if rank != 0:
        return None
    clocks = sampler.summary() if sampler else {}
    return ({
        "metric": "Mrays/s (primary + diffuse secondary, grid build included)",
        "value": round(rays / t_ms / 1e3, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "skewed_density_1048576tri_1024x1024_diffuse", "k": k, "ray_order": order,
                   "tuning": best, "triangles": sc.ntris, "rays_per_step": round(rays / args.steps / ws),
                   "steps_in_flight": 2,
                   "l2": "flushed before every pair of steps in flight (256 MiB write, outside the timed events)"},
        "one_step_in_flight": {"value": round(one_rays / one_ms / 1e3, 3), "ms_per_step": round(one_ms / args.steps, 4),
                               "how": "the same steps one at a time on one scene, the L2 flushed before each"},
        "build_ms": round(statistics.median(build_ms), 4),
        "trace_ms": round(trace_ms, 4),
        "counters": {"primary": c1, "secondary": c2,
                     "tests_per_ray": round((c1["tests"] + c2["tests"]) / max(1, c1["rays"] + c2["rays"]), 2),
                     "cells_per_ray": round((c1["cells"] + c2["cells"]) / max(1, c1["rays"] + c2["rays"]), 2)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": None,
                     "kernel": "primary + secondary trace launches with their deferred passes",
                     "alg_bytes_per_launch": int(alg_bytes)},
        "fp64_error": err,
        "gpu_launches": int(lc1 - lc0),
        "clocks": {"sm_mhz": clocks.get("sm_mhz"), "sm_max_mhz": clocks.get("sm_max_mhz"),
                   "reasons": clocks.get("reasons", []), "samples": clocks.get("samples", 0)},
    })


# ---------------------------------------------------------------------------
# instances: 16 transformed instances of three scenes (two-level trace) and
# the same world flattened into one scene (one-level trace), 1024^2 camera
# rays closest hit
# ---------------------------------------------------------------------------
def _instance_world(seed: int = 20261203, n_inst: int = 16):
    rng = np.random.default_rng(seed)
    base = [scenes.deforming_sphere(0), scenes.plane_and_debris(), scenes.tiny_scene(6, 20_000, spread=1.0)]
    inst = []
    for j in range(n_inst):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        sc_ = rng.uniform(0.6, 1.6)
        t = rng.uniform(-5.0, 5.0, size=3)
        M = np.concatenate([sc_ * R, t[:, None]], axis=1)
        Ri = R.T / sc_
        inv = np.concatenate([Ri, (-Ri @ t)[:, None]], axis=1)
        inst.append((j % len(base), M.astype(np.float32), inv.astype(np.float32)))
    return base, inst


def run_instances(args, rank, ws, local, dist):
    import torch
    from gridrt import lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    base, inst = _instance_world()
    k = 4
    scs = []
    for sc in base:
        s = lib.Scene(local)
        s.set_geometry(sc.verts, sc.idx)
        s.build(k)
        scs.append(s)
    I = lib.Instances([(scs[b], M, inv) for b, M, inv in inst])
    # the flattened world: every instance's vertices taken to world space
    fv, fi, off = [], [], 0
    for b, M, _ in inst:
        v = base[b].verts.astype(np.float64) @ M[:, :3].astype(np.float64).T + M[:, 3].astype(np.float64)
        fv.append(v.astype(np.float32))
        fi.append(base[b].idx + off)
        off += base[b].verts.shape[0]
    flat = lib.Scene(local)
    flat.set_geometry(np.concatenate(fv), np.concatenate(fi))
    flat.build(k)
    cam = scenes.look_at_camera((11.0, 7.0, 13.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 60.0, WIDTH, HEIGHT)
    rays = scenes.camera_rays(cam, "morton8")
    n = rays.shape[0]
    d_rays = torch.from_numpy(rays).to(dev)
    d_hits = torch.empty((n, 4), dtype=torch.int32, device=dev)
    d_inst = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.ExternalStream(scs[0].stream, device=dev)

    def timed(fn):
        for _ in range(args.warmup):
            with torch.cuda.stream(stream):
                fn()
        torch.cuda.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
        _barrier(dist)
        for e in evs:
            with torch.cuda.stream(stream):
                flush.zero_()
                e[0].record(stream)
                fn()
                e[1].record(stream)
        torch.cuda.synchronize()
        return _max_over_ranks(sum(e[0].elapsed_time(e[1]) for e in evs) / 1e3, dist)

    t_inst = timed(lambda: I.trace_nearest_device(d_rays, n, d_hits, d_inst, stream=stream.cuda_stream))
    hit_frac = float((d_inst >= 0).float().mean().item())
    t_flat = timed(lambda: flat.trace_nearest_device(d_rays, n, d_hits, stream=stream.cuda_stream))
    rays_all = _sum_over_ranks(n * args.steps, dist)
    if rank != 0:
        return None
    tris_inst = sum(base[b].ntris for b, _, _ in inst)
    return ({
        "metric": "Mrays/s (two-level instanced closest hit)", "value": round(rays_all / t_inst / 1e6, 3),
        "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * t_inst / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "instances_16_of_3_scenes_1024x1024", "k": k, "instances": len(inst),
                   "scene_triangles": [sc.ntris for sc in base], "instanced_triangles": int(tris_inst),
                   "hit_fraction": round(hit_frac, 4),
                   "l2": "flushed between steps (256 MiB write, outside the timed events)"},
        "flattened": {"value": round(rays_all / t_flat / 1e6, 3), "unit": "Mrays/s",
                      "ms_per_step": round(1e3 * t_flat / args.steps, 4),
                      "how": "all instances' triangles taken to world space in one scene, one-level trace"},
    })


# ---------------------------------------------------------------------------
# render: the shading wavefront (rtg_render) on the plane-and-debris scene,
# 1024^2 pixels, Phong / headlight materials, two point lights (one casting
# shadows), reflection on the plane, refraction on a quarter of the debris,
# recursion depth 3
# ---------------------------------------------------------------------------
def run_ingest(args, rank, ws, local, dist):
    """Scene ingest: the deforming sphere's mesh (102,400 triangles) written
    as an indexed OBJ and as a binary little-endian PLY, read back with the
    reference loaders' rules (rtg_mesh_load, host), then uploaded and built
    (k = 4).  Host clock, median of `steps` repetitions."""
    import tempfile
    import torch
    from gridrt import lib

    torch.cuda.set_device(local)
    v, idx, _ = scenes.sphere_mesh()
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        obj = os.path.join(tmp, "sphere.obj")
        with open(obj, "w") as f:
            f.write("".join(f"v {float(a)!r} {float(b)!r} {float(c)!r}\n" for a, b, c in v))
            f.write("".join(f"f {i + 1} {j + 1} {k + 1}\n" for i, j, k in idx))
        ply = os.path.join(tmp, "sphere.ply")
        with open(ply, "wb") as f:
            f.write((f"ply\nformat binary_little_endian 1.0\nelement vertex {len(v)}\nproperty float x\n"
                     f"property float y\nproperty float z\nelement face {len(idx)}\n"
                     f"property list uchar int vertex_indices\nend_header\n").encode())
            f.write(np.ascontiguousarray(v, np.float32).tobytes())
            rec = np.zeros(len(idx), dtype=np.dtype([("n", "u1"), ("i", "<i4", (3,))]))
            rec["n"] = 3
            rec["i"] = idx
            f.write(rec.tobytes())
        for name, path in (("obj", obj), ("ply_binary", ply)):
            size = os.path.getsize(path)
            load_s, build_s, ntris = [], [], 0
            for rep in range(max(args.steps, 3) + 1):
                t0 = time.perf_counter()
                mv, mt, _, _ = lib.load_mesh(path)
                t1 = time.perf_counter()
                s = lib.Scene(local)
                s.set_geometry(mv, mt)
                s.build(4)
                torch.cuda.synchronize()
                t2 = time.perf_counter()
                if rep:                                   # the first repetition warms caches and the context
                    load_s.append(t1 - t0)
                    build_s.append(t2 - t1)
                ntris = int(mt.shape[0])
                del s
            lm, bm = statistics.median(load_s), statistics.median(build_s)
            out[name] = {"bytes": size, "triangles": ntris, "load_ms": round(1e3 * lm, 3),
                         "load_mb_s": round(size / lm / 1e6, 1), "load_mtris_s": round(ntris / lm / 1e6, 2),
                         "upload_build_ms": round(1e3 * bm, 3)}
    if rank != 0:
        return None
    return {"metric": "Mtriangles/s read (rtg_mesh_load) + upload and grid build ms", "unit": "Mtriangles/s",
            "value": out["ply_binary"]["load_mtris_s"], "higher_is_better": True, "n_gpus": ws,
            "steps": args.steps, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "ingest_sphere_102400tri", "k": 4,
                       "timing": "host clock, median; upload + synchronous build on the device after the load"},
            "formats": out}


def run_render(args, rank, ws, local, dist):
    import torch
    from gridrt import lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sc = scenes.plane_and_debris()
    s = lib.Scene(local)
    s.set_geometry(sc.verts, sc.idx)
    s.build(4)
    v = sc.verts.astype(np.float64)
    f = sc.idx
    fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    nrm = np.zeros_like(v)
    for kk in range(3):
        np.add.at(nrm, f[:, kk], fn)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
    rng = np.random.default_rng(20261207)
    colors = rng.uniform(0.2, 1.0, size=sc.verts.shape).astype(np.float32)
    mat = (np.arange(sc.ntris) % 4).astype(np.int32)
    mat[:32768] = 0
    mats = [lib.material(lib.RTG_MAT_PHONG, reflexion=0.35),
            lib.material(lib.RTG_MAT_PHONG_COLOR, diffuse=(0.8, 0.3, 0.2), opacity=0.6, refraction_index=1.3),
            lib.material(lib.RTG_MAT_HEADLIGHT, ambient=(0.1, 0.1, 0.1)),
            lib.material(lib.RTG_MAT_HEADLIGHT_COLOR, ambient=(0.1, 0.1, 0.1), diffuse=(0.2, 0.6, 0.9))]
    lights = [lib.point_light((2.0, 4.0, 2.0), (0.8, 0.8, 0.8), True),
              lib.point_light((-3.0, 2.0, 1.0), (0.3, 0.3, 0.4), False)]
    d_n = torch.from_numpy(nrm.astype(np.float32)).to(dev)
    d_c = torch.from_numpy(colors).to(dev)
    d_m = torch.from_numpy(mat).to(dev)
    cam = scenes.plane_and_debris_camera(WIDTH, HEIGHT)
    d_rgb = torch.empty((WIDTH * HEIGHT, 3), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # lanes per ray for the bounce levels' trace launches (results do not
    # depend on it), each candidate timed on one frame after one untimed
    from gridrt import autotune

    def measure(cfg):
        s.set_tuning(lanes=cfg["lanes"])
        s.render(cam, d_n, mats, lights, d_rgb, d_colors=d_c, d_material=d_m, max_depth=3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.render(cam, d_n, mats, lights, d_rgb, d_colors=d_c, d_material=d_m, max_depth=3)
        return 1e3 * (time.perf_counter() - t0)

    best, allres = autotune.search(measure, space={"lanes": (1, 2, 4)}, reps=3)
    _save_autotune("render", allres)
    s.set_tuning(lanes=best["lanes"])
    for _ in range(args.warmup):
        s.render(cam, d_n, mats, lights, d_rgb, d_colors=d_c, d_material=d_m, max_depth=3)
    torch.cuda.synchronize()
    _barrier(dist)
    total, rays = 0.0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rays += s.render(cam, d_n, mats, lights, d_rgb, d_colors=d_c, d_material=d_m, max_depth=3)
        total += time.perf_counter() - t0
    total = _max_over_ranks(total, dist)
    rays_all = _sum_over_ranks(rays, dist)
    if rank != 0:
        return None
    return ({
        "metric": "Mrays/s (shading wavefront: primary + shadow + reflected + refracted)",
        "value": round(rays_all / total / 1e6, 3), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * total / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "render_plane_and_debris_1024x1024_depth3", "k": 4, "rays_per_step": rays // args.steps,
                   "lanes": best["lanes"],
                   "timing": "host clock around the synchronous rtg_render call (per-level count read-backs "
                             "included); L2 flushed before each frame, outside the timed call"},
    })


# ---------------------------------------------------------------------------
# serving: 16 resident scenes, Poisson request streams, continuous batching
# (rtg_serve_run) versus the plain one-request-at-a-time path
# ---------------------------------------------------------------------------
def run_serving(args, rank, ws, local, dist):
    import torch
    from gridrt import lib

    torch.cuda.set_device(local)
    rng = np.random.Generator(np.random.PCG64(scenes.SEED_BASE + 4))
    nscenes = 16
    scs, scene_bytes, tris = [], 0, 0
    for i in range(nscenes):
        n_tri = int(round(np.exp(rng.uniform(np.log(10_000), np.log(1_000_000)))))
        quads = max(2, int(round(np.sqrt(n_tri / 4.0))))
        sc = scenes.plane_and_debris(seed=scenes.SEED_BASE + 400 + i, quads=quads, debris=max(1, n_tri - 2 * quads * quads))
        s = lib.Scene(local)
        s.set_geometry(sc.verts, sc.idx)
        s.build(4)
        s.set_tuning(refill=args.serve_refill)
        inf = s.info()
        scene_bytes += 12 * sc.nverts + 12 * sc.ntris + 48 * sc.ntris + 8 * (inf["ncells"] + 1) + 8 * inf["nrefs"]
        tris += sc.ntris
        scs.append(s)
    # ray pools shared by all requests (every scene spans [-1,1] x [0,1] x [-1,1])
    pool_n = 4_000_000
    cam = scenes.plane_and_debris_camera(2000, 1000)
    near = np.concatenate([scenes.camera_rays(cam), scenes.random_rays(rng, pool_n - 2_000_000, (-1, 0, -1), (1, 1, 1))])
    anyr = scenes.random_rays(rng, pool_n, (-1, 0, -1), (1, 1, 1))
    anyr[:, 7] = 1.0
    h_near = torch.from_numpy(near).pin_memory()
    h_any = torch.from_numpy(anyr).pin_memory()
    h_out = torch.empty(16 * pool_n, dtype=torch.uint8).pin_memory()
    budget = 40 << 30
    pool_bytes = int(min(8 << 30, budget - scene_bytes))

    def make_requests(rate, count, seed):
        r = np.random.Generator(np.random.PCG64(seed))
        t = 0.0 if rate is None else np.cumsum(r.exponential(1.0 / rate, size=count))
        reqs = []
        for i in range(count):
            n = int(round(np.exp(r.uniform(np.log(1_000), np.log(4_000_000)))))
            off = int(r.integers(0, pool_n - n + 1))
            si = int(r.integers(0, nscenes))
            if r.uniform() < 0.3:
                mode, src = lib.RTG_MODE_ANY, h_any
            else:
                mode, src = lib.RTG_MODE_NEAREST, h_near
            arr = 0.0 if rate is None else float(t[i])
            reqs.append((arr, si, mode, src.data_ptr() + 32 * off, n, h_out))
        return reqs

    def run(reqs, plain, in_flight=None):
        # plain = one request at a time: upload, single-scene trace, download, wait
        # (in_flight 1); plain_pipelined keeps three such requests in flight
        if in_flight is None:
            in_flight = 1 if plain else 3
        admit, done = lib.serve(scs, reqs, pool_bytes=pool_bytes, plain=plain, max_in_flight=in_flight,
                                max_step_rays=args.serve_step_rays)
        arr = np.array([q[0] for q in reqs])
        lat = done - arr
        rays = sum(q[4] for q in reqs)
        span = done.max() - arr.min()
        return dict(p50_ms=round(1e3 * float(np.percentile(lat, 50)), 3),
                    p99_ms=round(1e3 * float(np.percentile(lat, 99)), 3),
                    mrays_s=round(rays / span / 1e6, 2), requests=len(reqs), rays=int(rays))

    # warm up both paths
    wu = make_requests(None, 20, 1)
    run(wu, False)
    run(wu, True)
    rates = [int(r) for r in args.serve_rates.split(",") if r]
    out = {}
    for rate in rates:
        count = int(min(10_000, rate * args.serve_seconds))
        reqs = make_requests(rate, count, 100 + rate)
        # one untimed pass of the same requests through each path first
        run(reqs, False)
        run(reqs, True)
        out[str(rate)] = {"served": run(reqs, False), "plain": run(reqs, True)}
    sat = make_requests(None, args.serve_saturation, 7)
    saturation = {"served": run(sat, False), "plain": run(sat, True),
                  "plain_pipelined": run(sat, True, in_flight=3)}

    # device-only ceiling: the saturation requests' rays already in HBM,
    # traced as one batch launch (no transfers, no request loop, no waits)
    dev = torch.device("cuda", local)
    d_src = {h_near.data_ptr(): h_near.to(dev), h_any.data_ptr(): h_any.to(dev)}
    tasks = []
    for (_, si, mode, ptr, n, _) in sat:
        hsrc = h_any if mode == lib.RTG_MODE_ANY else h_near
        d_rays = d_src[hsrc.data_ptr()].data_ptr() + (ptr - hsrc.data_ptr())
        d_out = torch.empty(n * (1 if mode == lib.RTG_MODE_ANY else 16), dtype=torch.uint8, device=dev)
        tasks.append((si, mode, d_rays, n, d_out))
    ceil_batch = lib.Batch(scs, [4] * nscenes, tasks)
    ceil_batch.set_tuning(refill=args.serve_refill)
    st = torch.cuda.Stream(device=dev)
    ceil_batch.trace_async(st.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        e0.record(st)
        ceil_batch.trace_async(st.cuda_stream)
        e1.record(st)
    torch.cuda.synchronize()
    ceil_ms = e0.elapsed_time(e1)
    saturation["device_ceiling"] = {"mrays_s": round(saturation["served"]["rays"] / ceil_ms / 1e3, 2),
                                    "ms": round(ceil_ms, 3),
                                    "how": "the same requests' rays resident in HBM, one rtg_batch trace launch "
                                           "over all of them (no copies, no request loop)"}
    del ceil_batch, tasks, d_src
    if rank != 0:
        return None
    return ({
        "metric": "Mrays/s at saturation (served) + p50/p99 latency", "value": saturation["served"]["mrays_s"],
        "unit": "Mrays/s", "n_gpus": ws, "steps": len(rates), "warmup": 1, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serving_16_scenes", "scenes": nscenes, "triangles": tris,
                   "scene_bytes": int(scene_bytes), "pool_bytes": pool_bytes, "hbm_budget_bytes": budget,
                   "rays_per_request": "log-uniform [1e3, 4e6]", "modes": "70% closest / 30% any-hit",
                   "max_in_flight": {"served": 3, "plain": 1, "plain_pipelined": 3},
                   "max_step_rays": args.serve_step_rays,
                   "refill": args.serve_refill},
        "saturation": saturation, "served_over_plain": round(saturation["served"]["mrays_s"] /
                                                              saturation["plain"]["mrays_s"], 3),
        "served_over_plain_pipelined": round(saturation["served"]["mrays_s"] /
                                             saturation["plain_pipelined"]["mrays_s"], 3),
        "rates": out,
    })


def _parse_tuning(text):
    """'k=8,order=morton8,empty_run=4,persistent=0,heavy_cell=32,cell_records=1,refill=16' -> dict, or None."""
    if not text:
        return None
    d = dict(kv.split("=", 1) for kv in text.split(","))
    yes = lambda v: v not in ("0", "false", "False")
    return {"k": int(d.get("k", 8)), "order": d.get("order", "morton8"), "empty_run": int(d.get("empty_run", 4)),
            "persistent": yes(d.get("persistent", "0")), "heavy_cell": int(d.get("heavy_cell", 0)),
            "heavy_lanes": int(d.get("heavy_lanes", 32)), "cell_records": yes(d.get("cell_records", "0")),
            "refill": int(d.get("refill", 0)), "block": int(d.get("block", 128)), "lanes": int(d.get("lanes", 1))}


def _apply_tuning(scene, cfg):
    """Launch-shape settings of one candidate; cell records take effect at the next build."""
    # every setting is applied, defaults included, so no candidate inherits
    # the one before it
    scene.set_tuning(empty_run=cfg["empty_run"], persistent=cfg["persistent"],
                     heavy_cell=cfg.get("heavy_cell", 0), heavy_lanes=cfg.get("heavy_lanes", 32),
                     cell_records=cfg.get("cell_records", False), refill=cfg.get("refill", 0),
                     block=cfg.get("block", 128), lanes=cfg.get("lanes", 1))


def _tune_str(cfg) -> str:
    """A launch-shape choice in a few characters: order/ER/persistent/heavy
    cell x lanes/refill/cell records."""
    if not cfg:
        return ""
    return (f"{cfg.get('order', '')}/er{cfg.get('empty_run', '')}/p{int(bool(cfg.get('persistent', 0)))}"
            f"/h{cfg.get('heavy_cell', 0)}x{cfg.get('heavy_lanes', 32)}/r{cfg.get('refill', 0)}"
            f"/c{int(bool(cfg.get('cell_records', 0)))}/b{cfg.get('block', 128)}/l{cfg.get('lanes', 1)}")


def _r(x, n=3):
    return None if x is None else round(float(x), n)


def compact_line(full: dict, subs: dict) -> dict:
    """The one result line: the headline workload's contract keys and
    figures, then one small object per further workload (about 2.5 KB in
    all; every figure of the sub-objects is in Mrays/s or ms as its key
    says; everything else goes to --detail)."""
    c = {k: full[k] for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                              "higher_is_better", "scaling", "vs_baseline", "dtype", "data")}
    cfg = full["config"]
    c["config"] = {"workload": cfg["workload"], "k": cfg["k"], "frames": cfg["frames"], "triangles": cfg["triangles"],
                   "rays_primary": cfg["rays_primary"], "frames_in_flight": cfg.get("frames_in_flight", 1),
                   "l2": ("flushed before every pair of frames in flight (256 MiB write)"
                          if cfg.get("frames_in_flight", 1) == 2 else "flushed between frames (256 MiB write)"),
                   "parallelism": cfg["parallelism"], "tuning": _tune_str(cfg["tuning"]),
                   "tuned_by": full.get("autotune", {}).get(str(cfg["k"]), {}).get("source")}
    if "one_frame_in_flight" in full:
        o = full["one_frame_in_flight"]
        c["one_frame_in_flight"] = {"value": _r(o["value"], 1), "ms_per_step": o["ms_per_step"]}
    c["build_ms"] = _r(full["build_ms"], 4)
    c["trace_mrays_s"] = _r(full["trace_mrays_s"], 1)
    c["per_k"] = {k: {"value": _r(v["value"], 1), "build_ms": _r(v["build_ms"], 4),
                      "stream_value": _r(v["stream_value"], 1),
                      **({"one_in_flight": _r(v["one_in_flight_value"], 1)} if "one_in_flight_value" in v else {})}
                  for k, v in full["per_k"].items()}
    rf = full["roofline"]
    c["roofline"] = {"bound": rf["bound"], "achieved": rf["achieved"], "peak": rf["peak"], "unit": rf["unit"],
                     "frac": rf["frac"], "traffic": rf["traffic"], "peak_source": rf["peak_source"],
                     "kernel": "trace_kernel frame + deferred pass", "kernel_ms": rf["kernel_ms"],
                     "alg_bytes": rf["alg_bytes_per_launch"], "l2_frac": rf["l2"]["frac"], "l2_peak": rf["l2"]["peak"]}
    br = full["build_roofline"]
    c["build_roofline"] = {"achieved": br["achieved"], "frac": br["frac"], "alg_bytes": br["alg_bytes"],
                           "ms": _r(br["ms"], 4)}
    cb = full["cpu_baseline"]
    c["cpu_baseline"] = {"value": cb["value"], "unit": cb["unit"], "cores": cb["cores"], "kind": cb["kind"],
                         "sample": f"10 frames k={cfg['k']}, every ray", "build_ms": cb["build_ms"]}
    e = full["e2e"]
    c["e2e"] = {"value": e["value"], "unit": e["unit"], "h2d_bytes_per_step": e["h2d_bytes_per_step"],
                "d2h_bytes_per_step": e["d2h_bytes_per_step"], "ms_per_step": e["ms_per_step"]}
    c["gpu_launches"] = full["gpu_launches"]
    ck = full["clocks"]
    c["clocks"] = {"sm_mhz": ck["sm_mhz"], "sm_max_mhz": ck["sm_max_mhz"], "reasons": ck["reasons"]}
    for name, sub in subs.items():
        c[name] = sub
    return c


def compact_skewed(d: dict) -> dict:
    if d is None or "error" in d:
        return d
    err = d["fp64_error"]
    return {"workload": "skewed_1048576tri_1024x1024_diffuse", "k": d["config"]["k"], "value": _r(d["value"], 1),
            "ms_per_step": d["ms_per_step"], "build_ms": d["build_ms"], "trace_ms": d["trace_ms"],
            "rays_per_step": d["config"]["rays_per_step"], "tests_per_ray": d["counters"]["tests_per_ray"],
            "roofline_frac": d["roofline"]["frac"], "tuning": _tune_str(d["config"]["tuning"]),
            **({"one_in_flight": _r(d["one_step_in_flight"]["value"], 1)} if "one_step_in_flight" in d else {}),
            "fp64_max": {g: [_r(err[g]["t_rel"]["max"], 8), _r(err[g]["u_abs"]["max"], 8),
                             _r(err[g]["v_abs"]["max"], 8)] for g in ("primary", "secondary")}}


def compact_batched(d: dict) -> dict:
    if d is None or "error" in d:
        return d
    b = d["breakdown_ms"]
    return {"workload": "batched_64_scenes", "value": _r(d["value"], 1), "plain": _r(d["plain"]["value"], 1),
            "ratio": d["batched_over_plain"], "ms_per_step": d["ms_per_step"], "plain_ms": d["plain"]["ms_per_step"],
            "build_ms": _r(b["batched_build_ms"], 3), "trace_ms": _r(b["batched_trace_ms"], 3),
            "tuning": "k{k}/{order}/er{empty_run}/r{refill}".format(**d["config"]["tuning"])}


def compact_serving(d: dict) -> dict:
    if d is None or "error" in d:
        return d
    sat = d["saturation"]
    out = {"workload": "serving_16_scenes", "value": sat["served"]["mrays_s"], "plain": sat["plain"]["mrays_s"],
           "ratio": d["served_over_plain"], "p50_ms": sat["served"]["p50_ms"], "p99_ms": sat["served"]["p99_ms"],
           "plain_p50_ms": sat["plain"]["p50_ms"], "plain_p99_ms": sat["plain"]["p99_ms"],
           "requests": sat["served"]["requests"], "device_ceiling": sat["device_ceiling"]["mrays_s"]}
    for rate, r in d["rates"].items():
        out[f"r{rate}"] = {"p50_ms": r["served"]["p50_ms"], "p99_ms": r["served"]["p99_ms"],
                           "plain_p50_ms": r["plain"]["p50_ms"], "plain_p99_ms": r["plain"]["p99_ms"],
                           "requests": r["served"]["requests"]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gridrt", choices=["gridrt", "reference"])
    ap.add_argument("--workload", default="default",
                    choices=["default", "deforming", "plain", "batched", "serving", "skewed", "instances", "render",
                             "ingest"],
                    help="default: the deforming-mesh headline plus the plain, skewed, batched and serving "
                         "workloads in one line; any other: that workload alone, in full")
    ap.add_argument("--serve-seconds", type=float, default=4.0)
    ap.add_argument("--serve-saturation", type=int, default=2000)
    ap.add_argument("--serve-rates", default="10,100,1000,2000")
    ap.add_argument("--serve-step-rays", type=int, default=1 << 22,
                    help="rays a serving step admits at most (a larger request still forms a step alone); "
                         "0: the library's default (16 M)")
    ap.add_argument("--serve-refill", type=int, default=8,
                    help="lane-refill threshold of the serving scenes (served and plain paths alike)")
    ap.add_argument("--fixed-tuning", default="",
                    help="skip the autotuner: e.g. k=8,order=morton8,empty_run=4,persistent=0 (profiling runs)")
    ap.add_argument("--detail", default="", help="also write every workload's full result to this JSON file")
    ap.add_argument("--profile-frames", type=int, default=0,
                    help="profiling runs: only this many deforming-sphere frames (build + frame trace), "
                         "launched call by call with --fixed-tuning's k and shape; prints nothing")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, ws, local, dist = _dist()
    single = {"plain": run_plain_small, "batched": run_batched, "serving": run_serving, "skewed": run_skewed,
              "instances": run_instances, "render": run_render, "ingest": run_ingest}
    detail = {}
    if args.impl == "reference":
        line = run_reference(args, rank, ws, dist)
    elif args.workload in single:
        line = single[args.workload](args, rank, ws, local, dist)
        detail[args.workload] = line
    else:
        full = run_gpu(args, rank, ws, local, dist)
        detail["deforming"] = full
        subs = {}
        if args.workload == "default" and ws == 1 and not args.profile_frames:
            import argparse as _ap
            import torch
            serve_args = _ap.Namespace(**vars(args))
            serve_args.serve_rates, serve_args.serve_seconds, serve_args.serve_saturation = "1000", 3.0, 2000
            for name, fn, squash in (("cfg0_plain", run_plain_small, None),
                                     ("cfg2_skewed", run_skewed, compact_skewed),
                                     ("cfg3_batched", run_batched, compact_batched),
                                     ("cfg4_serving", run_serving, compact_serving)):
                try:
                    d = fn(serve_args if name == "cfg4_serving" else args, rank, ws, local, dist)
                    detail[name] = d
                    subs[name] = squash(d) if squash else d
                except Exception as exc:          # one workload's failure keeps the headline line
                    subs[name] = {"error": f"{type(exc).__name__}: {exc}"[:160]}
                torch.cuda.synchronize()
                torch.cuda.empty_cache()
        line = compact_line(full, subs) if full is not None else None
    if rank == 0 and line is not None:
        if args.detail:
            with open(args.detail, "w") as f:
                json.dump(detail, f, indent=1, default=str)
        print(json.dumps(line, separators=(",", ":")), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
