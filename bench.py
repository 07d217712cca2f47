#!/usr/bin/env python3
"""FLIP step benchmark on GB300: Mparticle-steps/s at 128^3.

Workload (N=1): the 128^3 plain FLIP dam break (dx = 1/128, fluid box
x<0.4, y<0.6, 8 jittered particles per cell, seed 0) plus a falling sphere
(r = 0.15 at (0.7, 0.7, 0.5), v = (0, -2, 0)), FLIP blend 0.95, gravity
-9.81, CFL 5, PCG tolerance 1e-6; one step = one update(1/120) frame.
Inputs are synthetic (no dataset exists for this path).  Under torchrun each
rank runs its own replica of the scene on its own GPU (weak scaling, no
collective on the data path); the timing is max over ranks.

  value  device time of frames W+1..W+K after W untimed warm-up frames
         (CUDA events on the library's stream, L2 flushed between frames
         outside the events), particles at the start of each frame summed
         over frames and ranks.
  e2e    the same metric over the same frames through the public API with
         host buffers: a simulation loaded with the particles of frame W
         (loadMarkerParticleData + setCurrentFrame, untimed), then per frame
         update(dt) plus getMarkerParticlePositionData() into pinned host
         memory (host wall clock, device synchronised).
  plain_60  frames 1-60 of the 128^3 configuration from its seeded start.
  batched / served  the mixed-size and served scene sets (see
         run_batched_and_served); batched is compared with the same scenes
         stepped one after another through the plain step, same frames.
  --impl reference   the reference CPU path (the reference engine when it was
         compiled here, else the C++ oracle restating it) on frames W+1..W+K
         of the same workload, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
# Hardware work queues for concurrent streams (read when the CUDA context is
# created): the multi-scene runtime runs one stream per scene, and with the
# default of 8 queues streams share queues and serialise.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

FRAME_DT = 1.0 / 120.0
METRIC = "Mparticle-steps/s at 128^3 (plain FLIP step, dam break + sphere)"  # the plain_128 workload
METRICS = {"plain_128": METRIC, "plain_64": "Mparticle-steps/s at 64^3 (plain FLIP step, dam break)"}
SCENES = {
    "plain_128": "plain FLIP 128x128x128, dx=1/128, dam break + sphere, FLIP blend 0.95, PCG tol 1e-6, dt=1/120",
    "plain_64": "plain FLIP 64x64x64, dx=1/64, dam break, FLIP blend 0.95, PCG tol 1e-6, dt=1/120",
}


def make_scene(name):
    from flipengine3d_gb300 import scenes
    return getattr(scenes, name)()
UNIT = "Mparticle-steps/s"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


SWEEP_BYTES_PER_ROW = 24.0
TRAFFIC_FILE = ROOT / "profiles" / "k_wavefront_plain128.txt"


def sweep_traffic_per_launch():
    """DRAM bytes (read + write) per sweep launch from the committed ncu
    summary of this workload, or None when there is none."""
    try:
        for line in TRAFFIC_FILE.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(float(line.split(":", 1)[1]))
    except OSError:
        pass
    return None


def algorithmic_bytes(n_particles, n_cells, n_fluid, iters):
    """Per-substep algorithmic HBM bytes of the FLIP step: 120 B per particle
    (binning 48, SDF/P2G reads 24, G2P+RK3 read+write 48), 256 B per grid
    cell (SDF, flags, faces, 2x extrapolation, save, force, RHS, apply,
    2x constrain, G2P grid reads, weights) and 132 B per pressure cell per
    PCG iteration (stencil 24, two sweeps 56, three axpys 36, two dots 16)."""
    return 120.0 * n_particles + 256.0 * n_cells, 132.0 * n_fluid * iters


def combine_ranks(ms, e2e_s, particles, e2e_particles, world, device):
    """Whole-job figures of N replicas: the slowest rank's times (max) and the
    particles of all ranks (sum).  One rank: the values themselves."""
    import torch
    t = torch.tensor([ms, e2e_s], dtype=torch.float64, device=device)
    tot = torch.tensor([particles, e2e_particles], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(tot, op=torch.distributed.ReduceOp.SUM)
    return float(t[0]), float(t[1]), float(tot[0]), float(tot[1])


def timed_frames(sim, stream, steps, flush=None):
    """`steps` update(1/120) frames, each bracketed by CUDA events on the
    simulation's stream (L2 flushed before each, outside the events).
    Returns (ms, particles at the start of each frame, per-frame stats)."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    parts, frames = [], []
    for k in range(steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.zero_()
        parts.append(sim.getNumMarkerParticles())
        ev[k][0].record(stream)
        sim.update(FRAME_DT)
        ev[k][1].record(stream)
        st = sim.getFrameStatsData()
        frames.append((st.substeps, st.pressure_iterations, st.pressure_cells))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev), parts, frames


def run_gpu(args, rank, world):
    import torch

    import flipengine3d_gb300 as fg
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    sc = make_scene(args.scene)
    stream = torch.cuda.Stream()
    sim = fg.FluidSimulation.from_scene(sc)
    sim.setStream(stream.cuda_stream)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MB > 129 MB L2

    for _ in range(args.warmup):
        sim.update(FRAME_DT)
    torch.cuda.synchronize()
    # the state after warm-up: the e2e pass resumes from it, so both passes
    # (and the reference arm, which warms up the same way) time the same frames
    snap_pos = sim.getMarkerParticlePositionData().copy()
    snap_vel = sim.getMarkerParticleVelocityData().copy()
    start_frame = sim.getCurrentFrame()

    # device-timed frames
    sim.set_stage_timing(True)
    launches0 = sim.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        ms, parts, frames = timed_frames(sim, stream, args.steps, flush)
    launches = sim.launch_count() - launches0
    particles = sum(parts)
    stage_ms, substeps = sim.stage_times()
    sweep_ms, sweep_launches, sweep_rows = sim.sweep_times()
    sim.set_stage_timing(False)
    sim.close()

    # end to end through the public API with host buffers, over the same
    # frames: a fresh simulation loads the warmed-up particles from host
    # memory (loadMarkerParticleData + initialize + setCurrentFrame, untimed),
    # then each timed frame is update(dt) plus getMarkerParticlePositionData()
    # into one pinned host buffer, as a caller of the reference's
    # getMarkerParticlePositionData(char *) passes its own buffer
    e2e_sim = fg.FluidSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx)
    e2e_sim.disableSurfaceReconstruction()   # as the reference arm and `value`: the FLIP step alone
    e2e_sim.setPICFLIPRatio(sc.pic_ratio)
    e2e_sim.addBodyForce(*sc.gravity)
    e2e_sim.setCFLConditionNumber(sc.cfl)
    e2e_sim.setPressureSolveTolerance(sc.tolerance)
    e2e_sim.loadMarkerParticleData(snap_pos, snap_vel)
    e2e_sim.initialize()
    e2e_sim.setCurrentFrame(start_frame)
    e2e_sim.setStream(stream.cuda_stream)
    host = torch.empty((len(snap_pos), 3), dtype=torch.float32, pin_memory=True).numpy()
    d2h = 0
    e2e_parts, e2e_frames = [], []
    torch.cuda.synchronize()
    syncs0 = e2e_sim.host_sync_count()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_parts.append(e2e_sim.getNumMarkerParticles())
        e2e_sim.update(FRAME_DT)
        pos = e2e_sim.getMarkerParticlePositionData(out=host)
        d2h += pos.nbytes
        st = e2e_sim.getFrameStatsData()
        e2e_frames.append((st.substeps, st.pressure_iterations, st.pressure_cells))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    host_syncs = e2e_sim.host_sync_count() - syncs0
    e2e_sim.close()
    e2e_particles = sum(e2e_parts)
    same_window = e2e_parts == parts and e2e_frames == frames

    ms_max, e2e_max, ptot, e2e_ptot = combine_ranks(ms, e2e_s, particles, e2e_particles, world, "cuda")
    psub = sum(p * f[0] for p, f in zip(parts, frames)) * world
    if rank != 0:
        return None
    value = ptot / (ms_max / 1e3) / 1e6
    e2e_value = e2e_ptot / e2e_max / 1e6

    # roofline of the dominant kernel: the MIC(0) sweeps, event-timed per
    # launch on the simulation's stream inside the library
    peak, peak_kind = peaks()
    n_cells = sc.isize * sc.jsize * sc.ksize
    n_avg = particles / args.steps
    iters = [f[1] for f in frames]
    cells = [f[2] for f in frames]
    base_b, pcg_b = algorithmic_bytes(n_avg, n_cells, np.mean(cells), np.mean(iters))
    sweep_bytes_per_launch = SWEEP_BYTES_PER_ROW * sweep_rows / max(sweep_launches, 1)
    sweep_s_per_launch = sweep_ms / 1e3 / max(sweep_launches, 1)
    achieved = sweep_bytes_per_launch / sweep_s_per_launch / 1e9 if sweep_launches else 0.0
    step_achieved = (base_b + pcg_b) * substeps / (sum(stage_ms.values()) / 1e3) / 1e9

    cpu = cpu_baseline(args) if not args.no_cpu_baseline else None
    surface = run_surface(args, fg, stream) if world == 1 else None
    plain60 = run_full_length(args, fg, stream, flush) if (not args.no_full_length and world == 1) else None
    batched = served = None
    if not args.no_batched and world == 1:
        batched, served = run_batched_and_served(args)
    line = {
        "metric": METRICS[args.scene], "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 dots/refinement)",
        "data": "synthetic: seeded dam break + sphere, 8 jittered particles per cell",
        "config": {"workload": SCENES[args.scene], "particles": int(n_avg), "grid": [sc.isize, sc.jsize, sc.ksize],
                   "frames_timed": [start_frame + 1, start_frame + args.steps],
                   "substeps_per_frame": [f[0] for f in frames],
                   "pcg_iterations_per_frame": iters,
                   "pressure_cells": int(np.mean(cells)), "pcg_iterations_mean": float(np.mean(iters)),
                   "mparticle_substeps_per_s": round(psub / (ms_max / 1e3) / 1e6, 4),
                   "l2": "flushed between timed frames (256 MB write, outside the events)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": 8,
                "d2h_bytes_per_step": int(d2h / args.steps),
                "frames_timed": [start_frame + 1, start_frame + args.steps],
                "same_frames_as_value": same_window,
                "path": "FluidSimulation.update(dt) + getMarkerParticlePositionData(out=pinned host buffer) via the C "
                        "ABI, on a simulation loaded with the warmed-up particles (loadMarkerParticleData + "
                        "setCurrentFrame, untimed)",
                "timing": "wall clock over back-to-back frames, device synchronised at both ends (no L2 flush "
                          "between frames; the step's working set is larger than L2)"},
        "roofline": {"bound": "hbm", "kernel": "k_wavefront (MIC(0) forward + backward sweeps)",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": sweep_traffic_per_launch(),
                     "peak_source": peak_kind,
                     "bytes_per_launch": round(sweep_bytes_per_launch), "launches": int(sweep_launches),
                     "avg_launch_us": round(sweep_s_per_launch * 1e6, 2),
                     "share_of_step": round(sweep_ms / ms, 4) if ms else None,
                     "bytes_rule": f"{SWEEP_BYTES_PER_ROW:g} B per pressure row per sweep (factor row 16, rhs 4, result 4)",
                     "step_achieved_gbs": round(step_achieved, 1),
                     "step_frac": round(step_achieved / peak, 5),
                     "stage_ms_per_step": {k: round(v / args.steps, 3) for k, v in stage_ms.items()}},
        "cpu_baseline": cpu,
        "plain_60": plain60,
        "surface": surface,
        "batched": batched,
        "served": served,
        "gpu_launches": int(launches),
        "launches_per_frame": round(launches / args.steps, 1),
        # the library's waits on the device per frame in the e2e pass (the
        # API path, the positions' readback included), and per substep
        "host_syncs_per_frame": round(host_syncs / args.steps, 1),
        "host_syncs_per_substep": round(host_syncs / max(1, sum(f[0] for f in e2e_frames)), 1),
        "clocks": clocks.summary(),
    }
    return line


def run_surface(args, fg, stream, reps=5):
    """getIsomesh at the benchmark workload: the 128^3 state after the
    warm-up frames, meshed at subdivision levels 1 and 2 (FluidManager uses 2)
    `reps` times each; wall clock per mesh with the device synchronised (the
    mesher synchronises twice to size its outputs)."""
    import torch
    sc = make_scene(args.scene)
    sim = fg.FluidSimulation.from_scene(sc)
    sim.setStream(stream.cuda_stream)
    for _ in range(args.warmup):
        sim.update(FRAME_DT)
    out = {"particles": sim.getNumMarkerParticles()}
    for level in (1, 2):
        sim.setSurfaceSubdivisionLevel(level)
        sim.buildIsomesh()   # buffers sized
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            sim.buildIsomesh()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        v, t = sim.getIsomesh()
        out[f"subdivision_{level}"] = {"ms_per_mesh": round(1e3 * float(np.median(ts)), 3), "vertices": len(v),
                                       "triangles": len(t)}
    sim.close()
    out["how"] = ("buildIsomesh() on the state after the warm-up frames; median wall clock of " + str(reps) +
                  " meshes, device synchronised; vertices and triangles bit-identical to the reference's mesher")
    return out


def run_full_length(args, fg, stream, flush):
    """The 128^3 configuration over its full length: frames 1-60 from the
    seeded start, each event-timed as `value` is (L2 flushed between)."""
    if args.scene != "plain_128":
        return None
    sc = make_scene(args.scene)
    sim = fg.FluidSimulation.from_scene(sc)
    sim.setStream(stream.cuda_stream)
    ms, parts, frames = timed_frames(sim, stream, sc.steps, flush)
    sim.close()
    return {"value": round(sum(parts) / (ms / 1e3) / 1e6, 4), "unit": UNIT, "frames": sc.steps,
            "ms_per_frame": round(ms / sc.steps, 3), "substeps": sum(f[0] for f in frames),
            "pcg_iterations_mean": round(float(np.mean([f[1] for f in frames])), 2),
            "particles_first_last": [parts[0], parts[-1]],
            "timing": "frames 1-60 from the seeded start, CUDA events per frame, L2 flushed between frames"}


def mixed_scenes(count, seed=1):
    from flipengine3d_gb300.scenes import mixed_scene
    return [mixed_scene(q, count, seed) for q in range(count)]


def resident_scenes(rt, make, count, threads=16):
    """Create `count` scenes through the runtime's admission by free HBM: the
    host generates the particles on `threads` threads, and each scene is
    admitted and made resident in order.  Returns (simulations, rejected)."""
    from concurrent.futures import ThreadPoolExecutor

    import flipengine3d_gb300 as fg
    sims, rejected = [], 0
    with ThreadPoolExecutor(max_workers=threads) as ex:
        for first in range(0, count, 2 * threads):   # a bounded number of scenes on the host at once
            for sc in ex.map(make, range(first, min(count, first + 2 * threads))):
                need = fg.estimate_device_bytes(sc.isize, sc.jsize, sc.ksize, sc.num_particles)
                if not rt.admit(need):
                    rejected += 1
                    continue
                sims.append(fg.FluidSimulation.from_scene(sc, tuned=True))
    return sims, rejected


def run_batched_and_served(args):
    """Many resident scenes on one GPU through the C++ runtime (one CUDA
    stream per scene, args.workers host threads).

    Batched: the mixed-size set, stepped together (update_all) and, as the
    comparison, the same set stepped one scene after another through the
    plain single-scene step; both wall-clock timed over the same frames
    (args.warmup untimed, then args.batch_steps).  Served: the served set of
    args.served_scenes resident scenes; capacity = one-step requests per
    second that update_all sustains over it; Poisson arrivals of one-step
    requests for random scenes at fractions of that capacity and at the
    configured rate, latency from submission to completion."""
    import torch

    import flipengine3d_gb300 as fg
    dt = FRAME_DT
    rt = fg.FluidRuntime(workers=args.workers, reserve_bytes=2 << 30)

    def timed_rounds(handles, step_all):
        for _ in range(args.warmup):
            step_all(handles)
        torch.cuda.synchronize()
        parts, frames = 0, 0
        t0 = time.perf_counter()
        for _ in range(args.batch_steps):
            parts += sum(s.getNumMarkerParticles() for s in handles)
            step_all(handles)
        torch.cuda.synchronize()
        return parts, time.perf_counter() - t0

    def sequential(handles):
        for h in handles:
            h.update(dt)

    out = {}
    for mode, step_all in (("plain_sequential", sequential), ("batched", lambda hs: rt.update_all(hs, dt))):
        scs = mixed_scenes(args.batch_scenes)
        handles, rejected = resident_scenes(rt, lambda q: scs[q], len(scs))
        del scs
        parts, t = timed_rounds(handles, step_all)
        out[mode] = (parts, t, len(handles), rejected)
        for h in handles:
            h.close()
        torch.cuda.synchronize()
    (pp, pt, _, _), (bp, bt, nb, rejected) = out["plain_sequential"], out["batched"]
    plain_seq = pp / pt / 1e6
    bval = bp / bt / 1e6
    batched = {"value": round(bval, 3), "unit": UNIT, "scenes": nb, "rejected_at_admission": rejected,
               "particles": int(bp / args.batch_steps), "steps": args.batch_steps,
               "frames_timed": [args.warmup + 1, args.warmup + args.batch_steps],
               "ms_per_step": round(bt / args.batch_steps * 1e3, 2), "workers": args.workers,
               "plain_sequential": {"value": round(plain_seq, 3), "unit": UNIT,
                                    "ms_per_step": round(pt / args.batch_steps * 1e3, 2),
                                    "how": "the same scenes and frames, each scene stepped in turn through the "
                                           "plain single-scene update(dt) on one stream"},
               "vs_plain": round(bval / plain_seq, 3) if plain_seq else None,
               "timing": "wall clock around each round (all scenes one frame), device synchronised at both ends",
               "config": "mixed sizes: edges from {32,48,64,80,96} (seed 1), dam x-fill U[0.2,0.6], y<=0.6, "
                         "8 particles per cell, FLIP blend 0.95, PCG tol 1e-6, dt=1/120; one stream per scene"}

    # served: the served set resident; capacity, then Poisson arrivals
    from flipengine3d_gb300.scenes import served_scene
    handles, srejected = resident_scenes(rt, served_scene, args.served_scenes)
    for _ in range(max(args.warmup, 1)):
        rt.update_all(handles, dt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cap_rounds = 2
    for _ in range(cap_rounds):
        rt.update_all(handles, dt)
    torch.cuda.synchronize()
    capacity = cap_rounds * len(handles) / (time.perf_counter() - t0)   # one-step requests per second
    sizes = [s.getNumMarkerParticles() for s in handles]
    rng = np.random.default_rng(7)

    def load_point(rate, requests):
        gaps = rng.exponential(1.0 / rate, size=requests)
        picks = rng.integers(0, len(handles), size=requests)
        ids = []
        t0 = time.perf_counter()
        due = t0
        for g, q in zip(gaps, picks):
            due += g
            while time.perf_counter() < due:
                pass
            ids.append(rt.submit(handles[q], dt))
        lat = np.array([rt.wait(i)[0] for i in ids])
        ts = time.perf_counter() - t0
        return {"arrival_rate_hz": round(rate, 1), "requests": requests,
                "p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
                "value": round(float(sum(sizes[q] for q in picks)) / ts / 1e6, 3),
                "completed_per_s": round(requests / ts, 1)}

    curve = []
    for frac in (0.25, 0.5, 0.8, 1.0):
        rate = frac * capacity
        pt_ = load_point(rate, max(50, min(args.requests, int(rate * 2.0))))
        pt_["load_fraction"] = frac
        curve.append(pt_)
    main = load_point(args.arrival_rate, args.requests)
    at80 = next(c for c in curve if c["load_fraction"] == 0.8)
    served = {"p50_ms": main["p50_ms"], "p99_ms": main["p99_ms"], "requests": args.requests,
              "arrival_rate_hz": args.arrival_rate, "value": main["value"], "unit": UNIT,
              "capacity_steps_s": round(capacity, 1),
              "p50_ms_at_80pct": at80["p50_ms"], "p99_ms_at_80pct": at80["p99_ms"],
              "saturation_curve": curve,
              "resident_scenes": len(handles), "rejected_at_admission": srejected,
              "resident_particles": int(sum(sizes)), "workers": args.workers,
              "config": "edges uniform in [32,160] (seed 2), dam x-fill U[0.2,0.6], y<=0.6, 4-8 particles per "
                        "cell, FLIP blend 0.95, PCG tol 1e-5, dt=1/120; one stream per scene",
              "note": "latency = submission to completion (queueing included); one-step requests; capacity = "
                      "requests/s that update_all over all resident scenes sustains; the configured rate is "
                      "above capacity, so its latency is mostly queueing"}
    rt.close()
    for s in handles:
        s.close()
    return batched, served


def cpu_sample_sim(args, threads):
    """The reference CPU path on one bounded sample of the workload."""
    from oracle import refsim
    sc = make_scene(args.scene)
    if refsim.available("ref"):
        kind, cls = "reference", refsim.RefSimulation
    else:   # the C++ restatement, threaded where the reference threads
        kind, cls = "port", refsim.OracleSimulation
    sim = cls(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=threads).setup(sc)
    return sc, sim, kind, threads


def cpu_baseline(args):
    """The reference CPU path on the machine's host cores: the GPU arm's frames
    after the same warm-up, a bounded number of them (args.cpu_frames)."""
    threads = os.cpu_count() or 1
    sc, sim, kind, threads = cpu_sample_sim(args, threads)
    for _ in range(args.warmup):
        sim.update(FRAME_DT)
    total, t = 0, 0.0
    frames = max(1, min(args.steps, args.cpu_frames))
    for _ in range(frames):
        total += sim.particles()[0].shape[0]
        t0 = time.perf_counter()
        sim.update(FRAME_DT)
        t += time.perf_counter() - t0
    return {"value": round(total / t / 1e6, 5), "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"frames {args.warmup + 1}-{args.warmup + frames} of the {args.scene} workload (the first "
                      f"{frames} of the GPU arm's timed frames) after {args.warmup} untimed, {t:.1f} s"}


def run_reference(args, rank, world):
    """The reference CPU path on the GPU arm's frames: args.warmup untimed
    frames, then args.steps timed ones (capped at args.reference_max_steps)."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    sc, sim, kind, threads = cpu_sample_sim(args, threads)
    steps = max(1, min(args.steps, args.reference_max_steps))
    for _ in range(args.warmup):
        sim.update(FRAME_DT)
    total, psub, t = 0, 0, 0.0
    substeps = []
    for _ in range(steps):
        n = sim.particles()[0].shape[0]
        t0 = time.perf_counter()
        sim.update(FRAME_DT)
        t += time.perf_counter() - t0
        total += n
        substeps.append(int(sim.L.ref_frame_substeps(sim.h)))
        psub += n * substeps[-1]
    value = total / t / 1e6
    sample = (f"frames {args.warmup + 1}-{args.warmup + steps} of the {args.scene} workload after {args.warmup} "
              f"untimed, {'reference engine' if kind == 'reference' else 'C++ oracle restating it'}, "
              f"{threads} thread(s)")
    return {"metric": METRICS[args.scene], "value": round(value, 5), "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": args.warmup, "ms_per_step": round(t / steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic: seeded dam break + sphere",
            "config": {"workload": SCENES[args.scene], "frames_timed": [args.warmup + 1, args.warmup + steps],
                       "substeps_per_frame": substeps,
                       "mparticle_substeps_per_s": round(psub / t / 1e6, 5)},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-max-steps", type=int, default=60)
    ap.add_argument("--cpu-frames", type=int, default=3, help="timed frames of the GPU arm's cpu_baseline")
    ap.add_argument("--no-full-length", action="store_true", help="skip the 60-frame 128^3 timing")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--requests", type=int, default=800)
    ap.add_argument("--served-scenes", type=int, default=256)
    ap.add_argument("--arrival-rate", type=float, default=2000.0)
    ap.add_argument("--surface-only", action="store_true",
                    help="only the getIsomesh timing (a short run for profiling the mesher)")
    ap.add_argument("--scene", default="plain_128", choices=sorted(SCENES),
                    help="plain_128 is the benchmark workload; plain_64 is the small case for profiling")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "gb300":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    if args.surface_only:
        import torch
        import flipengine3d_gb300 as fg
        line = {"surface": run_surface(args, fg, torch.cuda.Stream())}
    elif args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_gpu(args, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1 and args.impl == "gb300":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
