#!/usr/bin/env python3
"""FLIP step benchmark on GB300: Mparticle-steps/s at 128^3.

Workload (N=1): the 128^3 plain FLIP dam break (dx = 1/128, fluid box
x<0.4, y<0.6, 8 jittered particles per cell, seed 0) plus a falling sphere
(r = 0.15 at (0.7, 0.7, 0.5), v = (0, -2, 0)), FLIP blend 0.95, gravity
-9.81, CFL 5, PCG tolerance 1e-6; one step = one update(1/120) frame.
Inputs are synthetic (no dataset exists for this path).  Under torchrun each
rank runs its own replica of the scene on its own GPU (weak scaling, no
collective on the data path); the timing is max over ranks.

  value  device time of K frames (CUDA events on the library's stream,
         L2 flushed between frames outside the events), particles at the
         start of each frame summed over frames and ranks.
  e2e    the same metric through the public API with host buffers: each
         frame is update(dt) plus getMarkerParticlePositionData() into host
         memory (host wall clock, device synchronised).
  --impl reference   the reference CPU path (the reference engine when it was
         compiled here, else the C++ oracle restating it) on a bounded sample
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

    # device-timed frames
    sim.set_stage_timing(True)
    launches0 = sim.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    particles = 0
    iters, cells = [], []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            particles += sim.getNumMarkerParticles()
            ev[k][0].record(stream)
            sim.update(FRAME_DT)
            ev[k][1].record(stream)
            st = sim.getFrameStatsData()
            iters.append(st.pressure_iterations)
            cells.append(st.pressure_cells)
        torch.cuda.synchronize()
    launches = sim.launch_count() - launches0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    stage_ms, substeps = sim.stage_times()
    sweep_ms, sweep_launches, sweep_rows = sim.sweep_times()
    sim.set_stage_timing(False)

    # end to end through the public API with host buffers: the positions go
    # into one pinned host buffer, as a caller of the reference's
    # getMarkerParticlePositionData(char *) passes its own buffer
    d2h = 0
    host = torch.empty((sim.getNumMarkerParticles(), 3), dtype=torch.float32, pin_memory=True).numpy()
    torch.cuda.synchronize()
    e2e_particles = 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_particles += sim.getNumMarkerParticles()
        sim.update(FRAME_DT)
        pos = sim.getMarkerParticlePositionData(out=host)
        d2h += pos.nbytes
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    ms_max, e2e_max, ptot, e2e_ptot = combine_ranks(ms, e2e_s, particles, e2e_particles, world, "cuda")
    if rank != 0:
        return None
    value = ptot / (ms_max / 1e3) / 1e6
    e2e_value = e2e_ptot / e2e_max / 1e6

    # roofline of the dominant kernel: the MIC(0) sweeps, event-timed per
    # launch on the simulation's stream inside the library
    peak, peak_kind = peaks()
    n_cells = sc.isize * sc.jsize * sc.ksize
    n_avg = particles / args.steps
    base_b, pcg_b = algorithmic_bytes(n_avg, n_cells, np.mean(cells), np.mean(iters))
    sweep_bytes_per_launch = SWEEP_BYTES_PER_ROW * sweep_rows / max(sweep_launches, 1)
    sweep_s_per_launch = sweep_ms / 1e3 / max(sweep_launches, 1)
    achieved = sweep_bytes_per_launch / sweep_s_per_launch / 1e9 if sweep_launches else 0.0
    step_achieved = (base_b + pcg_b) * substeps / (sum(stage_ms.values()) / 1e3) / 1e9

    cpu = cpu_baseline(args) if not args.no_cpu_baseline else None
    batched = served = None
    if not args.no_batched and world == 1:
        sim.close()   # free the plain scene's memory first
        batched, served = run_batched_and_served(args, value)
    line = {
        "metric": METRICS[args.scene], "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 dots/refinement)",
        "data": "synthetic: seeded dam break + sphere, 8 jittered particles per cell",
        "config": {"workload": SCENES[args.scene], "particles": int(n_avg), "grid": [sc.isize, sc.jsize, sc.ksize],
                   "pressure_cells": int(np.mean(cells)), "pcg_iterations_mean": float(np.mean(iters)),
                   "l2": "flushed between timed frames (256 MB write, outside the events)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": 8,
                "d2h_bytes_per_step": int(d2h / args.steps),
                "path": "FluidSimulation.update(dt) + getMarkerParticlePositionData(out=pinned host buffer) via the C ABI",
                "timing": "wall clock over back-to-back frames (no L2 flush between them; the step's working set "
                          "is larger than L2), where `value` flushes L2 between event-timed frames"},
        "roofline": {"bound": "hbm", "kernel": "k_wavefront (MIC(0) forward + backward sweeps)",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 5), "traffic": sweep_traffic_per_launch(),
                     "peak_source": peak_kind,
                     "bytes_per_launch": round(sweep_bytes_per_launch), "launches": int(sweep_launches),
                     "avg_launch_us": round(sweep_s_per_launch * 1e6, 2),
                     "share_of_step": round(sweep_ms / ms, 4) if ms else None,
                     "bytes_rule": f"{SWEEP_BYTES_PER_ROW:g} B per pressure row per sweep (factor row 16, rhs 4, result 4)",
                     "step_achieved_gbs": round(step_achieved, 1),
                     "stage_ms_per_step": {k: round(v / args.steps, 3) for k, v in stage_ms.items()}},
        "cpu_baseline": cpu,
        "batched": batched,
        "served": served,
        "gpu_launches": int(launches),
        "clocks": clocks.summary(),
    }
    return line


def mixed_scenes(count, seed=1):
    """The mixed-size scene set: cubic grids with edges drawn from
    {32, 48, 64, 80, 96} (dx = 1/edge), each a dam break whose x extent
    (the fill fraction) is drawn from [0.2, 0.6], y <= 0.6, full z, 8 jittered
    particles per cell, FLIP blend 0.95."""
    return [mixed_scene(q, count, seed) for q in range(count)]


def mixed_scene_params(count, seed=1):
    """(edge, fill) of each scene of the mixed-size set, without its particles."""
    rng = np.random.default_rng(seed)
    edges = rng.choice([32, 48, 64, 80, 96], size=count)
    fills = rng.uniform(0.2, 0.6, size=count)
    return [(int(e), float(f)) for e, f in zip(edges, fills)]


def mixed_scene(q, count=64, seed=1):
    """Scene q of the mixed-size set."""
    from flipengine3d_gb300.scenes import dam_break
    e, f = mixed_scene_params(count, seed)[q]
    return dam_break(e, seed=seed * 1000 + q, fill=(f, 0.6, 1.0))


def served_scene(q, seed=2):
    """Scene q of the served set: a cubic grid with its edge drawn uniformly
    from [32, 160] (dx = 1/edge), a dam break whose x extent is drawn from
    [0.2, 0.6], y <= 0.6, full z, 4-8 jittered particles per cell (drawn per
    scene), FLIP blend 0.95, PCG tolerance 1e-5."""
    from flipengine3d_gb300.scenes import dam_break
    rng = np.random.default_rng([seed, q])
    edge = int(rng.integers(32, 161))
    fill = float(rng.uniform(0.2, 0.6))
    ppc = int(rng.integers(4, 9))
    return dam_break(edge, seed=seed * 100000 + q, fill=(fill, 0.6, 1.0), ppc=ppc, tolerance=1e-5)


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
                sims.append(fg.FluidSimulation.from_scene(sc))
    return sims, rejected


def run_batched_and_served(args, plain_value):
    """Many resident scenes on one GPU through the C++ runtime (one CUDA
    stream per scene, args.workers host threads).  Batched: the mixed-size
    set, every scene one step per round (update_all), wall-clock timed over
    args.batch_steps rounds.  Served: the served set of args.served_scenes
    resident scenes, Poisson arrivals of one-step requests for random
    scenes, latency from submission to completion."""
    import torch

    import flipengine3d_gb300 as fg
    scs = mixed_scenes(args.batch_scenes)
    rt = fg.FluidRuntime(workers=args.workers, reserve_bytes=2 << 30)
    handles, rejected = resident_scenes(rt, lambda q: scs[q], len(scs))
    del scs
    dt = FRAME_DT
    for _ in range(max(args.warmup, 1)):
        rt.update_all(handles, dt)
    torch.cuda.synchronize()
    parts = 0
    t0 = time.perf_counter()
    for _ in range(args.batch_steps):
        parts += sum(s.getNumMarkerParticles() for s in handles)
        rt.update_all(handles, dt)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t0
    bval = parts / tb / 1e6
    batched = {"value": round(bval, 3), "unit": UNIT, "scenes": len(handles), "rejected_at_admission": rejected,
               "particles": int(parts / args.batch_steps), "steps": args.batch_steps,
               "ms_per_step": round(tb / args.batch_steps * 1e3, 2), "workers": args.workers,
               "vs_plain": round(bval / plain_value, 3) if plain_value else None,
               "timing": "wall clock around update_all (all scenes one frame), device synchronised",
               "config": "mixed sizes: edges from {32,48,64,80,96} (seed 1), dam x-fill U[0.2,0.6], y<=0.6, "
                         "8 particles per cell, FLIP blend 0.95, PCG tol 1e-6, dt=1/120; one stream per scene"}
    for s in handles:
        s.close()
    torch.cuda.synchronize()
    # served: Poisson arrivals over the served set
    handles, srejected = resident_scenes(rt, served_scene, args.served_scenes)
    for _ in range(max(args.warmup, 1)):
        rt.update_all(handles, dt)
    torch.cuda.synchronize()
    rng = np.random.default_rng(7)
    gaps = rng.exponential(1.0 / args.arrival_rate, size=args.requests)
    picks = rng.integers(0, len(handles), size=args.requests)
    sizes = [s.getNumMarkerParticles() for s in handles]
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
    served = {"p50_ms": round(float(np.percentile(lat, 50)), 2), "p99_ms": round(float(np.percentile(lat, 99)), 2),
              "requests": args.requests, "arrival_rate_hz": args.arrival_rate,
              "value": round(float(sum(sizes[q] for q in picks)) / ts / 1e6, 3), "unit": UNIT,
              "resident_scenes": len(handles), "rejected_at_admission": srejected,
              "resident_particles": int(sum(sizes)), "workers": args.workers,
              "config": "edges uniform in [32,160] (seed 2), dam x-fill U[0.2,0.6], y<=0.6, 4-8 particles per "
                        "cell, FLIP blend 0.95, PCG tol 1e-5, dt=1/120; one stream per scene",
              "note": "latency = submission to completion (queueing included); one-step requests"}
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
    threads = os.cpu_count() or 1
    sc, sim, kind, threads = cpu_sample_sim(args, threads)
    sim.update(FRAME_DT)                       # first frame builds the solid level set: untimed
    n = sim.particles()[0].shape[0]
    t0 = time.perf_counter()
    sim.update(FRAME_DT)
    dt = time.perf_counter() - t0
    return {"value": round(n / dt / 1e6, 5), "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"1 timed frame of the {args.scene} workload ({n} particles) after 1 untimed frame, {dt:.1f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    sc, sim, kind, threads = cpu_sample_sim(args, threads)
    steps = max(1, min(args.steps, args.reference_max_steps))
    warm = max(0, min(args.warmup, 1))
    for _ in range(warm):
        sim.update(FRAME_DT)
    total, t = 0, 0.0
    for _ in range(steps):
        n = sim.particles()[0].shape[0]
        t0 = time.perf_counter()
        sim.update(FRAME_DT)
        t += time.perf_counter() - t0
        total += n
    value = total / t / 1e6
    sample = (f"{steps} timed frame(s) of the {args.scene} workload after {warm} untimed, "
              f"{'reference engine' if kind == 'reference' else 'C++ oracle restating it'}, {threads} thread(s)")
    return {"metric": METRICS[args.scene], "value": round(value, 5), "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": warm, "ms_per_step": round(t / steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/f64", "data": "synthetic: seeded dam break + sphere",
            "config": {"workload": SCENES[args.scene]},
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
    ap.add_argument("--reference-max-steps", type=int, default=3)
    ap.add_argument("--no-batched", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--requests", type=int, default=800)
    ap.add_argument("--served-scenes", type=int, default=256)
    ap.add_argument("--arrival-rate", type=float, default=2000.0)
    ap.add_argument("--scene", default="plain_128", choices=sorted(SCENES),
                    help="plain_128 is the benchmark workload; plain_64 is the small case for profiling")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "gb300":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
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
