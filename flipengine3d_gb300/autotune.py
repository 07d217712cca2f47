"""Autotuner of the device kernels' tuning knobs (flip_set_tuning).

The knobs change how work is laid on the GPU, not what is computed:

* ``sdf_threads``: the CTA size of the liquid-SDF kernel (one CTA per block
  of 10^3 cells): 256, 512 or 1024 threads;
* ``pcg_cells_per_cta``: grid cells per CTA of the PCG row kernels'
  reduction grid;
* ``sweep_orientation``: the preconditioner sweep tiles' lane axis, j (0) or
  k (1), or the per-solve choice from the rows' extent (-1).

For each grid edge the tuner builds the mixed-size set's dam break (fill 0.4,
8 particles per cell), steps it to a warm state, and times the same frames
from that state once per candidate setting (a fresh context loaded with the
warm particles each time), knob by knob: the liquid-SDF stage's device time
for ``sdf_threads``, the pressure stage's for the other two.  The best value
of each knob is kept before the next is tried.  The table it writes
(``tuning_gb300.json`` beside this file) is what
``FluidSimulation.applyTunedSettings()`` (and ``from_scene(..., tuned=True)``,
which the many-scene bench uses) applies: the entry of the nearest edge.

    python -m flipengine3d_gb300.autotune [--edges 32 64 96 128 160] [--frames 4]
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

TABLE = Path(__file__).resolve().parent / "tuning_gb300.json"
DEFAULT = {"sdf_threads": 512, "pcg_cells_per_cta": 4096, "sweep_orientation": -1}
CANDIDATES = {
    "sdf_threads": (256, 512, 1024),
    "pcg_cells_per_cta": (1024, 2048, 4096, 8192, 16384),
    "sweep_orientation": (-1, 0, 1),
}
STAGE_OF = {"sdf_threads": "liquid_sdf", "pcg_cells_per_cta": "pressure", "sweep_orientation": "pressure"}


def load_table(path: Path = TABLE):
    """The tuned entries, sorted by edge, or [] without a table."""
    if not path.exists():
        return []
    return sorted(json.loads(path.read_text())["entries"], key=lambda e: e["edge"])


def lookup(isize: int, jsize: int, ksize: int, table=None):
    """The tuning for a grid: the entry whose edge is nearest the grid's
    cube-root size, or the defaults without a table."""
    table = load_table() if table is None else table
    if not table:
        return dict(DEFAULT)
    edge = (isize * jsize * ksize) ** (1.0 / 3.0)
    best = min(table, key=lambda e: abs(e["edge"] - edge))
    return {k: int(best[k]) for k in DEFAULT}


def _warm_state(edge: int, warm: int):
    from .fluidsimulation import FluidSimulation
    from .scenes import dam_break
    sc = dam_break(edge, seed=7, fill=(0.4, 0.6, 1.0))
    sim = FluidSimulation.from_scene(sc)
    for _ in range(warm):
        sim.update(sc.frame_dt)
    state = (sim.getMarkerParticlePositionData().copy(), sim.getMarkerParticleVelocityData().copy(),
             sim.getCurrentFrame())
    sim.close()
    return sc, state


def _time(sc, state, tuning, frames):
    """Device ms per frame of each stage over `frames` frames from `state`."""
    from .fluidsimulation import FluidSimulation
    pos, vel, frame = state
    sim = FluidSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx)
    sim.disableSurfaceReconstruction()
    sim.setPICFLIPRatio(sc.pic_ratio)
    sim.addBodyForce(*sc.gravity)
    sim.setCFLConditionNumber(sc.cfl)
    sim.setPressureSolveTolerance(sc.tolerance)
    sim.loadMarkerParticleData(pos, vel)
    sim.initialize()
    sim.setCurrentFrame(frame)
    sim.setTuning(**tuning)
    sim.update(sc.frame_dt)          # one untimed frame: graphs captured, caches warm
    sim.set_stage_timing(True)
    for _ in range(frames):
        sim.update(sc.frame_dt)
    ms, _ = sim.stage_times()
    sim.close()
    return {k: v / frames for k, v in ms.items()}


def tune_edge(edge: int, frames: int = 4, warm: int = 3, log=print):
    sc, state = _warm_state(edge, warm)
    best = dict(DEFAULT)
    report = {}
    for knob, values in CANDIDATES.items():
        stage = STAGE_OF[knob]
        times = {}
        for v in values:
            t = dict(best, **{knob: v})
            times[v] = _time(sc, state, t, frames)[stage]
        best[knob] = min(times, key=times.get)
        report[knob] = {str(v): round(ms, 4) for v, ms in times.items()}
        log(f"edge {edge}: {knob} {report[knob]} -> {best[knob]}")
    return dict(edge=edge, **best, stage_ms=report)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--edges", type=int, nargs="+", default=[32, 64, 96, 128, 160])
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--out", type=Path, default=TABLE)
    a = ap.parse_args(argv)
    import torch
    t0 = time.time()
    entries = [tune_edge(e, a.frames) for e in a.edges]
    out = {"device": torch.cuda.get_device_name(0), "frames": a.frames, "seconds": round(time.time() - t0, 1),
           "how": "per knob, the stage's device time (CUDA events) over the same frames from one warm state",
           "entries": entries}
    a.out.write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
