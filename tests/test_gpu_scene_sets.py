"""GPU against the oracle on scenes of the multi-scene sets, alone and
inside the runtime.

* Batched set (mixed sizes): the first scenes with edges 32, 64 and 96
  (8 particles per cell, fills 0.2-0.6, tolerance 1e-6).
* Served set: the first scene with an edge above 128 and 4 particles per
  cell (tolerance 1e-5).

Each scene: two frames through update(), positions within 1e-5 relative of
the oracle after the first frame and 1e-4 after the second, the same
particle counts, PCG iteration counts within one of the oracle's; then the
same scenes stepped together through the runtime (update_all) give the
results of the scenes alone, bit for bit.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import rel_err
from flipengine3d_gb300 import FluidRuntime, FluidSimulation
from flipengine3d_gb300 import scenes
from oracle import refsim

pytestmark = pytest.mark.gpu

RTOL = 1e-5
RTOL_MULTI = 1e-4
FRAMES = 2
THREADS = os.cpu_count() or 1


def chosen_scenes():
    params = scenes.mixed_scene_params(64)
    out = [scenes.mixed_scene(next(q for q, (e, _) in enumerate(params) if e == edge)) for edge in (32, 64, 96)]
    q = next(q for q in range(256) if scenes.served_scene_params(q)[0] > 128 and scenes.served_scene_params(q)[2] == 4)
    out.append(scenes.served_scene(q))
    return out


def test_scene_sets_match_oracle_alone_and_in_the_runtime(gpu):
    scs = chosen_scenes()
    alone = []
    for sc in scs:
        orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=THREADS).setup(sc)
        with FluidSimulation.from_scene(sc) as sim:
            for f in range(FRAMES):
                sim.update(sc.frame_dt)
                orc.update(sc.frame_dt)
                pos = sim.getMarkerParticlePositionData()
                rpos, _ = orc.particles()
                label = f"{sc.name} (tol {sc.tolerance:g}) frame {f + 1}"
                assert pos.shape == rpos.shape, f"{label}: particle count"
                assert rel_err(pos, rpos) <= (RTOL if f == 0 else RTOL_MULTI), f"{label}: positions"
                gi = sim.getFrameStatsData().pressure_iterations
                oi = orc.L.ref_last_pcg_iters(orc.h)
                assert abs(gi - oi) <= 1, f"{label}: PCG iterations {gi} vs the oracle's {oi}"
            alone.append((sim.getMarkerParticlePositionData(), sim.getMarkerParticleVelocityData()))
        orc.close()
    sims = [FluidSimulation.from_scene(sc) for sc in scs]
    try:
        with FluidRuntime(workers=4) as rt:
            for _ in range(FRAMES):
                rt.update_all(sims, scs[0].frame_dt)
        for q, sim in enumerate(sims):
            assert np.array_equal(sim.getMarkerParticlePositionData(), alone[q][0]), f"{scs[q].name}: in the mix"
            assert np.array_equal(sim.getMarkerParticleVelocityData(), alone[q][1]), f"{scs[q].name}: in the mix"
    finally:
        for s in sims:
            s.close()
