"""Many scenes on one GPU through the C++ runtime: batched (update_all) and
served (submit/wait) results equal each scene run alone, bit for bit, since
a scene's kernels and their order do not depend on the other scenes."""
from __future__ import annotations

import numpy as np
import pytest

from flipengine3d_gb300 import FluidRuntime, FluidSimulation, estimate_device_bytes
from flipengine3d_gb300.scenes import dam_break

pytestmark = pytest.mark.gpu

SCENES = [dict(n=16, seed=1), dict(n=20, seed=2, sphere=True), dict(n=24, seed=3, fill=(0.6, 0.5, 1.0)),
          dict(n=12, jsize=18, ksize=14, dx=1 / 12, seed=4)]
FRAMES = 3


def alone(kw):
    sc = dam_break(**kw)
    with FluidSimulation.from_scene(sc) as sim:
        for _ in range(FRAMES):
            sim.update(sc.frame_dt)
        return sim.getMarkerParticlePositionData(), sim.getMarkerParticleVelocityData()


def test_batched_scenes_match_alone(gpu):
    ref = [alone(kw) for kw in SCENES]
    scs = [dam_break(**kw) for kw in SCENES]
    sims = [FluidSimulation.from_scene(sc) for sc in scs]
    try:
        with FluidRuntime(workers=4) as rt:
            for _ in range(FRAMES):
                rt.update_all(sims, scs[0].frame_dt)
        for q, sim in enumerate(sims):
            pos, vel = sim.getMarkerParticlePositionData(), sim.getMarkerParticleVelocityData()
            assert np.array_equal(pos, ref[q][0]), f"scene {q}: positions differ from the scene alone"
            assert np.array_equal(vel, ref[q][1]), f"scene {q}: velocities differ from the scene alone"
    finally:
        for s in sims:
            s.close()


def test_served_requests_match_alone_and_keep_order(gpu):
    ref = [alone(kw) for kw in SCENES]
    scs = [dam_break(**kw) for kw in SCENES]
    sims = [FluidSimulation.from_scene(sc) for sc in scs]
    try:
        with FluidRuntime(workers=3) as rt:
            ids = []
            # interleaved arrivals: one step of each scene at a time, FRAMES rounds
            for _ in range(FRAMES):
                for q, sim in enumerate(sims):
                    ids.append(rt.submit(sim, scs[q].frame_dt))
            lat = [rt.wait(i) for i in ids]
        assert all(ms > 0.0 and st == 0 for ms, st in lat)
        for q, sim in enumerate(sims):
            assert np.array_equal(sim.getMarkerParticlePositionData(), ref[q][0]), f"scene {q}"
    finally:
        for s in sims:
            s.close()


def test_admission_and_device_bytes(gpu):
    sc = dam_break(20, seed=5)
    est = estimate_device_bytes(sc.isize, sc.jsize, sc.ksize, len(sc.positions))
    with FluidSimulation.from_scene(sc) as sim:
        used = sim.device_bytes()
    assert used > 0 and est >= used, (est, used)
    with FluidRuntime(workers=1, reserve_bytes=0) as rt:
        assert rt.admit(est)
        assert not rt.admit(1 << 50)   # a petabyte never fits
        with pytest.raises(ValueError):
            rt.wait(12345)
