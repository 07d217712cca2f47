"""GPU: the bounded device waits give up, report, and leave the simulation
usable.  No GPU fault, trap or hang is involved: the sweeps' tiles are made
to await edge terms under an epoch that no tile publishes (a flag nothing
sets), with a short poll limit, so each wait ends at its limit and sets the
error flag the host reads (FLIP_E_DEVICE_TIMEOUT).  The host then clears the
exchange state; the next update runs the frame afresh and matches the
oracle."""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import rel_err
from flipengine3d_gb300 import FlipDeviceTimeout, FluidSimulation
from flipengine3d_gb300.scenes import dam_break
from oracle import refsim

pytestmark = pytest.mark.gpu


def test_sweep_wait_times_out_and_the_next_update_recovers(gpu):
    sc = dam_break(40, seed=8)   # several sweep tiles, so tiles wait on neighbours
    orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    orc.update(sc.frame_dt)
    with FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
        sim.set_device_wait_limit(4096)
        sim.inject_sweep_stall(True)
        t0 = time.perf_counter()
        with pytest.raises(FlipDeviceTimeout):
            sim.update(sc.frame_dt)
        assert time.perf_counter() - t0 < 30.0, "the waits must end at their short limit"
        assert sim.getCurrentFrame() == 0, "a frame that timed out is not counted"
        sim.inject_sweep_stall(False)
        sim.set_device_wait_limit(0)
        sim.update(sc.frame_dt)
        pos = sim.getMarkerParticlePositionData()
        rpos, _ = orc.particles()
        assert pos.shape == rpos.shape
        assert rel_err(pos, rpos) <= 1e-5
        assert sim.getFrameStatsData().pressure_status == 0
        # and the one after that, with the default limit, too
        sim.update(sc.frame_dt)
        orc.update(sc.frame_dt)
        assert rel_err(sim.getMarkerParticlePositionData(), orc.particles()[0]) <= 1e-4
