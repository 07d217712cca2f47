"""GPU: the FluidSimulation API's error behaviour and edge cases, the way the
reference behaves (src/engine/fluidsimulation.cpp)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from flipengine3d_gb300 import FluidSimulation
from flipengine3d_gb300.scenes import dam_break
from oracle import refsim

pytestmark = pytest.mark.gpu


def test_update_before_initialize_raises_runtime_error(gpu):
    with FluidSimulation(8, 8, 8, 1 / 8) as sim:
        with pytest.raises(RuntimeError):
            sim.update(0.01)


def test_negative_dt_and_bad_ratio_raise_domain_error(gpu):
    with FluidSimulation(8, 8, 8, 1 / 8) as sim:
        sim.initialize()
        with pytest.raises(ValueError):
            sim.update(-1.0)
        with pytest.raises(ValueError):
            sim.setPICFLIPRatio(1.5)
        sim.setPICFLIPRatio(0.25)
        assert sim.getPICFLIPRatio() == 0.25


def test_empty_scene_steps(gpu):
    with FluidSimulation(12, 12, 12, 1 / 12) as sim:
        sim.addBodyForce(0, -9.81, 0)
        sim.initialize()
        for _ in range(2):
            sim.update(1 / 120)
        assert sim.getNumMarkerParticles() == 0
        assert sim.getCurrentFrame() == 2
        assert np.all(sim.liquid_sdf() == np.float32(3.0 / 12))


def test_particles_outside_the_domain_are_dropped_at_load(gpu):
    sc = dam_break(12, seed=0)
    pos = sc.positions.copy()
    pos[::2] += 3.0
    with FluidSimulation(12, 12, 12, sc.dx) as sim:
        sim.loadMarkerParticleData(pos, sc.velocities)
        sim.initialize()
        kept = pos[1::2]
        assert sim.getNumMarkerParticles() == kept.shape[0]
        assert np.array_equal(sim.getMarkerParticlePositionData(), kept)


def test_range_readback_and_errors(gpu):
    sc = dam_break(12, seed=0)
    with FluidSimulation.from_scene(sc) as sim:
        n = sim.getNumMarkerParticles()
        full = sim.getMarkerParticlePositionData()
        assert np.array_equal(sim.getMarkerParticlePositionDataRange(10, 50), full[10:50])
        with pytest.raises(ValueError):
            sim.getMarkerParticlePositionDataRange(5, n + 1)
        with pytest.raises(ValueError):
            sim.getMarkerParticleVelocityDataRange(-1, 3)


def test_single_particle_matches_oracle(gpu):
    sc = dam_break(10, seed=0)
    sc.positions = np.array([[0.5, 0.55, 0.45]], np.float32)
    sc.velocities = np.array([[0.3, -0.2, 0.1]], np.float32)
    orc = refsim.OracleSimulation(10, 10, 10, sc.dx).setup(sc, tolerance=1e-9)
    with FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
        for _ in range(3):
            sim.update(sc.frame_dt)
            orc.update(sc.frame_dt)
        rpos, rvel = orc.particles()
        assert sim.getNumMarkerParticles() == rpos.shape[0]
        assert rel_err(sim.getMarkerParticlePositionData(), rpos) <= 1e-5


def test_pressure_non_convergence_is_reported_not_raised(gpu):
    sc = dam_break(16, seed=0)
    with FluidSimulation.from_scene(sc, tolerance=1e-12) as sim:
        sim.setMaxPressureSolveIterations(1)
        sim.update(sc.frame_dt)
        st = sim.getFrameStatsData()
        assert st.pressure_iterations == 1
        assert st.pressure_status != 0
        assert sim.getNumMarkerParticles() > 0


@pytest.mark.parametrize("max_iterations", [1000, 21])
def test_device_side_pcg_loop_matches_host_batches(gpu, max_iterations):
    """Untimed solves run the PCG batches inside a device-side loop; with
    stage timing on, the host launches them batch by batch.  Both run the
    same kernels in the same order: the results are bit-identical, also when
    the iteration cap (21: two full batches and an eager tail of 5) stops the
    solve before convergence."""
    sc = dam_break(24, seed=3, sphere=True)
    out = []
    for timed in (False, True):
        with FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
            sim.setMaxPressureSolveIterations(max_iterations)
            sim.set_stage_timing(timed)
            stats = []
            for _ in range(3):
                sim.update(sc.frame_dt)
                st = sim.getFrameStatsData()
                stats.append((st.substeps, st.pressure_iterations, st.pressure_status))
            out.append((sim.getMarkerParticlePositionData(), sim.getMarkerParticleVelocityData(), stats))
    (p0, v0, s0), (p1, v1, s1) = out
    assert s0 == s1
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
    if max_iterations == 21:
        assert max(it for _, it, _ in s0) == 21


def test_nan_velocity_input_does_not_fault(gpu):
    sc = dam_break(12, seed=0)
    vel = sc.velocities.copy()
    vel[7] = np.nan
    with FluidSimulation(12, 12, 12, sc.dx) as sim:
        sim.addBodyForce(0, -9.81, 0)
        sim.loadMarkerParticleData(sc.positions, vel)
        sim.initialize()
        sim.update(sc.frame_dt)
        st = sim.getFrameStatsData()
        assert st.frame == 0


def test_launches_are_counted(gpu):
    sc = dam_break(12, seed=0)
    with FluidSimulation.from_scene(sc) as sim:
        before = sim.launch_count()
        sim.update(sc.frame_dt)
        assert sim.launch_count() > before + 20


def test_host_synchronisations_are_counted(gpu):
    """A substep waits on the device after the binning, the system build,
    the first sweep pair and each batch of PCG iterations; a readback waits
    once more."""
    sc = dam_break(12, seed=0)
    with FluidSimulation.from_scene(sc) as sim:
        sim.update(sc.frame_dt)
        before = sim.host_sync_count()
        sim.update(sc.frame_dt)
        substeps = sim.getFrameStatsData().substeps
        per_update = sim.host_sync_count() - before
        assert per_update >= 4 * substeps
        before = sim.host_sync_count()
        sim.getMarkerParticlePositionData()
        assert sim.host_sync_count() == before + 1


def test_readback_into_a_caller_buffer(gpu):
    """getMarkerParticlePositionData(char *) writes into the caller's buffer;
    the Python mirror takes one as `out` and rejects one that is too small."""
    sc = dam_break(12, seed=1)
    with FluidSimulation.from_scene(sc) as sim:
        sim.update(sc.frame_dt)
        n = sim.getNumMarkerParticles()
        ref = sim.getMarkerParticlePositionData()
        buf = np.full((n + 5, 3), -1.0, np.float32)
        got = sim.getMarkerParticlePositionData(out=buf)
        assert np.shares_memory(got, buf) and np.array_equal(got, ref)
        assert np.all(buf[n:] == -1.0)
        assert np.array_equal(sim.getMarkerParticleVelocityData(out=np.empty((n, 3), np.float32)),
                              sim.getMarkerParticleVelocityData())
        with pytest.raises(ValueError):
            sim.getMarkerParticlePositionData(out=np.empty((n - 1, 3), np.float32))
