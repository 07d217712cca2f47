"""GPU: particle binning and the removal rules.

Binning (velocityadvector.cpp:272-388 bins by block; the library bins by
cell): after initialize() and after every update() the particles on the
device are in cell order, cell = floor((double)p * (1/dx)) per axis
(grid3d.h:56-61), stable by id within a cell; the cell offsets are the
prefix sums of the per-cell counts.  Checked against keys recomputed on the
host in FP64 from the device's own positions, bit for bit, and, on the
loaded particles, against the oracle's particle cells.

Removal (fluidsimulation.cpp:4298-4353), against the oracle:
* at most 250 particles per cell, the first 250 in particle order kept;
* extreme speeds: the fastest particles removed, up to 0.05% of them and at
  most 35, in whole speed bands of CFL * dx / dt.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from flipengine3d_gb300 import FluidSimulation
from flipengine3d_gb300.scenes import dam_break
from oracle import refsim

pytestmark = pytest.mark.gpu


def host_keys(pos, dims, dx):
    I, J, K = dims
    ijk = np.floor(pos.astype(np.float64) * (1.0 / dx)).astype(np.int64)
    return ijk[:, 0] + I * (ijk[:, 1] + J * ijk[:, 2])


def check_binning(sim, label):
    pos, ids, start = sim.binned_particles()
    I, J, K = sim.dims
    keys = host_keys(pos, sim.dims, sim.dx)
    assert (keys >= 0).all() and (keys < I * J * K).all(), f"{label}: key out of the grid"
    assert (np.diff(keys) >= 0).all(), f"{label}: not in cell order"
    same = np.diff(keys) == 0
    assert (np.diff(ids.astype(np.int64))[same] > 0).all(), f"{label}: not stable by id within a cell"
    counts = np.bincount(keys, minlength=I * J * K)
    assert start[0] == 0 and np.array_equal(np.diff(start), counts), f"{label}: cell offsets"
    assert len(np.unique(ids)) == len(ids), f"{label}: repeated ids"
    # the id order is the reference's particle order: readback by id equals
    # the binned positions sorted by id
    assert np.array_equal(sim.getMarkerParticlePositionData(), pos[np.argsort(ids, kind="stable")])
    return keys


def test_binning_is_a_stable_counting_sort_by_cell(gpu):
    sc = dam_break(28, jsize=20, ksize=33, dx=1 / 28, seed=12, sphere=True, fill=(0.6, 0.5, 1.1))
    with FluidSimulation.from_scene(sc) as sim:
        keys = check_binning(sim, "after initialize")
        # loaded particles: the same cells as the oracle's keys for its particles
        orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc)
        opos, _ = orc.particles()
        assert np.array_equal(np.sort(keys), np.sort(host_keys(opos, sim.dims, sim.dx)))
        for f in range(3):
            sim.update(sc.frame_dt)
            check_binning(sim, f"frame {f + 1}")


def with_crowded_cell(sc, cell, count, seed):
    """The scene with `count` extra particles at rest inside one cell,
    appended after the others (so they come last in particle order)."""
    rng = np.random.default_rng(seed)
    extra = ((np.asarray(cell) + rng.uniform(0.05, 0.95, size=(count, 3))) * sc.dx).astype(np.float32)
    sc.positions = np.concatenate([sc.positions, extra])
    sc.velocities = np.concatenate([sc.velocities, np.zeros_like(extra)])
    return sc


def with_fast_particles(sc, count, speed, seed):
    """The scene with `count` of its particles (spread through the body)
    given a large velocity."""
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(sc.positions), size=count, replace=False)
    d = rng.normal(size=(count, 3))
    sc.velocities = sc.velocities.copy()
    sc.velocities[pick] = (speed * d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return sc


def compare_after_frames(sc, frames, label):
    orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    with FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
        for f in range(frames):
            n0 = sim.getNumMarkerParticles()
            sim.update(sc.frame_dt)
            orc.update(sc.frame_dt)
            pos = sim.getMarkerParticlePositionData()
            rpos, _ = orc.particles()
            assert pos.shape == rpos.shape, f"{label} frame {f + 1}: {pos.shape[0]} vs the oracle's {rpos.shape[0]}"
            assert rel_err(pos, rpos) <= 1e-5, f"{label} frame {f + 1}: positions"
        return n0, sim.getNumMarkerParticles(), pos, sim


def test_per_cell_cap_keeps_the_first_250(gpu):
    sc = with_crowded_cell(dam_break(24, seed=21), cell=(5, 4, 12), count=300, seed=3)
    orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    with FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
        n0 = sim.getNumMarkerParticles()
        sim.update(sc.frame_dt)
        orc.update(sc.frame_dt)
        pos = sim.getMarkerParticlePositionData()
        rpos, _ = orc.particles()
        assert pos.shape == rpos.shape, (pos.shape, rpos.shape)
        assert rel_err(pos, rpos) <= 1e-5
        _, _, start = sim.binned_particles()
        assert np.diff(start).max() == 250, "the crowded cell holds the cap"
        assert n0 - pos.shape[0] >= 300 - 250 + 8, "the crowded cell lost its particles beyond the cap"


def test_extreme_speed_removal(gpu):
    sc = with_fast_particles(dam_break(24, seed=22), count=9, speed=400.0, seed=5)
    n = len(sc.positions)
    assert 9 <= min(int(n * 0.0005), 35), "the scene must allow the removal of all fast particles"
    orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    with FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
        n0 = sim.getNumMarkerParticles()
        sim.update(sc.frame_dt)
        orc.update(sc.frame_dt)
        pos = sim.getMarkerParticlePositionData()
        vel = sim.getMarkerParticleVelocityData()
        rpos, rvel = orc.particles()
        assert sim.getFrameStatsData().substeps == orc.L.ref_frame_substeps(orc.h)
        assert pos.shape == rpos.shape, (pos.shape, rpos.shape)
        assert rel_err(pos, rpos) <= 1e-4 and rel_err(vel, rvel) <= 1e-4
        assert np.linalg.norm(vel, axis=1).max() < 400.0, "the fast particles were removed"
        assert n0 > pos.shape[0]
