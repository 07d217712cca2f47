"""Tuning knobs (flip_set_tuning) and the autotuner's table.

* CPU: the table lookup (nearest edge, defaults without a table) and the
  committed table's shape when there is one.
* GPU: the knobs' argument checks; the liquid SDF is bit-identical for every
  CTA size; another PCG reduction grid moves positions only in the last bits;
  a pinned sweep orientation gives the same results as the per-solve choice.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from flipengine3d_gb300 import autotune
from flipengine3d_gb300 import fluidsimulation as fs
from flipengine3d_gb300.scenes import dam_break


def test_lookup_nearest_edge_and_defaults():
    table = [dict(edge=32, sdf_threads=256, pcg_cells_per_cta=1024, sweep_orientation=0),
             dict(edge=128, sdf_threads=1024, pcg_cells_per_cta=8192, sweep_orientation=1)]
    assert autotune.lookup(30, 30, 30, table)["sdf_threads"] == 256
    assert autotune.lookup(100, 100, 100, table)["pcg_cells_per_cta"] == 8192
    assert autotune.lookup(256, 128, 128, table)["sweep_orientation"] == 1   # cube root 161
    assert autotune.lookup(64, 64, 64, []) == autotune.DEFAULT


def test_committed_table_is_well_formed():
    table = autotune.load_table()
    if not table:
        pytest.skip("no tuning table committed")
    for e in table:
        assert e["sdf_threads"] in autotune.CANDIDATES["sdf_threads"]
        assert e["pcg_cells_per_cta"] in autotune.CANDIDATES["pcg_cells_per_cta"]
        assert e["sweep_orientation"] in autotune.CANDIDATES["sweep_orientation"]


def _run(tuning, frames=3):
    sc = dam_break(24, seed=2, sphere=True)
    with fs.FluidSimulation.from_scene(sc, tolerance=1e-9) as sim:
        sim.setTuning(**tuning)
        assert sim.getTuning() == tuning
        phis = []
        for _ in range(frames):
            sim.update(sc.frame_dt)
            phis.append(sim.liquid_sdf())
        return phis, sim.getMarkerParticlePositionData(), sim.getFrameStatsData().pressure_iterations


@pytest.mark.gpu
def test_gpu_tuning_knobs(gpu):
    with fs.FluidSimulation(8, 8, 8, 0.125) as sim:
        for bad in (dict(sdf_threads=128), dict(pcg_cells_per_cta=16), dict(sweep_orientation=2)):
            with pytest.raises(ValueError):
                sim.setTuning(**bad)
        assert sim.getTuning() == autotune.DEFAULT
    base_phi, base_pos, base_it = _run(dict(autotune.DEFAULT))
    for threads in (256, 1024):
        phi, pos, it = _run(dict(autotune.DEFAULT, sdf_threads=threads))
        assert all(np.array_equal(a, b) for a, b in zip(phi, base_phi)), threads
        assert np.array_equal(pos, base_pos) and it == base_it
    for orient in (0, 1):
        phi, pos, it = _run(dict(autotune.DEFAULT, sweep_orientation=orient))
        assert np.array_equal(pos, base_pos) and it == base_it, orient
    phi, pos, it = _run(dict(autotune.DEFAULT, pcg_cells_per_cta=1024))
    assert rel_err(pos, base_pos) <= 1e-6
