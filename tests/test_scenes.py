"""Host-side scene generation: the seeded inputs every other test and the
bench use (8 jittered particles per cell, as the reference seeds fluid,
src/engine/fluidsimulation.cpp:4522-4562)."""
from __future__ import annotations

import numpy as np

from flipengine3d_gb300.scenes import dam_break


def test_seeded_scene_is_reproducible():
    a, b = dam_break(12, seed=3), dam_break(12, seed=3)
    assert np.array_equal(a.positions, b.positions)
    assert not np.array_equal(a.positions, dam_break(12, seed=4).positions)


def test_particles_per_cell_subsets_the_eight():
    full = dam_break(12, seed=1)
    assert np.array_equal(full.positions, dam_break(12, seed=1, ppc=8).positions)
    for k in (4, 5, 7):
        sub = dam_break(12, seed=1, ppc=k)
        assert sub.num_particles * 8 == full.num_particles * k
        cells = np.floor(sub.positions / sub.dx).astype(np.int64)
        _, counts = np.unique(cells, axis=0, return_counts=True)
        assert np.all(counts == k)
        # each kept particle is one of the cell's eight jittered sub-cell particles
        fullset = {tuple(p) for p in full.positions.tolist()}
        assert all(tuple(p) in fullset for p in sub.positions.tolist())
