"""Static mesh obstacles (addMeshObstacle) in the solid set-up, without a
device: the nodal solid level set, the face weights, the near-solid grid and
the face friction of the constrain step, bit for bit against the reference
(its fixtures, and the compiled reference where it is built here).

The reference's inside test jitters its ray origins by a random amount
below 0.001 dx; the library uses a fixed amount in that range, which gives
the same signs wherever no node lies that close to a surface or an edge,
as in these scenes (meshutils.cpp:99-215)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, golden_scene, load_golden
from flipengine3d_gb300 import fluidsimulation as fs
from flipengine3d_gb300 import scenes
from oracle import refsim

needs_ref = pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")


def face_friction(F):
    """Mean of the closest-object friction at a face's four nodes, summed in
    the reference's order (fluidsimulation.cpp:3785-3846); F is nodal (k, j, i)."""
    def mean4(a, b, c, d):
        f = np.zeros_like(a)
        for x in (a, b, c, d):
            f = (f + x).astype(np.float32)
        return (np.float32(0.25) * f).astype(np.float32)
    return (mean4(F[:-1, :-1, :], F[:-1, 1:, :], F[1:, :-1, :], F[1:, 1:, :]),
            mean4(F[:-1, :, :-1], F[:-1, :, 1:], F[1:, :, :-1], F[1:, :, 1:]),
            mean4(F[:, :-1, :-1], F[:, :-1, 1:], F[:, 1:, :-1], F[:, 1:, 1:]))


def obstacle_cases():
    return [c for c in golden_cases() if "solid_phi" in load_golden(c)[1]]


@pytest.mark.parametrize("case", obstacle_cases())
def test_solid_setup_matches_reference_fixture(built, case):
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    nodal, w, near, fr = fs.compute_solid(sc.isize, sc.jsize, sc.ksize, sc.dx, sc.cfl, sc.obstacles)
    assert np.array_equal(nodal, g["solid_phi"]), f"{case}: solid level set"
    for a, b, name in zip(w, (g["wu"], g["wv"], g["ww"]), "uvw"):
        assert np.array_equal(a, b), f"{case}: face weights {name}"
    for a, b, name in zip(fr, face_friction(g["node_friction"]), "uvw"):
        assert np.array_equal(a, b), f"{case}: face friction {name}"
    walls, _, _, _ = fs.compute_solid(sc.isize, sc.jsize, sc.ksize, sc.dx, sc.cfl, [])
    assert (nodal < 0).sum() > (walls < 0).sum(), f"{case}: the obstacle adds solid nodes"


MORE = [
    # touching the floor and the far wall: sub-grids clamped by the domain
    ("box", dict(lo=(0.61, -0.05, 0.7), hi=(0.93, 0.27, 1.2)), 0.5),
    # a sphere partly outside the domain
    ("sphere", dict(centre=(0.97, 0.51, 0.29), radius=0.17), 0.2),
    # a small box between nodes, inside the band of the walls
    ("box", dict(lo=(0.041, 0.043, 0.047), hi=(0.117, 0.121, 0.113)), 1.0),
]


def mesh(kind, kw):
    return scenes.box_mesh(kw["lo"], kw["hi"]) if kind == "box" else scenes.icosphere_mesh(kw["centre"], kw["radius"])


@needs_ref
@pytest.mark.parametrize("n,placed", [(22, [0]), (26, [1]), (24, [2]), (24, [0, 1, 2])])
def test_solid_setup_matches_reference_engine(built, n, placed):
    sc = scenes.dam_break(n, seed=4)
    sc.obstacles = [(*mesh(MORE[q][0], MORE[q][1]), MORE[q][2]) for q in placed]
    ref = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    ref.update(sc.frame_dt)   # the first step builds the solid level set
    nodal, w, near, fr = fs.compute_solid(sc.isize, sc.jsize, sc.ksize, sc.dx, sc.cfl, sc.obstacles)
    assert np.array_equal(nodal, ref.solid_phi())
    assert all(np.array_equal(a, b) for a, b in zip(w, ref.weights()[:3]))
    assert np.array_equal(near, ref.near_solid())
    assert all(np.array_equal(a, b) for a, b in zip(fr, face_friction(ref.node_friction())))


def test_obstacle_arguments_are_checked(built):
    v, t = scenes.box_mesh((0.2, 0.2, 0.2), (0.4, 0.4, 0.4))
    with pytest.raises(ValueError):   # a triangle index beyond the vertices
        fs.compute_solid(16, 16, 16, 1 / 16, 5, [(v, np.array([[0, 1, 8]], np.int32), 0.0)])
    with pytest.raises(ValueError):   # friction outside [0, 1]
        fs.compute_solid(16, 16, 16, 1 / 16, 5, [(v, t, 1.5)])
    bad = v.copy()
    bad[0, 0] = np.nan
    with pytest.raises(ValueError):
        fs.compute_solid(16, 16, 16, 1 / 16, 5, [(bad, t, 0.0)])
    # an obstacle wholly outside the domain changes nothing
    far = scenes.box_mesh((3.0, 3.0, 3.0), (3.5, 3.5, 3.5))
    a = fs.compute_solid(16, 16, 16, 1 / 16, 5, [])
    b = fs.compute_solid(16, 16, 16, 1 / 16, 5, [(*far, 0.0)])
    assert np.array_equal(a[0], b[0])
