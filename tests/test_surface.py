"""Surface reconstruction (getIsomesh): the marker particles' surface mesh.

* CPU: the oracle's numpy restatement of the reference's mesher
  (oracle/mesher.py) against the meshes the reference itself made
  (tests/golden/iso_*.npz, from tests/golden/make_golden.py), bit for bit:
  walls only, a box obstacle (solid nodes clamped, vertices kept off the
  solid) and a fluid mesh in the middle of the domain (a chunk offset from
  the origin), at subdivision levels 1 and 2; where the reference is built
  here, against the reference engine on scenes not in the fixtures.
* GPU: the library's mesher on the same particles, bit for bit against the
  reference's fixtures and against the oracle on larger states; the mesh a
  frame makes against the reference's mesh of that frame; the settings'
  argument checks.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, golden_scene, surface_cases
from flipengine3d_gb300 import fluidsimulation as fs
from flipengine3d_gb300 import scenes
from oracle import refsim
from oracle.mesher import mesh_particles

needs_ref = pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")


def level_cases():
    return [(c, s) for c in surface_cases() for s in load_golden(c)[0]["levels"]]


def scene_solid(sc):
    nodal, *_ = fs.compute_solid(sc.isize, sc.jsize, sc.ksize, sc.dx, sc.cfl, getattr(sc, "obstacles", []))
    return nodal


@pytest.mark.parametrize("case,level", level_cases())
def test_oracle_mesher_matches_reference_fixture(built, case, level):
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    v, t = mesh_particles(g["positions"], sc.isize, sc.jsize, sc.ksize, sc.dx, scene_solid(sc), level)
    assert np.array_equal(t, g[f"tris_s{level}"]), f"{case} s={level}: triangles"
    assert np.array_equal(v, g[f"verts_s{level}"]), f"{case} s={level}: vertices"


@needs_ref
@pytest.mark.parametrize("builder,kw,frames,level", [
    ("dam_with_obstacles", dict(n=20, seed=5, which="sphere"), 2, 2),
    ("dam_break", dict(n=14, jsize=18, ksize=12, dx=1.0 / 14, seed=9, sphere=True), 3, 3),
])
def test_oracle_mesher_matches_reference_engine(built, builder, kw, frames, level):
    sc = getattr(scenes, builder)(**kw)
    ref = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    for _ in range(frames):
        ref.update(sc.frame_dt)
    ref.set_surface_reconstruction(True, level)
    ref.mesh_now()
    rv, rt = ref.isomesh()
    pos, _ = ref.particles()
    v, t = mesh_particles(pos, sc.isize, sc.jsize, sc.ksize, sc.dx, ref.solid_phi(), level)
    assert len(rt) > 0
    assert np.array_equal(t, rt) and np.array_equal(v, rv)


def test_oracle_mesher_empty_and_settings(built):
    nodal = np.full((9, 9, 9), 1.0, np.float32)
    v, t = mesh_particles(np.zeros((0, 3), np.float32), 8, 8, 8, 0.125, nodal, 2)
    assert v.shape == (0, 3) and t.shape == (0, 3)
    # one particle: a closed blob, smoothing off keeps every vertex on a cut edge
    v, t = mesh_particles(np.array([[0.5, 0.5, 0.5]], np.float32), 8, 8, 8, 0.125, nodal, 2,
                          smooth_iterations=0)
    assert len(t) > 0 and len(v) > 0
    on_edge = (np.isclose(v * 16, np.round(v * 16), atol=0, rtol=0)).sum(axis=1) >= 2
    assert on_edge.all()


# ------------------------------------------------------------------- GPU
def loaded_sim(sc, positions, level):
    """A simulation of the scene's grid and obstacles holding `positions`."""
    sim = fs.FluidSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx)
    sim.setSurfaceSubdivisionLevel(level)
    for ob in getattr(sc, "obstacles", ()):
        sim.addMeshObstacle(*ob)
    sim.loadMarkerParticleData(positions, np.zeros_like(positions))
    sim.initialize()
    return sim


@pytest.mark.gpu
@pytest.mark.parametrize("case,level", level_cases())
def test_gpu_isomesh_matches_reference_fixture(gpu, case, level):
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    with loaded_sim(sc, g["positions"], level) as sim:
        sim.buildIsomesh()
        v, t = sim.getIsomesh()
    assert t.shape == g[f"tris_s{level}"].shape, f"{case} s={level}: {len(t)} triangles"
    assert np.array_equal(t, g[f"tris_s{level}"]), f"{case} s={level}: triangles"
    assert np.array_equal(v, g[f"verts_s{level}"]), f"{case} s={level}: vertices"


@pytest.mark.gpu
@pytest.mark.parametrize("case", surface_cases())
def test_gpu_frame_mesh_matches_reference_frame(gpu, case):
    """The mesh update() makes (after the frame's first substep, here the only
    one): bit for bit the oracle's mesh of the library's own particles, and
    the reference's mesh of its frame up to the particles' 1e-6 differences:
    as many triangles within 0.5%, and all but 0.5% of the vertices within
    1e-3 dx of one of the reference's (a node whose field value is that
    close to zero can flip a cube and move a vertex by a cell)."""
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    level = meta["levels"][-1]
    with fs.FluidSimulation.from_scene(sc, tolerance=meta["tolerance"], surface_subdivisions=level) as sim:
        sim.update(meta["dt"])
        assert sim.getFrameStatsData().substeps == 1
        v, t = sim.getIsomesh()
        pos = sim.getMarkerParticlePositionData()
        ov, ot = mesh_particles(pos, sc.isize, sc.jsize, sc.ksize, sc.dx, sim.solid_sdf(), level)
    assert np.array_equal(t, ot) and np.array_equal(v, ov)
    rv, rt = g["frame_verts"], g["frame_tris"]
    assert abs(len(t) - len(rt)) <= 0.005 * len(rt)
    from scipy.spatial import cKDTree
    d, _ = cKDTree(rv.astype(np.float64)).query(v.astype(np.float64))
    assert (d > 1e-3 * sc.dx).mean() <= 0.005, np.sort(d)[-5:] / sc.dx


@pytest.mark.gpu
def test_gpu_isomesh_matches_oracle_on_a_larger_state(gpu):
    """40^3 dam break with a sphere after 4 frames, subdivision 2: several
    chunk blocks per axis, solid clamping at the walls."""
    sc = scenes.dam_break(40, seed=3, sphere=True)
    with fs.FluidSimulation.from_scene(sc, surface_subdivisions=2) as sim:
        for _ in range(4):
            sim.update(sc.frame_dt)
        sim.buildIsomesh()
        v, t = sim.getIsomesh()
        pos = sim.getMarkerParticlePositionData()
        ov, ot = mesh_particles(pos, sc.isize, sc.jsize, sc.ksize, sc.dx, sim.solid_sdf(), 2)
    assert len(t) > 1000
    assert np.array_equal(t, ot) and np.array_equal(v, ov)


@pytest.mark.gpu
def test_gpu_surface_settings(gpu):
    sc = scenes.dam_break(12, seed=1)
    sim = fs.FluidSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx)
    assert sim.isSurfaceReconstructionEnabled()            # on by default, as the reference
    assert sim.getSurfaceSubdivisionLevel() == 1
    assert sim.getSurfaceSmoothingValue() == 0.5 and sim.getSurfaceSmoothingIterations() == 2
    assert sim.getMarkerParticleScale() == 3.0
    with pytest.raises(ValueError):
        sim.setSurfaceSubdivisionLevel(0)
    with pytest.raises(ValueError):
        sim.setSurfaceSmoothingIterations(-1)
    with pytest.raises(ValueError):
        sim.setMarkerParticleScale(-0.5)
    with pytest.raises(RuntimeError):
        sim.buildIsomesh()                                   # before initialize
    sim.addBodyForce(0, -9.81, 0)
    sim.initialize()                                         # no particles: an empty mesh
    sim.update(sc.frame_dt)
    v, t = sim.getIsomesh()
    assert v.shape == (0, 3) and t.shape == (0, 3)
    sim.close()
    # disabled: update() leaves the last mesh as it was
    with fs.FluidSimulation.from_scene(sc, surface_subdivisions=1) as sim:
        sim.update(sc.frame_dt)
        v1, t1 = sim.getIsomesh()
        assert len(t1) > 0
        sim.disableSurfaceReconstruction()
        sim.update(sc.frame_dt)
        v2, t2 = sim.getIsomesh()
        assert np.array_equal(v1, v2) and np.array_equal(t1, t2)
        sim.setSurfaceSmoothingIterations(0)
        sim.buildIsomesh()
        v3, t3 = sim.getIsomesh()
        ov, ot = mesh_particles(sim.getMarkerParticlePositionData(), sc.isize, sc.jsize, sc.ksize, sc.dx,
                                sim.solid_sdf(), 1, smooth_iterations=0)
        assert np.array_equal(v3, ov) and np.array_equal(t3, ot)


@pytest.mark.gpu
def test_gpu_isomesh_subdivision_three_with_an_obstacle(gpu):
    """Subdivision 3 (no aligned shortcut for the solid nodes, interpolated
    solid samples everywhere) around a sphere obstacle, against the oracle."""
    sc = scenes.dam_with_obstacles(20, seed=5, which="sphere")
    with fs.FluidSimulation.from_scene(sc, surface_subdivisions=3) as sim:
        for _ in range(2):
            sim.update(sc.frame_dt)
        v, t = sim.getIsomesh()
        pos = sim.getMarkerParticlePositionData()
        ov, ot = mesh_particles(pos, sc.isize, sc.jsize, sc.ksize, sc.dx, sim.solid_sdf(), 3)
    assert len(t) > 0
    assert np.array_equal(t, ot) and np.array_equal(v, ov)
