"""Fluid added as meshes (addMeshFluid): voxelisation, level set, seeding.

* CPU: the library's host inputs of seeding (the cells around grid nodes
  inside the mesh, and the mesh's nodal level set) against the reference's
  MeshObject::getCells and MeshLevelSet (through oracle/_ref where it is
  built), including meshes that cross the domain boundary and nested
  islands; and the seeding rule restated in numpy from those inputs against
  the particles the reference engine seeded (tests/golden/mf32_*.npz).
* GPU: the device seeding and the steps after it against the reference
  engine's fixtures: the seeded particles bit for bit (jitter factor 0.001,
  whose jitter is exactly zero), later frames within 1e-5 / 1e-4; with the
  default jitter, the same particles within the jitter's range.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_scene, load_golden, rel_err
from flipengine3d_gb300 import scenes
import flipengine3d_gb300.fluidsimulation as fs
from oracle import refsim

needs_ref = pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")


def _nested_crossing(n, dx):
    """Two islands: a box reaching out of the domain's top, with a smaller
    box inside it (whole-mesh ray parity would hollow the inner box out)."""
    L = n * dx
    v1, t1 = scenes.box_mesh((0.31 * L, 0.52 * L, 0.27 * L), (0.71 * L, 1.13 * L, 0.69 * L))
    v2, t2 = scenes.box_mesh((0.41 * L, 0.61 * L, 0.37 * L), (0.57 * L, 0.83 * L, 0.55 * L))
    return np.concatenate([v1, v2]), np.concatenate([t1, t2 + len(v1)])


def mesh_cases():
    n, dx = 32, 0.125
    L = n * dx
    out = [("fluid_manager_box", n, dx) + scenes.fluid_manager_box(n, dx)]
    out.append(("sphere", n, dx) + scenes.icosphere_mesh((0.71 * L, 0.62 * L, 0.43 * L), 0.17 * L, subdivisions=2))
    out.append(("box_through_floor", n, dx) + scenes.box_mesh((0.23 * L, -0.21 * L, 0.33 * L),
                                                                (0.61 * L, 0.37 * L, 0.59 * L)))
    out.append(("nested_crossing_top", n, dx) + _nested_crossing(n, dx))
    out.append(("sphere_24x20x28", 24, 0.05) + scenes.icosphere_mesh((0.6, 0.5, 0.7), 0.33, subdivisions=3))
    return out


def test_mesh_fluid_arguments_are_checked(built):
    v, t = scenes.box_mesh((0.1, 0.1, 0.1), (0.2, 0.2, 0.2))
    with pytest.raises(ValueError):
        fs.mesh_fluid_cells(8, 8, 8, 0.1, v, t + 5)          # vertex index out of range
    bad = v.copy()
    bad[0, 0] = np.nan
    with pytest.raises(ValueError):
        fs.mesh_fluid_cells(8, 8, 8, 0.1, bad, t)
    with pytest.raises(ValueError):
        fs.mesh_fluid_cells(0, 8, 8, 0.1, v, t)


@needs_ref
@pytest.mark.parametrize("case", mesh_cases(), ids=lambda c: c[0])
def test_fluid_cells_and_level_set_match_reference(built, case):
    name, n, dx, v, t = case
    I, J, K = (24, 20, 28) if name == "sphere_24x20x28" else (n, n, n)
    c_lib, phi_lib = fs.mesh_fluid_cells(I, J, K, dx, v, t)
    c_ref, phi_ref = refsim.mesh_fluid_cells(I, J, K, dx, v, t)
    assert len(c_lib) > 0
    assert np.array_equal(c_lib, c_ref), f"{name}: {len(c_lib)} vs {len(c_ref)} cells"
    assert np.array_equal(phi_lib.view(np.uint32), phi_ref.view(np.uint32)), name


# -- the seeding rule in numpy, from the library's host inputs --------------

def _nodal_at(G, dx, p):
    """Interpolation::trilinearInterpolate over a nodal (k, j, i) grid in the
    reference's arithmetic: float offsets from the node, FP64 weights."""
    inv = 1.0 / dx
    g = np.floor(p.astype(np.float64) * inv).astype(np.int64)
    gpos = (g.astype(np.float32).astype(np.float64) * dx).astype(np.float32)
    f = (p - gpos).astype(np.float64) * inv
    nk, nj, ni = G.shape

    def at(a, b, c):
        ok = (a >= 0) & (b >= 0) & (c >= 0) & (a < ni) & (b < nj) & (c < nk)
        return np.where(ok, G[np.clip(c, 0, nk - 1), np.clip(b, 0, nj - 1), np.clip(a, 0, ni - 1)].astype(np.float64), 0.0)

    i, j, k = g[:, 0], g[:, 1], g[:, 2]
    x, y, z = f[:, 0], f[:, 1], f[:, 2]
    return (at(i, j, k) * (1 - x) * (1 - y) * (1 - z) + at(i + 1, j, k) * x * (1 - y) * (1 - z) +
            at(i, j + 1, k) * (1 - x) * y * (1 - z) + at(i, j, k + 1) * (1 - x) * (1 - y) * z +
            at(i + 1, j, k + 1) * x * (1 - y) * z + at(i, j + 1, k + 1) * (1 - x) * y * z +
            at(i + 1, j + 1, k) * x * y * (1 - z) + at(i + 1, j + 1, k + 1) * x * y * z)


def seed_without_jitter(sc, existing):
    """The particles seeding adds for the scene's fluid meshes, with zero
    jitter (_addNewFluidCellsThread / _addNewFluidCells,
    fluidsimulation.cpp:4397-4430, 4522-4562; ParticleMaskGrid), given the
    particles present when it runs: (positions, velocities)."""
    I, J, K, dx = sc.isize, sc.jsize, sc.ksize, sc.dx
    solid = fs.compute_solid(I, J, K, dx, sc.cfl, sc.obstacles)[0]
    q = np.float32(0.25 * dx)
    offs = np.array([[(-q if not (o & 1) else q), (-q if not (o & 2) else q), (-q if not (o & 4) else q)]
                     for o in range(8)], np.float32)
    sub = lambda p: np.floor(p.astype(np.float64) * (1.0 / (0.5 * dx))).astype(np.int64)
    held = set(map(tuple, sub(np.asarray(existing, np.float32)))) if len(existing) else set()
    pos, vel = [], []
    for v, t, velocity in sc.fluid_meshes:
        cells, phi = fs.mesh_fluid_cells(I, J, K, dx, v, t)
        i, j, k = cells % I, (cells // I) % J, cells // (I * J)
        centre = np.stack([(a.astype(np.float32).astype(np.float64) * dx + 0.5 * dx).astype(np.float32)
                           for a in (i, j, k)], axis=1)
        p = (centre[:, None, :] + offs[None, :, :]).reshape(-1, 3).astype(np.float32)
        d = _nodal_at(phi, dx, p).astype(np.float32)
        keep = (d <= 0) & (_nodal_at(solid, dx, p).astype(np.float32) > 0)
        for row in p[keep]:
            key = tuple(sub(row[None, :])[0])
            if key in held:
                continue
            held.add(key)
            pos.append(row)
            vel.append(np.asarray(velocity, np.float32))
    return np.array(pos, np.float32).reshape(-1, 3), np.array(vel, np.float32).reshape(-1, 3)


@pytest.mark.parametrize("name", ["mf32_box", "mf32_both"])
def test_seeding_rule_matches_reference_fixture(built, name):
    """Seeding restated in numpy from the library's cells and level sets
    gives exactly the particles the reference engine added (its first frame
    is one substep that ends with the seeding: frame 1 holds the loaded
    particles, advected, then the seeded ones, unmoved)."""
    meta, g = load_golden(name)
    sc = golden_scene(meta)
    n0 = len(sc.positions)   # the loaded particles, advected by the first substep (none removed)
    pos, vel = seed_without_jitter(sc, g["positions_1"][:n0])
    assert len(pos) > 0
    assert g["positions_1"].shape[0] == n0 + len(pos)
    assert np.array_equal(g["positions_1"][n0:], pos)
    assert np.array_equal(g["velocities_1"][n0:], vel)


# -- GPU ---------------------------------------------------------------------

def _run(sc, frames):
    sim = fs.FluidSimulation.from_scene(sc)
    out = []
    for _ in range(frames):
        sim.update(sc.frame_dt)
        out.append((sim.getMarkerParticlePositionData().copy(), sim.getMarkerParticleVelocityData().copy()))
    sim.close()
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mf32_box", "mf32_both"])
def test_gpu_mesh_fluid_matches_reference(gpu, name):
    """FluidManager's set-up (addMeshFluid, gravity -25, 1/30 s frames):
    the seeded particles bit for bit (loaded ones, after their first FLIP
    substep, within 1e-5), the next frames within 1e-5 (frame 2) and 1e-4
    (frame 3) of the reference engine."""
    meta, g = load_golden(name)
    sc = golden_scene(meta)
    res = _run(sc, meta["frames"])
    p1, v1 = res[0]
    assert p1.shape == g["positions_1"].shape
    n0 = len(sc.positions)   # loaded particles: one FLIP substep, then the seeded ones
    assert np.array_equal(p1[n0:], g["positions_1"][n0:]) and np.array_equal(v1[n0:], g["velocities_1"][n0:])
    if n0:
        assert rel_err(p1[:n0], g["positions_1"][:n0]) <= 1e-5
        assert rel_err(v1[:n0], g["velocities_1"][:n0]) <= 1e-5
    for f in range(2, meta["frames"] + 1):
        p, v = res[f - 1]
        assert p.shape == g[f"positions_{f}"].shape, f"frame {f}: particle count"
        tol = 1e-5 if f == 2 else 1e-4
        assert rel_err(p, g[f"positions_{f}"]) <= tol, f"frame {f}"
        assert rel_err(v, g[f"velocities_{f}"]) <= 10 * tol, f"frame {f}"


@pytest.mark.gpu
def test_gpu_mesh_fluid_default_jitter(gpu):
    """With the reference's default jitter factor (0) interior particles move
    by up to 0.00025 dx per axis, drawn from rand() in the reference and from
    a counter hash here: the same particles, each within twice that of the
    reference's."""
    meta, g = load_golden("mf32_box_jitter")
    sc = golden_scene(meta)
    (p1, v1), = _run(sc, 1)
    ref = g["positions_1"]
    assert p1.shape == ref.shape
    jit = 0.25 * 1e-3 * sc.dx
    assert np.abs(p1 - ref).max() <= 2 * jit * (1 + 1e-3)
    assert np.abs(p1 - ref).max() > 0          # jittered
    assert np.array_equal(v1, g["velocities_1"])
    # repeatable: the jitter is a function of the candidate, not of a clock
    (p1b, _), = _run(sc, 1)
    assert np.array_equal(p1, p1b)


@pytest.mark.gpu
def test_gpu_mesh_fluid_added_between_frames(gpu):
    """addMeshFluid on a running simulation: the mesh is filled at the end of
    the next substep, with the given velocity, after the existing
    particles, which keep their order; no seeded particle shares a sub-cell
    with a particle that was there."""
    sc = scenes.dam_break(24, seed=3)
    sim = fs.FluidSimulation.from_scene(sc)
    sim.update(sc.frame_dt)
    before = sim.getMarkerParticlePositionData().copy()
    v, t = scenes.icosphere_mesh((0.45, 0.35, 0.5), 0.2, subdivisions=2)
    sim.addMeshFluid(v, t, (0.0, -1.0, 0.5))
    n0 = sim.getNumMarkerParticles()
    st0 = sim.getFrameStatsData()
    sim.update(1e-4)           # one short substep: seeding happens at its end
    after = sim.getMarkerParticlePositionData()
    vel = sim.getMarkerParticleVelocityData()
    added = len(after) - n0
    assert added > 0 and st0.substeps >= 1
    new = after[-added:]
    lo, hi = v.min(axis=0) - sc.dx, v.max(axis=0) + sc.dx
    assert ((new >= lo) & (new <= hi)).all()
    assert np.array_equal(vel[-added:], np.tile(np.float32([0.0, -1.0, 0.5]), (added, 1)))
    sub = lambda p: set(map(tuple, np.floor(p.astype(np.float64) / (0.5 * sc.dx)).astype(np.int64)))
    moved = after[:n0]
    assert not (sub(new) & sub(moved))
    assert len(sub(new)) == added
    sim.close()


@pytest.mark.gpu
def test_gpu_jitter_factor_is_checked(gpu):
    sim = fs.FluidSimulation(8, 8, 8, 0.125)
    with pytest.raises(ValueError):
        sim.setMarkerParticleJitterFactor(-0.5)
    sim.setMarkerParticleJitterFactor(0.25)
    assert sim.getMarkerParticleJitterFactor() == 0.25
    assert not sim.isJitterSurfaceMarkerParticlesEnabled()
    sim.enableJitterSurfaceMarkerParticles()
    assert sim.isJitterSurfaceMarkerParticlesEnabled()
    v, t = scenes.box_mesh((0.3, 0.3, 0.3), (0.6, 0.6, 0.6))
    with pytest.raises(ValueError):
        sim.addMeshFluid(v, t + 8)
    sim.close()
