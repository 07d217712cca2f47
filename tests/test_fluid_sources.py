"""Mesh fluid sources (addMeshFluidSource): inflow emission, constrained
velocities, outflow removal.

* CPU: each source's host set-up (the cells of the grid nodes inside its
  mesh, its level set over the padded sub-grid and that sub-grid's offset)
  bit for bit against the reference's MeshFluidSource (through oracle/_ref
  where it is built): the scenes' sources, a source crossing the domain
  boundary and one outside it; the argument checks.
* GPU: scenes with an inflow, an outflow, both plus a second inflow that
  emits once per frame and constrains nothing, and an inversed outflow,
  against the reference engine's fixtures (tests/golden/src24_*.npz): the
  particle count after every frame exactly, positions after the first frame
  within 1e-5 and after the last frames within 1e-4 (relative); the source
  calls' argument checks.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import aligned_rel_err, golden_scene, load_golden, rel_err
from flipengine3d_gb300 import fluidsimulation as fs
from flipengine3d_gb300 import scenes
from oracle import refsim

needs_ref = pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")
CASES = ["src24_inflow", "src24_outflow", "src24_both", "src24_inversed"]


def source_meshes():
    out = []
    for which in ("inflow", "outflow", "both", "inversed"):
        for q, src in enumerate(scenes.fluid_sources(24, which=which).sources):
            out.append((f"{which}{q}", 24, 1.0 / 24, src["vertices"], src["triangles"]))
    # a box reaching through the top and the +z wall, on a non-cubic grid
    v, t = scenes.box_mesh((0.31, 0.62, 0.41), (0.77, 1.13, 1.09))
    out.append(("crossing", 20, 0.05, v, t))
    # a sphere wholly outside the domain: no cells, an empty level set
    v, t = scenes.icosphere_mesh((2.5, 0.5, 0.5), 0.2, subdivisions=1)
    out.append(("outside", 16, 1.0 / 16, v, t))
    return out


@needs_ref
@pytest.mark.parametrize("name,n,dx,verts,tris", source_meshes(), ids=[m[0] for m in source_meshes()])
def test_source_setup_matches_reference_engine(built, name, n, dx, verts, tris):
    nodes, off, phi, cells = fs.fluid_source_setup(n, n, n, dx, verts, tris)
    rn, roff, rphi, rcells = refsim.fluid_source_setup(n, n, n, dx, verts, tris)
    assert nodes == rn
    assert np.array_equal(off, roff)
    assert np.array_equal(phi, rphi)
    assert np.array_equal(cells, rcells)


def test_source_setup_arguments_are_checked(built):
    v, t = scenes.box_mesh((0.1, 0.1, 0.1), (0.3, 0.3, 0.3))
    with pytest.raises(ValueError):
        fs.fluid_source_setup(8, 8, 8, 0.125, v, t + 8)
    with pytest.raises(ValueError):
        fs.fluid_source_setup(8, 0, 8, 0.125, v, t)


# ------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_sources_match_reference_fixture(gpu, case):
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    frames = meta["frames"]
    counts = []
    with fs.FluidSimulation.from_scene(sc) as sim:
        for f in range(1, frames + 1):
            sim.update(meta["dt"])
            counts.append(sim.getNumMarkerParticles())
            if f"positions_{f}" not in g:
                continue
            pos = sim.getMarkerParticlePositionData()
            rpos = g[f"positions_{f}"]
            if f == 1:
                assert pos.shape == rpos.shape
                assert rel_err(pos, rpos) <= 1e-5, f"{case} frame 1"
                assert rel_err(sim.getMarkerParticleVelocityData(), g["velocities_1"]) <= 1e-5
            else:
                err, skips = aligned_rel_err(pos, rpos, max_skips=2)
                assert err <= 1e-4, f"{case} frame {f}: {err} ({skips} unmatched)"
    assert counts == [int(c) for c in g["counts"]], f"{case}: particle counts {counts}"


@pytest.mark.gpu
def test_gpu_source_calls(gpu):
    sc = scenes.fluid_sources(16, which="inflow")
    src = sc.sources[0]
    with fs.FluidSimulation(16, 16, 16, 1.0 / 16) as sim:
        sim.disableSurfaceReconstruction()
        ids = [sim.addMeshFluidSource(src["vertices"], src["triangles"], velocity=(1.0, 0.0, 0.0))
               for _ in range(8)]
        assert len(set(ids)) == 8
        with pytest.raises(ValueError):   # a ninth inflow that constrains the velocity
            sim.addMeshFluidSource(src["vertices"], src["triangles"])
        extra = sim.addMeshFluidSource(src["vertices"], src["triangles"], constrained=False)
        with pytest.raises(ValueError):
            sim.setMeshFluidSource(extra, constrained=True)
        with pytest.raises(ValueError):
            sim.addMeshFluidSource(src["vertices"], src["triangles"], velocity=(np.nan, 0.0, 0.0))
        with pytest.raises(ValueError):
            sim.removeMeshFluidSource(12345)
        for q in ids[1:]:
            sim.removeMeshFluidSource(q)
        sim.setMeshFluidSource(extra, enabled=False)
        sim.addBodyForce(0.0, -9.81, 0.0)
        sim.initialize()
        for _ in range(3):
            sim.update(1.0 / 60.0)
        n = sim.getNumMarkerParticles()
        assert n > 0                      # the remaining inflow emitted
        sim.setMeshFluidSource(ids[0], enabled=False)
        sim.update(1.0 / 60.0)
        assert sim.getNumMarkerParticles() <= n   # nothing emitted while disabled


@pytest.mark.gpu
def test_gpu_source_emissions_and_removal(gpu):
    """With the seeding jitter at zero, emitting twice per substep adds
    nothing (every sub-cell the second emission would fill is taken, as in
    the reference's mask); removing the source mid-run stops emission."""
    sc = scenes.fluid_sources(24, which="inflow")
    counts = {}
    for emissions in (1, 2):
        sc.sources[0]["substep_emissions"] = emissions
        with fs.FluidSimulation.from_scene(sc) as sim:
            for _ in range(3):
                sim.update(sc.frame_dt)
            counts[emissions] = sim.getNumMarkerParticles()
            pos = sim.getMarkerParticlePositionData()
            if emissions == 1:
                first = pos
            else:
                assert np.array_equal(pos, first)
    assert counts[1] == counts[2]
    sc.sources[0]["substep_emissions"] = 1
    with fs.FluidSimulation.from_scene(sc) as sim:
        sim.update(sc.frame_dt)
        sim.removeMeshFluidSource(0)
        n = sim.getNumMarkerParticles()
        for _ in range(2):
            sim.update(sc.frame_dt)
        assert sim.getNumMarkerParticles() <= n
