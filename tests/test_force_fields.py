"""Point force fields (enableForceFields, ForceFieldPoint, ForceFieldGrid).

* CPU: the force-field grid the library builds on the host, bit for bit
  against the reference's ForceFieldGrid (through oracle/_ref where it is
  built): the scenes' fields, several fields with and without distance
  limits, a zero-strength field, a field centred exactly on a face, gravity
  along each axis, no fields at all; the argument checks.
* GPU: dam breaks under one point field and under three (one disabled, on a
  grid of half the resolution) against the reference engine's fixtures
  (tests/golden/ff24_*.npz): the particle count after every frame exactly,
  positions after the first frame within 1e-5 and after the last frames
  within 1e-4 (relative); the API's argument checks and error behaviour.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import aligned_rel_err, golden_scene, load_golden, rel_err
from flipengine3d_gb300 import fluidsimulation as fs
from flipengine3d_gb300 import scenes
from oracle import refsim

needs_ref = pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")
CASES = ["ff24_point", "ff24_two"]


def _centred_on_a_face(n):
    """Four vertices whose float centroid is exactly the U face (n/2, n/2, n/2)."""
    dx = 1.0 / n
    y = (n // 2 + 0.5) * dx
    v = np.array([[0.75, y, y], [0.25, y, y], [0.5, y + 0.25, y], [0.5, y - 0.25, y]], np.float32)
    t = np.array([[0, 1, 2], [0, 1, 3]], np.int32)
    return v, t


def grid_cases():
    out = []
    for which in ("point", "two"):
        sc = scenes.force_fields(24, which=which)
        n = -(-24 // sc.force_field_reduction)
        fields = [(f["vertices"], f["triangles"], f["params"]) for f in sc.force_fields]
        out.append((f"scene_{which}", n, sc.dx * sc.force_field_reduction, fields, sc.gravity))
    v1, t1 = scenes.icosphere_mesh((0.3113, 0.6217, 0.4519), 0.05, subdivisions=1)
    v2, t2 = scenes.box_mesh((0.6, 0.1, 0.2), (0.7, 0.2, 0.3))
    out.append(("limits", 20, 0.05, [(v1, t1, dict(strength=3.0, falloff_power=1.5, min_distance=0.07)),
                                     (v2, t2, dict(strength=-2.0, falloff_power=0.5, max_distance=0.33,
                                                   max_force_limit_factor=1.25, gravity_scale=-0.5,
                                                   gravity_scale_width=0.41))], (0.0, -9.81, 0.0)))
    out.append(("zero_strength", 16, 1.0 / 16, [(v1, t1, dict(strength=0.0, gravity_scale=0.0,
                                                              gravity_scale_width=0.25))], (1.5, 0.0, -2.25)))
    vf, tf = _centred_on_a_face(16)
    out.append(("on_a_face", 16, 1.0 / 16, [(vf, tf, dict(strength=1.0, falloff_power=2.0))], (0.0, 0.0, 9.81)))
    out.append(("min_at_a_face", 16, 1.0 / 16, [(vf, tf, dict(strength=1.0, min_distance=0.02))], (0.0, -1.0, 0.0)))
    out.append(("gravity_only", 12, 1.0 / 12, [], (0.5, -9.81, 0.25)))
    return out


@needs_ref
@pytest.mark.parametrize("name,n,dx,fields,gravity", grid_cases(), ids=[c[0] for c in grid_cases()])
def test_force_grid_matches_reference(built, name, n, dx, fields, gravity):
    ours = fs.point_force_grid(n, n, n, dx, [(v, q) for v, _, q in fields], gravity)
    ref = refsim.point_force_grid(n, n, n, dx, fields, gravity)
    for a, b, comp in zip(ours, ref, "uvw"):
        assert a.shape == b.shape
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), \
            f"{name} {comp}: {int((a != b).sum())} faces differ, max {float(np.nanmax(np.abs(a - b)))}"


def test_force_grid_arguments_are_checked(built):
    v, _ = scenes.box_mesh((0.1, 0.1, 0.1), (0.3, 0.3, 0.3))
    with pytest.raises(ValueError):
        fs.point_force_grid(0, 8, 8, 0.125, [(v, {})], (0, -9.81, 0))
    with pytest.raises(ValueError):
        fs.point_force_grid(8, 8, 8, -1.0, [(v, {})], (0, -9.81, 0))
    with pytest.raises(TypeError):
        fs.point_force_grid(8, 8, 8, 0.125, [(v, dict(strenght=1.0))], (0, -9.81, 0))


# ------------------------------------------------------------------- GPU
@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_force_fields_match_reference_fixture(gpu, case):
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    counts = []
    with fs.FluidSimulation.from_scene(sc) as sim:
        for f in range(1, meta["frames"] + 1):
            sim.update(meta["dt"])
            counts.append(sim.getNumMarkerParticles())
            if f"positions_{f}" not in g:
                continue
            pos = sim.getMarkerParticlePositionData()
            if f == 1:
                assert pos.shape == g["positions_1"].shape
                assert rel_err(pos, g["positions_1"]) <= 1e-5, f"{case} frame 1"
                assert rel_err(sim.getMarkerParticleVelocityData(), g["velocities_1"]) <= 1e-5
            else:
                err, skips = aligned_rel_err(pos, g[f"positions_{f}"], max_skips=2)
                assert err <= 1e-4, f"{case} frame {f}: {err} ({skips} unmatched)"
    assert counts == [int(c) for c in g["counts"]], f"{case}: particle counts {counts}"


@pytest.mark.gpu
def test_gpu_force_field_calls(gpu):
    sc = scenes.force_fields(16, which="point")
    ff = sc.force_fields[0]
    with fs.FluidSimulation(16, 16, 16, 1.0 / 16) as sim:
        sim.disableSurfaceReconstruction()
        assert not sim.isForceFieldsEnabled()
        with pytest.raises(ValueError):   # getForceFieldGrid() throws std::domain_error while they are off
            sim.addPointForceField(ff["vertices"], **ff["params"])
        sim.enableForceFields()
        with pytest.raises(ValueError):
            sim.setForceFieldReductionLevel(0)
        sim.setForceFieldReductionLevel(2)
        assert sim.getForceFieldReductionLevel() == 2
        fid = sim.addPointForceField(ff["vertices"], **ff["params"])
        got = sim.getPointForceField(fid)
        assert got.strength == np.float32(ff["params"]["strength"]) and got.min_distance_enabled == 1
        with pytest.raises(ValueError):
            sim.setPointForceField(fid + 99, strength=1.0)
        sim.setPointForceField(fid, strength=2.0, falloff_power=1.0)
        assert sim.getPointForceField(fid).max_distance_enabled == 0
        sim.addBodyForce(0.0, -9.81, 0.0)
        sim.loadMarkerParticleData(sc.positions, sc.velocities)
        sim.initialize()
        sim.update(sc.frame_dt)
        assert sim.getNumMarkerParticles() > 0
        assert np.isfinite(sim.getMarkerParticlePositionData()).all()
