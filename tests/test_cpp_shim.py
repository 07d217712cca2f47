"""include/FluidSimulation.hpp: the header-only C++ face compiles against the
C ABI and maps status codes onto the reference's exception types.  Only the
device-free paths run here (argument checks come before any device call)."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

from flipengine3d_gb300 import build

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include <cstdio>
#include <stdexcept>
#include "FluidSimulation.hpp"

int main() {
    int ok = 0;
    try { flip3d::FluidSimulation s(0, 8, 8, 0.1); } catch (const std::domain_error &) { ok |= 1; }
    try { flip3d::FluidSimulation s(8, 8, 8, -1.0); } catch (const std::domain_error &) { ok |= 2; }
    flip3d::FluidSimulationMarkerParticleData d;
    ok |= (d.size == 0 && d.positions == nullptr) ? 4 : 0;
    std::printf("%d\n", ok);
    return ok == 7 ? 0 : 1;
}
"""


def test_cpp_shim_compiles_and_maps_domain_errors(built, tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    src = tmp_path / "shim.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "shim"
    libdir = build.library_path().parent
    subprocess.run([gxx, "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(libdir), "-lflip3d_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env={**os.environ})
    assert r.returncode == 0, (r.stdout, r.stderr)
    assert r.stdout.strip() == "7"


DRIVER = r"""
// FluidManager's sequence on the FLIP step (src/FluidManager.cpp:9-13,47-84),
// with the fluid loaded as marker particles: construct, body force,
// load particles, initialize, three update() frames, read positions back.
#include <cstdio>
#include <vector>
#include "FluidSimulation.hpp"

int main(int argc, char **argv) {
    int I, J, K, n;
    double dx, pic;
    std::FILE *in = std::fopen(argv[1], "rb");
    if (!in || std::fread(&I, 4, 1, in) != 1 || std::fread(&J, 4, 1, in) != 1 || std::fread(&K, 4, 1, in) != 1 ||
        std::fread(&dx, 8, 1, in) != 1 || std::fread(&pic, 8, 1, in) != 1 || std::fread(&n, 4, 1, in) != 1)
        return 2;
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n);
    if (std::fread(pos.data(), 4, pos.size(), in) != pos.size() || std::fread(vel.data(), 4, vel.size(), in) != vel.size())
        return 2;
    int nobs = 0;
    if (std::fread(&nobs, 4, 1, in) != 1) return 2;
    std::vector<flip3d::MeshObject> obstacles(nobs);
    for (int q = 0; q < nobs; q++) {   // vertex count, triangle count, friction, vertices, triangles
        int nv, nt;
        float fr;
        if (std::fread(&nv, 4, 1, in) != 1 || std::fread(&nt, 4, 1, in) != 1 || std::fread(&fr, 4, 1, in) != 1) return 2;
        flip3d::TriangleMesh m;
        m.vertices.resize((size_t)nv);
        m.triangles.resize((size_t)nt);
        if (std::fread(m.vertices.data(), 12, m.vertices.size(), in) != m.vertices.size() ||
            std::fread(m.triangles.data(), 12, m.triangles.size(), in) != m.triangles.size())
            return 2;
        obstacles[q].updateMeshStatic(m);
        obstacles[q].setFriction(fr);
    }
    std::fclose(in);
    flip3d::FluidSimulation fluidsim(I, J, K, dx);
    fluidsim.disableSurfaceReconstruction();
    fluidsim.setPICFLIPRatio(pic);
    fluidsim.addBodyForce(0.0, -9.81, 0.0);
    for (auto &o : obstacles) fluidsim.addMeshObstacle(&o);
    flip3d::FluidSimulationMarkerParticleData data;
    data.size = n;
    data.positions = reinterpret_cast<char *>(pos.data());
    data.velocities = reinterpret_cast<char *>(vel.data());
    fluidsim.loadMarkerParticleData(data);
    fluidsim.initialize();
    for (int f = 0; f < 3; f++) fluidsim.update(1.0 / 120.0);
    std::vector<char> out(fluidsim.getMarkerParticlePositionDataSize());
    fluidsim.getMarkerParticlePositionData(out.data());
    std::FILE *o = std::fopen(argv[2], "wb");
    unsigned int m = fluidsim.getNumMarkerParticles();
    std::fwrite(&m, 4, 1, o);
    std::fwrite(out.data(), 1, out.size(), o);
    std::fclose(o);
    std::printf("%d %u\n", fluidsim.getCurrentFrame(), m);
    return 0;
}
"""


def _write_scene(path, sc):
    import numpy as np
    with open(path, "wb") as f:
        np.array([sc.isize, sc.jsize, sc.ksize], np.int32).tofile(f)
        np.array([sc.dx, sc.pic_ratio], np.float64).tofile(f)
        np.array([len(sc.positions)], np.int32).tofile(f)
        np.ascontiguousarray(sc.positions, np.float32).tofile(f)
        np.ascontiguousarray(sc.velocities, np.float32).tofile(f)
        np.array([len(sc.obstacles)], np.int32).tofile(f)
        for v, t, fr in sc.obstacles:
            np.array([len(v), len(t)], np.int32).tofile(f)
            np.array([fr], np.float32).tofile(f)
            np.ascontiguousarray(v, np.float32).tofile(f)
            np.ascontiguousarray(t, np.int32).tofile(f)


def _run_driver(tmp_path, sc):
    """Compile the driver against the header, run it on the scene; the
    positions after three frames."""
    import numpy as np
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    inp = tmp_path / "scene.bin"
    _write_scene(inp, sc)
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    libdir = build.library_path().parent
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(libdir), "-lflip3d_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = tmp_path / "positions.bin"
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    frame, m = (int(v) for v in r.stdout.split())
    assert frame == 3
    raw = np.fromfile(out, dtype=np.uint32, count=1)
    pos = np.fromfile(out, dtype=np.float32, offset=4).reshape(-1, 3)
    assert int(raw[0]) == m == len(pos)
    return pos


@pytest.mark.gpu
def test_cpp_drop_in_steps_a_scene_like_the_oracle(gpu, tmp_path):
    """The C++ face drives the GPU the way FluidManager drives the reference:
    its three frames match the oracle's (reference defaults: tolerance 1e-9)."""
    from conftest import rel_err
    from flipengine3d_gb300.scenes import dam_break
    from oracle import refsim
    sc = dam_break(20, seed=31, sphere=True)
    pos = _run_driver(tmp_path, sc)
    orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx).setup(sc, tolerance=1e-9)
    for _ in range(3):
        orc.update(sc.frame_dt)
    rpos, _ = orc.particles()
    assert pos.shape == rpos.shape
    assert rel_err(pos, rpos) <= 1e-4


@pytest.mark.gpu
def test_cpp_drop_in_with_a_mesh_obstacle_matches_the_reference(gpu, tmp_path):
    """MeshObject + addMeshObstacle through the C++ face: a box obstacle with
    friction in a dam break; after three frames the positions are the
    reference engine's (its fixture dam24_box) within 1e-4."""
    from conftest import golden_scene, load_golden, rel_err
    meta, g = load_golden("dam24_box")
    assert meta["tolerance"] == 1e-9 and meta["frames"] == 3
    pos = _run_driver(tmp_path, golden_scene(meta))
    assert pos.shape == g["positions_3"].shape
    assert rel_err(pos, g["positions_3"]) <= 1e-4


MESH_FLUID_DRIVER = r"""
// FluidManager::initialize (src/FluidManager.cpp:47-68) verbatim in its
// calls, on a 32^3 grid of dx 0.125 with the jitter factor at 0.001 (the
// seeding jitter exactly zero), then three 1/30 s frames; the particles and
// the surface mesh FluidManager draws (getIsomesh, :100-166) written out.
#include <cstdio>
#include <vector>
#include "FluidSimulation.hpp"

int main(int argc, char **argv) {
    const int isize = 32, jsize = 32, ksize = 32;
    const double dx = 0.125;
    flip3d::FluidSimulation fluidsim(isize, jsize, ksize, dx);
    fluidsim.setSurfaceSubdivisionLevel(2);
    double x, y, z;
    fluidsim.getSimulationDimensions(&x, &y, &z);
    double boxWidth = (1.0 / 3.0) * x, boxHeight = (1.0 / 3.0) * y, boxDepth = (1.0 / 3.0) * z;
    flip3d::vec3 p(0.5 * (x - boxWidth), 0.5 * (y - boxHeight), 0.5 * (z - boxDepth));
    // getTriangleMeshFromAABB (src/FluidManager.cpp:20-44)
    std::vector<flip3d::vec3> verts{
        flip3d::vec3(p.x, p.y, p.z),
        flip3d::vec3(p.x + boxWidth, p.y, p.z),
        flip3d::vec3(p.x + boxWidth, p.y, p.z + boxDepth),
        flip3d::vec3(p.x, p.y, p.z + boxDepth),
        flip3d::vec3(p.x, p.y + boxHeight, p.z),
        flip3d::vec3(p.x + boxWidth, p.y + boxHeight, p.z),
        flip3d::vec3(p.x + boxWidth, p.y + boxHeight, p.z + boxDepth),
        flip3d::vec3(p.x, p.y + boxHeight, p.z + boxDepth)};
    std::vector<flip3d::Triangle> tris{
        flip3d::Triangle(0, 1, 2), flip3d::Triangle(0, 2, 3), flip3d::Triangle(4, 7, 6), flip3d::Triangle(4, 6, 5),
        flip3d::Triangle(0, 3, 7), flip3d::Triangle(0, 7, 4), flip3d::Triangle(1, 5, 6), flip3d::Triangle(1, 6, 2),
        flip3d::Triangle(0, 4, 5), flip3d::Triangle(0, 5, 1), flip3d::Triangle(3, 2, 6), flip3d::Triangle(3, 6, 7)};
    flip3d::TriangleMesh boxMesh;
    boxMesh.vertices = verts;
    boxMesh.triangles = tris;
    flip3d::MeshObject boxFluidObject(isize, jsize, ksize, dx);
    boxFluidObject.updateMeshStatic(boxMesh);
    fluidsim.setMarkerParticleJitterFactor(0.001);
    fluidsim.addMeshFluid(boxFluidObject);
    fluidsim.addBodyForce(0.0, -25.0, 0.0);
    fluidsim.initialize();
    for (int f = 0; f < 3; f++) fluidsim.update(1.0 / 30.0);
    unsigned int m = fluidsim.getNumMarkerParticles();
    std::vector<char> buf(12 * (size_t)m);
    fluidsim.getMarkerParticlePositionData(buf.data());
    flip3d::TriangleMesh isomesh = fluidsim.getIsomesh();
    std::FILE *out = std::fopen(argv[1], "wb");
    std::fwrite(&m, 4, 1, out);
    std::fwrite(buf.data(), 1, buf.size(), out);
    std::fclose(out);
    out = std::fopen(argv[2], "wb");
    unsigned int nv = (unsigned int)isomesh.vertices.size(), nt = (unsigned int)isomesh.triangles.size();
    std::fwrite(&nv, 4, 1, out);
    std::fwrite(&nt, 4, 1, out);
    std::fwrite(isomesh.vertices.data(), 12, nv, out);
    std::fwrite(isomesh.triangles.data(), 12, nt, out);
    std::fclose(out);
    std::printf("%d %u %u\n", fluidsim.getCurrentFrame(), m, nt);
    return 0;
}
"""


@pytest.mark.gpu
def test_cpp_fluid_manager_initialize_matches_reference(gpu, tmp_path):
    """FluidManager's own set-up through the C++ face: subdivision level 2,
    addMeshFluid of its centred box, gravity -25, three 1/30 s frames; the
    particles are the reference engine's (fixture mf32_box) within 1e-4, and
    getIsomesh returns the mesh of the last frame, the one the Python face
    returns for the same calls."""
    import numpy as np
    from conftest import load_golden, rel_err
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    src = tmp_path / "fm.cpp"
    src.write_text(MESH_FLUID_DRIVER)
    exe = tmp_path / "fm"
    libdir = build.library_path().parent
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(libdir), "-lflip3d_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = tmp_path / "positions.bin"
    mesh = tmp_path / "isomesh.bin"
    r = subprocess.run([str(exe), str(out), str(mesh)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    frame, m, nt = (int(v) for v in r.stdout.split())
    assert frame == 3 and nt > 0
    pos = np.fromfile(out, dtype=np.float32, offset=4).reshape(-1, 3)
    meta, g = load_golden("mf32_box")
    assert meta["scene"] == {"n": 32, "which": "box"}
    assert pos.shape == g["positions_3"].shape == (m, 3)
    assert rel_err(pos, g["positions_3"]) <= 1e-4
    counts = np.fromfile(mesh, dtype=np.uint32, count=2)
    verts = np.fromfile(mesh, dtype=np.float32, count=3 * int(counts[0]), offset=8).reshape(-1, 3)
    tris = np.fromfile(mesh, dtype=np.int32, offset=8 + 12 * int(counts[0])).reshape(-1, 3)
    assert len(tris) == nt
    # the same sequence through the Python face gives the same mesh (the
    # mesher's parity with the reference is tests/test_surface.py's)
    from flipengine3d_gb300 import fluidsimulation as fs
    from flipengine3d_gb300 import scenes
    with fs.FluidSimulation(32, 32, 32, 0.125) as sim:
        sim.setSurfaceSubdivisionLevel(2)
        sim.setMarkerParticleJitterFactor(0.001)
        sim.addMeshFluid(*scenes.fluid_manager_box(32, 0.125))
        sim.addBodyForce(0.0, -25.0, 0.0)
        sim.initialize()
        for _ in range(3):
            sim.update(1.0 / 30.0)
        ov, ot = sim.getIsomesh()
    assert np.array_equal(tris, ot) and np.array_equal(verts, ov)
    assert (verts >= 0).all() and (verts <= 4.0).all()


FORCE_FIELD_DRIVER = r"""
// Point force fields through the C++ face: the reference's calls
// (enableForceFields, setForceFieldReductionLevel, a ForceFieldPoint on a
// static mesh added with getForceFieldGrid()->addForceField), then one 1/60 s
// frame of the loaded particles under gravity; positions written out.
#include <cstdio>
#include <vector>
#include "FluidSimulation.hpp"

int main(int argc, char **argv) {
    int I, J, K, n, red, nfields;
    double dx, pic;
    std::FILE *in = std::fopen(argv[1], "rb");
    if (!in || std::fread(&I, 4, 1, in) != 1 || std::fread(&J, 4, 1, in) != 1 || std::fread(&K, 4, 1, in) != 1 ||
        std::fread(&dx, 8, 1, in) != 1 || std::fread(&pic, 8, 1, in) != 1 || std::fread(&n, 4, 1, in) != 1)
        return 2;
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n);
    if (std::fread(pos.data(), 4, pos.size(), in) != pos.size() || std::fread(vel.data(), 4, vel.size(), in) != vel.size() ||
        std::fread(&red, 4, 1, in) != 1 || std::fread(&nfields, 4, 1, in) != 1)
        return 2;
    std::vector<flip3d::ForceFieldPoint> fields(nfields);
    for (int q = 0; q < nfields; q++) {   // vertex count, triangle count, 10 parameters, vertices, triangles
        int nv, nt;
        float p[10];
        if (std::fread(&nv, 4, 1, in) != 1 || std::fread(&nt, 4, 1, in) != 1 || std::fread(p, 4, 10, in) != 10) return 2;
        flip3d::TriangleMesh m;
        m.vertices.resize((size_t)nv);
        m.triangles.resize((size_t)nt);
        if (std::fread(m.vertices.data(), 12, m.vertices.size(), in) != m.vertices.size() ||
            std::fread(m.triangles.data(), 12, m.triangles.size(), in) != m.triangles.size())
            return 2;
        flip3d::ForceFieldPoint &f = fields[q];
        f.updateMeshStatic(m);
        f.setStrength(p[0]);
        f.setFalloffPower(p[1]);
        f.setMaxForceLimitFactor(p[2]);
        if (p[3] != 0.0f) f.enableMinDistance();
        f.setMinDistance(p[4]);
        if (p[5] != 0.0f) f.enableMaxDistance();
        f.setMaxDistance(p[6]);
        f.setGravityScale(p[7]);
        f.setGravityScaleWidth(p[8]);
        if (p[9] == 0.0f) f.disable();
    }
    std::fclose(in);
    flip3d::FluidSimulation fluidsim(I, J, K, dx);
    fluidsim.disableSurfaceReconstruction();
    fluidsim.setPICFLIPRatio(pic);
    fluidsim.addBodyForce(0.0, -9.81, 0.0);
    fluidsim.enableForceFields();
    fluidsim.setForceFieldReductionLevel(red);
    for (auto &f : fields) fluidsim.getForceFieldGrid()->addForceField(&f);
    flip3d::FluidSimulationMarkerParticleData data;
    data.size = n;
    data.positions = reinterpret_cast<char *>(pos.data());
    data.velocities = reinterpret_cast<char *>(vel.data());
    fluidsim.loadMarkerParticleData(data);
    fluidsim.initialize();
    fluidsim.update(1.0 / 60.0);
    std::vector<char> out(fluidsim.getMarkerParticlePositionDataSize());
    fluidsim.getMarkerParticlePositionData(out.data());
    std::FILE *o = std::fopen(argv[2], "wb");
    unsigned int m = fluidsim.getNumMarkerParticles();
    std::fwrite(&m, 4, 1, o);
    std::fwrite(out.data(), 1, out.size(), o);
    std::fclose(o);
    std::printf("%d %u\n", fluidsim.getCurrentFrame(), m);
    return 0;
}
"""


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["ff24_point", "ff24_two"])
def test_cpp_force_fields_match_the_reference(gpu, tmp_path, case):
    """The point-field scenes set up through the C++ face (ForceFieldPoint,
    getForceFieldGrid()->addForceField) give the reference engine's
    particles after the first frame (fixtures ff24_*) within 1e-5."""
    import numpy as np
    from conftest import golden_scene, load_golden, rel_err
    from oracle import refsim
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    inp = tmp_path / "scene.bin"
    with open(inp, "wb") as f:
        np.array([sc.isize, sc.jsize, sc.ksize], np.int32).tofile(f)
        np.array([sc.dx, sc.pic_ratio], np.float64).tofile(f)
        np.array([len(sc.positions)], np.int32).tofile(f)
        np.ascontiguousarray(sc.positions, np.float32).tofile(f)
        np.ascontiguousarray(sc.velocities, np.float32).tofile(f)
        np.array([sc.force_field_reduction, len(sc.force_fields)], np.int32).tofile(f)
        for ff in sc.force_fields:
            np.array([len(ff["vertices"]), len(ff["triangles"])], np.int32).tofile(f)
            refsim.force_field_params(ff["params"]).tofile(f)
            np.ascontiguousarray(ff["vertices"], np.float32).tofile(f)
            np.ascontiguousarray(ff["triangles"], np.int32).tofile(f)
    src = tmp_path / "ff.cpp"
    src.write_text(FORCE_FIELD_DRIVER)
    exe = tmp_path / "ff"
    libdir = build.library_path().parent
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(libdir), "-lflip3d_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = tmp_path / "positions.bin"
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout, r.stderr)
    frame, m = (int(v) for v in r.stdout.split())
    pos = np.fromfile(out, dtype=np.float32, offset=4).reshape(-1, 3)
    assert frame == 1 and pos.shape == g["positions_1"].shape == (m, 3)
    assert rel_err(pos, g["positions_1"]) <= 1e-5
