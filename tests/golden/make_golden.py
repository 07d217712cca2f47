"""Generate tests/golden/*.npz from the reference engine itself.

Runs jklae/FLIPEngine3D's FluidSimulation (compiled from its sources by
oracle/build_ref.sh into oracle/_ref/libflipref.so) headless on small seeded
scenes and stores the state after each stage of the first frame plus the
particles after later frames.  Inputs are not stored: the scenes are
regenerated from flipengine3d_gb300.scenes with the recorded arguments.

    python tests/golden/make_golden.py [name ...]   # needs the reference sources
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from flipengine3d_gb300 import scenes  # noqa: E402
from oracle.refsim import RefSimulation  # noqa: E402

OUT = Path(__file__).resolve().parent

# name -> (dam_break kwargs, frames, reduction partitions, pressure tolerance)
CASES = {
    "dam16": (dict(n=16, seed=0), 3, 1, 1e-9),
    "sphere13x17x11": (dict(n=13, jsize=17, ksize=11, dx=1.0 / 13, seed=5, sphere=True, fill=(0.5, 0.5, 0.6)), 3, 1, 1e-9),
    "dam12_loose": (dict(n=12, seed=2, fill=(0.6, 0.9, 1.0)), 2, 1, 1e-6),
}
# scenes with static mesh obstacles (scenes.dam_with_obstacles): the solid
# level set, face weights and per-node closest-object friction are stored too
OBSTACLE_CASES = {
    "dam24_box": (dict(n=24, seed=3, which="box"), 3, 1, 1e-9),
    "dam20_sphere": (dict(n=20, seed=5, which="sphere"), 3, 1, 1e-9),
    "dam20_both": (dict(n=20, seed=7, which="both"), 2, 1, 1e-9),
}
# fluid added with addMeshFluid (scenes.mesh_fluid): the particles after
# every frame (the first frame seeds them at the end of its first substep)
MESH_FLUID_CASES = {
    "mf32_box": (dict(n=32, which="box"), 3, 4),
    "mf32_both": (dict(n=32, which="both"), 3, 4),
    "mf32_box_jitter": (dict(n=32, which="box", jitter_factor=None), 1, 4),
}
# mesh fluid sources (scenes.fluid_sources): the particles after every frame
SOURCE_CASES = {
    "src24_inflow": (dict(n=24, which="inflow"), 6, 4),
    "src24_outflow": (dict(n=24, which="outflow"), 9, 4),
    "src24_both": (dict(n=24, which="both"), 8, 4),
    "src24_inversed": (dict(n=24, which="inversed"), 9, 4),
}
# point force fields (scenes.force_fields): the particles after every frame
FORCE_FIELD_CASES = {
    "ff24_point": (dict(n=24, which="point"), 6, 4),
    "ff24_two": (dict(n=24, which="two"), 6, 4),
}
# viscosity (setViscosity): dam break + sphere with a constant viscosity;
# the particles after every frame and the viscosity solver's status
VISCOSITY_CASES = {
    "visc20": ("dam_break", dict(n=20, seed=1, sphere=True), 0.1, 3),
    "visc16_thin": ("dam_break", dict(n=16, seed=4), 0.01, 2),
    "visc20_box": ("dam_with_obstacles", dict(n=20, seed=6, which="box"), 0.05, 2),
}
# surface meshes (getIsomesh): the reference's mesher run on the particles
# after frame 1 at each subdivision level (default smoothing), and the mesh
# the reference made during frame 1 itself at the last level
SURFACE_CASES = {
    "iso_dam16": ("dam_break", dict(n=16, seed=0), (1, 2), 1e-9),
    "iso_dam24_box": ("dam_with_obstacles", dict(n=24, seed=3, which="box"), (2,), 1e-9),
    "iso_mf32_box": ("mesh_fluid", dict(n=32, which="box"), (1, 2), None),
}
STAGE_KEYS = ("phi", "vu_p2g", "vv_p2g", "vw_p2g", "u_p2g", "v_p2g", "w_p2g", "pressure", "u_final", "v_final",
              "w_final", "vel_g2p", "pos_adv")


def make(name, kwargs, frames, threads, tol, builder="dam_break"):
    sc = getattr(scenes, builder)(**kwargs)
    ref = RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=threads).setup(sc, tolerance=tol)
    st = ref.update_staged(sc.frame_dt)
    data = {k: st[k] for k in STAGE_KEYS}
    if builder != "dam_break":   # the solid set-up of the first step
        data["solid_phi"] = ref.solid_phi()
        data["wu"], data["wv"], data["ww"] = ref.weights()
        data["node_friction"] = ref.node_friction()
    data["pcg_iters"] = st["pcg_iters"]
    data["pcg_error"] = st["pcg_error"]
    data["positions_1"], data["velocities_1"] = st["positions"], st["velocities"]
    for f in range(2, frames + 1):
        ref.update(sc.frame_dt)
    pos, vel = ref.particles()
    data[f"positions_{frames}"], data[f"velocities_{frames}"] = pos, vel
    meta = dict(scene=kwargs, builder=builder, frames=frames, threads=threads, tolerance=tol, dt=sc.frame_dt,
                gravity=list(sc.gravity), pic_ratio=sc.pic_ratio, cfl=sc.cfl,
                seeded=int(sc.num_particles), source="jklae/FLIPEngine3D src/engine via oracle/build_ref.sh")
    np.savez_compressed(OUT / f"{name}.npz", meta=np.array(json.dumps(meta)), **data)
    print(name, "particles", sc.num_particles, "->", pos.shape[0], "iters", int(st["pcg_iters"][0]),
          f"{(OUT / f'{name}.npz').stat().st_size / 1024:.0f} KB")


def make_mesh_fluid(name, kwargs, frames, threads, builder="mesh_fluid", keep=None):
    """The particles after each frame (after the frames in `keep` only, and
    the particle count after every frame, when given)."""
    sc = getattr(scenes, builder)(**kwargs)
    ref = RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=threads).setup(sc)
    data = {}
    counts = []
    for f in range(1, frames + 1):
        ref.update(sc.frame_dt)
        pos, vel = ref.particles()
        counts.append(len(pos))
        if keep is None or f in keep:
            data[f"positions_{f}"], data[f"velocities_{f}"] = pos, vel
    if keep is not None:
        data["counts"] = np.array(counts, np.int32)
    meta = dict(scene=kwargs, builder=builder, frames=frames, threads=threads, tolerance=sc.tolerance,
                dt=sc.frame_dt, gravity=list(sc.gravity), pic_ratio=sc.pic_ratio, cfl=sc.cfl,
                loaded=int(sc.num_particles), source="jklae/FLIPEngine3D src/engine via oracle/build_ref.sh")
    np.savez_compressed(OUT / f"{name}.npz", meta=np.array(json.dumps(meta)), **data)
    print(name, "loaded", sc.num_particles, "->", counts,
          f"{(OUT / f'{name}.npz').stat().st_size / 1024:.0f} KB")


def make_surface(name, builder, kwargs, levels, tol):
    sc = getattr(scenes, builder)(**kwargs)
    ref = RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=1).setup(sc, tolerance=tol)
    ref.set_surface_reconstruction(True, levels[-1])
    ref.update(sc.frame_dt)
    data = {"frame_verts": None, "frame_tris": None}
    data["frame_verts"], data["frame_tris"] = ref.isomesh()
    data["positions"], data["velocities"] = ref.particles()
    for s in levels:
        ref.set_surface_reconstruction(True, s)
        ref.mesh_now()
        data[f"verts_s{s}"], data[f"tris_s{s}"] = ref.isomesh()
    meta = dict(scene=kwargs, builder=builder, levels=list(levels), tolerance=tol, dt=sc.frame_dt,
                gravity=list(sc.gravity), pic_ratio=sc.pic_ratio, cfl=sc.cfl, smoothing=[0.5, 2],
                substeps=int(ref.L.ref_frame_substeps(ref.h)),
                source="jklae/FLIPEngine3D src/engine via oracle/build_ref.sh")
    np.savez_compressed(OUT / f"{name}.npz", meta=np.array(json.dumps(meta)), **data)
    print(name, "particles", data["positions"].shape[0],
          {s: (len(data[f"verts_s{s}"]), len(data[f"tris_s{s}"])) for s in levels},
          f"{(OUT / f'{name}.npz').stat().st_size / 1024:.0f} KB")


def make_viscosity(name, builder, kwargs, viscosity, frames):
    sc = getattr(scenes, builder)(**kwargs)
    sc.viscosity = viscosity
    ref = RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=1).setup(sc, tolerance=1e-9)
    data, status = {}, []
    for f in range(1, frames + 1):
        ref.update(sc.frame_dt)
        data[f"positions_{f}"], data[f"velocities_{f}"] = ref.particles()
        status.append(ref.L.ref_viscosity_status(ref.h).decode())
    meta = dict(scene=kwargs, builder=builder, viscosity=viscosity, frames=frames, tolerance=1e-9,
                dt=sc.frame_dt, gravity=list(sc.gravity), pic_ratio=sc.pic_ratio, cfl=sc.cfl, status=status,
                source="jklae/FLIPEngine3D src/engine via oracle/build_ref.sh")
    np.savez_compressed(OUT / f"{name}.npz", meta=np.array(json.dumps(meta)), **data)
    print(name, [data[f"positions_{f}"].shape[0] for f in range(1, frames + 1)], status,
          f"{(OUT / f'{name}.npz').stat().st_size / 1024:.0f} KB")


if __name__ == "__main__":
    only = set(sys.argv[1:])   # names to (re)generate; all by default
    for name, (kw, frames, thr, tol) in CASES.items():
        if not only or name in only:
            make(name, kw, frames, thr, tol)
    for name, (kw, frames, thr, tol) in OBSTACLE_CASES.items():
        if not only or name in only:
            make(name, kw, frames, thr, tol, builder="dam_with_obstacles")
    for name, (kw, frames, thr) in MESH_FLUID_CASES.items():
        if not only or name in only:
            make_mesh_fluid(name, kw, frames, thr)
    for name, (kw, frames, thr) in SOURCE_CASES.items():
        if not only or name in only:
            make_mesh_fluid(name, kw, frames, thr, builder="fluid_sources", keep=(1, frames - 1, frames))
    for name, (kw, frames, thr) in FORCE_FIELD_CASES.items():
        if not only or name in only:
            make_mesh_fluid(name, kw, frames, thr, builder="force_fields", keep=(1, frames - 1, frames))
    for name, (builder, kw, visc, frames) in VISCOSITY_CASES.items():
        if not only or name in only:
            make_viscosity(name, builder, kw, visc, frames)
    for name, (builder, kw, levels, tol) in SURFACE_CASES.items():
        if not only or name in only:
            make_surface(name, builder, kw, levels, tol)
