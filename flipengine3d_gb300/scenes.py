"""Seeded synthetic scenes for the FLIP step (host-side input generation).

The reference has no datasets or benchmark inputs; its own demo seeds fluid
bodies with 8 particles per cell, one per 2x2x2 sub-cell, jittered inside the
sub-cell (src/engine/fluidsimulation.cpp:4522-4562).  The scenes here do the
same with numpy's PCG64 generator, so a seed gives identical particles on
every host.  Particles are returned as float32 (N, 3) position and velocity
arrays in the layout `FluidSimulation::loadMarkerParticleData` takes
(src/engine/fluidsimulation.h:102-106: packed xyz floats, 12 bytes each).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Scene:
    isize: int
    jsize: int
    ksize: int
    dx: float
    positions: np.ndarray          # (N, 3) float32
    velocities: np.ndarray         # (N, 3) float32
    gravity: tuple = (0.0, -9.81, 0.0)
    pic_ratio: float = 0.05        # FLIP blend 0.95
    cfl: int = 5
    frame_dt: float = 1.0 / 120.0
    tolerance: float = 1e-6
    steps: int = 10
    name: str = ""
    meta: dict = field(default_factory=dict)
    # static mesh obstacles: (vertices (m, 3) float32, triangles (t, 3) int32, friction)
    obstacles: list = field(default_factory=list)
    # fluid meshes added with addMeshFluid: (vertices, triangles, velocity xyz)
    fluid_meshes: list = field(default_factory=list)
    jitter_factor: float | None = None   # setMarkerParticleJitterFactor, when set
    # mesh fluid sources (addMeshFluidSource): dicts with vertices, triangles,
    # inflow (bool), velocity xyz, substep_emissions, constrained,
    # fluid_outflow, inversed
    sources: list = field(default_factory=list)
    viscosity: float | None = None       # setViscosity, when set
    # point force fields (enableForceFields + addForceField): dicts with
    # vertices, triangles (the field sits at their centroid) and params (as
    # PointForceFieldParams.make takes them); the grid's reduction level
    force_fields: list = field(default_factory=list)
    force_field_reduction: int = 1

    @property
    def num_particles(self) -> int:
        return int(self.positions.shape[0])


def _jittered_cells(cells: np.ndarray, dx: float, rng: np.random.Generator, ppc: int = 8) -> np.ndarray:
    """8 particles per cell, one per 2x2x2 sub-cell, uniform inside the
    sub-cell; with ppc < 8, a random ppc of the 8 sub-cells per cell (kept in
    sub-cell order)."""
    sub = np.array([[a, b, c] for c in (0, 1) for b in (0, 1) for a in (0, 1)], dtype=np.float64)
    n = cells.shape[0]
    base = (cells[:, None, :].astype(np.float64) + 0.5 * sub[None, :, :]) * dx
    jitter = rng.random((n, 8, 3)) * (0.5 * dx)
    pts = base + jitter
    if ppc < 8:
        keep = np.sort(np.argsort(rng.random((n, 8)), axis=1)[:, :ppc], axis=1)
        pts = np.take_along_axis(pts, keep[:, :, None], axis=1)
    return pts.reshape(-1, 3).astype(np.float32)


def _box_cells(isize, jsize, ksize, dx, lo, hi) -> np.ndarray:
    i0, j0, k0 = [int(np.ceil(l / dx - 1e-9)) for l in lo]
    i1 = min(int(np.floor(hi[0] / dx + 1e-9)), isize)
    j1 = min(int(np.floor(hi[1] / dx + 1e-9)), jsize)
    k1 = min(int(np.floor(hi[2] / dx + 1e-9)), ksize)
    k, j, i = np.meshgrid(np.arange(k0, k1), np.arange(j0, j1), np.arange(i0, i1), indexing="ij")
    return np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)


def _sphere_cells(isize, jsize, ksize, dx, centre, radius) -> np.ndarray:
    k, j, i = np.meshgrid(np.arange(ksize), np.arange(jsize), np.arange(isize), indexing="ij")
    c = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    p = (c + 0.5) * dx
    d2 = ((p - np.asarray(centre)) ** 2).sum(axis=1)
    return c[d2 < radius * radius]


def dam_break(n: int = 64, *, seed: int = 0, fill=(0.4, 0.6, 1.0), sphere: bool = False,
              jsize: int | None = None, ksize: int | None = None, dx: float | None = None,
              steps: int = 10, pic_ratio: float = 0.05, tolerance: float = 1e-6, ppc: int = 8) -> Scene:
    """Dam break in an n^3 (or n x jsize x ksize) box of side n*dx.

    The fluid block spans x in [0, fill[0]], y in [0, fill[1]], z in [0, fill[2]]
    of a unit-length domain edge; cells entirely inside it get 8 particles.
    With `sphere`, a ball of radius 0.15 centred at (0.7, 0.7, 0.5) moving at
    (0, -2, 0) is added.  Particles in the outer three cells sit inside the
    domain walls and are removed by the first step, as in the reference.
    `ppc` (1-8) keeps that many of each cell's 8 particles.
    """
    jsize = n if jsize is None else jsize
    ksize = n if ksize is None else ksize
    dx = 1.0 / n if dx is None else dx
    rng = np.random.default_rng(seed)
    cells = _box_cells(n, jsize, ksize, dx, (0.0, 0.0, 0.0), fill)
    pos = _jittered_cells(cells, dx, rng, ppc)
    vel = np.zeros_like(pos)
    if sphere:
        sc = _sphere_cells(n, jsize, ksize, dx, (0.7, 0.7, 0.5), 0.15)
        sp = _jittered_cells(sc, dx, rng, ppc)
        sv = np.zeros_like(sp)
        sv[:, 1] = -2.0
        pos = np.concatenate([pos, sp])
        vel = np.concatenate([vel, sv])
    return Scene(n, jsize, ksize, dx, pos, vel, steps=steps, pic_ratio=pic_ratio,
                 tolerance=tolerance, name=f"dam{'+sphere' if sphere else ''}_{n}x{jsize}x{ksize}")


def box_mesh(lo, hi):
    """A closed box mesh from corner lo to corner hi: 8 vertices, 12
    triangles (two per face, outward winding)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float32)
    t = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [3, 7, 6], [3, 6, 2], [0, 4, 7], [0, 7, 3], [1, 2, 6], [1, 6, 5]], np.int32)
    return v, t


def icosphere_mesh(centre, radius, subdivisions=2):
    """A closed sphere mesh: an icosahedron subdivided `subdivisions` times,
    vertices pushed to the sphere (20 * 4^subdivisions triangles)."""
    g = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g), (0, 1, -g),
             (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    tris = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
            (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
            (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]
        new = []
        for a, b, c in tris:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            new += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        tris = new
    v = (np.array(verts) * radius + np.asarray(centre, np.float64)).astype(np.float32)
    return v, np.array(tris, np.int32)


def dam_with_obstacles(n: int = 24, *, seed: int = 0, which: str = "box", **kw) -> Scene:
    """A dam break (as dam_break) with a static mesh obstacle inside the fluid
    block: `box` (a box of friction 0.3 on its faces) or `sphere` (an
    icosphere, no friction), placed off the grid's node planes."""
    sc = dam_break(n, seed=seed, **kw)
    if which == "box":
        v, t = box_mesh((0.253, 0.0817, 0.3113), (0.371, 0.3929, 0.5471))
        sc.obstacles = [(v, t, 0.3)]
    elif which == "sphere":
        v, t = icosphere_mesh((0.2231, 0.3327, 0.5119), 0.1307, subdivisions=2)
        sc.obstacles = [(v, t, 0.0)]
    elif which == "both":
        v, t = box_mesh((0.253, 0.0817, 0.3113), (0.371, 0.3929, 0.5471))
        v2, t2 = icosphere_mesh((0.2131, 0.3327, 0.7519), 0.1107, subdivisions=2)
        sc.obstacles = [(v, t, 0.3), (v2, t2, 0.6)]
    else:
        raise ValueError(which)
    sc.name += f"+{which}"
    return sc


def fluid_manager_box(n: int = 32, dx: float = 0.125):
    """The fluid box FluidManager::initialize adds (src/FluidManager.cpp:
    47-68): a third of the domain on each axis, centred; vertices and
    triangles as its getTriangleMeshFromAABB (:20-44)."""
    x = y = z = n * dx
    w, h, d = x / 3.0, y / 3.0, z / 3.0
    p = np.array([0.5 * (x - w), 0.5 * (y - h), 0.5 * (z - d)], np.float32).astype(np.float64)
    # float position plus double extent, rounded to float (vmath::vec3)
    v = np.array([[p[0], p[1], p[2]], [p[0] + w, p[1], p[2]], [p[0] + w, p[1], p[2] + d], [p[0], p[1], p[2] + d],
                  [p[0], p[1] + h, p[2]], [p[0] + w, p[1] + h, p[2]], [p[0] + w, p[1] + h, p[2] + d],
                  [p[0], p[1] + h, p[2] + d]], np.float64).astype(np.float32)
    t = np.array([[0, 1, 2], [0, 2, 3], [4, 7, 6], [4, 6, 5], [0, 3, 7], [0, 7, 4],
                  [1, 5, 6], [1, 6, 2], [0, 4, 5], [0, 5, 1], [3, 2, 6], [3, 6, 7]], np.int32)
    return v, t


def mesh_fluid(n: int = 32, *, which: str = "box", dx: float = 0.125, jitter_factor: float | None = 0.001,
               steps: int = 3, seed: int = 0) -> Scene:
    """Fluid added as meshes, the way FluidManager sets up its scene: an
    n^3 grid (FluidManager's demo: 30^3, dx 0.125, 1/30 s frames, gravity
    -25), fluid from addMeshFluid, no loaded particles.

    `box`: FluidManager's box (a third of the domain, centred; with n = 32 its
    faces lie off the grid nodes).  `both`: that box, a moving icosphere of
    fluid, and a loaded block of particles overlapping the sphere, so that
    seeding skips the sub-cells the loaded particles hold.  `jitter_factor`
    0.001 makes the seeding jitter exactly zero; None keeps the reference's
    default (0: jitter of up to 0.00025 dx)."""
    v, t = fluid_manager_box(n, dx)
    pos = np.zeros((0, 3), np.float32)
    vel = np.zeros((0, 3), np.float32)
    meshes = [(v, t, (0.0, 0.0, 0.0))]
    if which == "both":
        L = n * dx
        sv, st = icosphere_mesh((0.71 * L, 0.62 * L, 0.43 * L), 0.17 * L, subdivisions=2)
        meshes.append((sv, st, (-0.5, -1.0, 0.25)))
        rng = np.random.default_rng(seed)
        cells = _box_cells(n, n, n, dx, (0.6 * L, 0.55 * L, 0.3 * L), (0.8 * L, 0.7 * L, 0.5 * L))
        pos = _jittered_cells(cells, dx, rng, 8)
        vel = np.zeros_like(pos)
        vel[:, 0] = 0.3
    elif which != "box":
        raise ValueError(which)
    sc = Scene(n, n, n, dx, pos, vel, gravity=(0.0, -25.0, 0.0), frame_dt=1.0 / 30.0, tolerance=1e-9,
               steps=steps, name=f"mesh_fluid_{which}_{n}", fluid_meshes=meshes, jitter_factor=jitter_factor)
    return sc


def fluid_sources(n: int = 24, *, which: str = "inflow", seed: int = 0, steps: int = 4) -> Scene:
    """Mesh fluid sources in an n^3 box (dx 1/n, 1/60 s frames, gravity
    -9.81, jitter factor 0.001 so that emitted particles are exactly the
    sub-cell centres):

    `inflow`: an inflow box high up near the -x wall emitting fluid moving at
    (1.5, 0, 0.2) every substep, its velocity constrained, over a small
    loaded pool; `outflow`: a dam break whose fluid runs into an outflow box
    on the floor at the far wall; `both`: the inflow, the outflow, and a
    second inflow (a sphere) that emits only at a frame's first substep and
    does not constrain velocities; `inversed`: a dam break inside an
    inversed outflow box, which removes fluid that leaves the box."""
    L = 1.0
    dx = L / n
    rng = np.random.default_rng(seed)
    inflow = dict(inflow=True, velocity=(1.5, 0.0, 0.2), substep_emissions=1, constrained=True)
    inflow["vertices"], inflow["triangles"] = box_mesh((0.0913, 0.6131, 0.3217), (0.2389, 0.7523, 0.5431))
    outflow = dict(inflow=False)
    outflow["vertices"], outflow["triangles"] = box_mesh((0.5217, -0.05, 0.2013), (1.05, 0.2311, 0.8219))
    pos = np.zeros((0, 3), np.float32)
    if which in ("inflow", "both"):
        cells = _box_cells(n, n, n, dx, (0.0, 0.0, 0.0), (0.5, 0.12, 1.0))
    else:
        cells = _box_cells(n, n, n, dx, (0.0, 0.0, 0.0), (0.45, 0.55, 0.5))
    pos = _jittered_cells(cells, dx, rng, 8)
    if which == "inflow":
        sources = [inflow]
    elif which == "outflow":
        sources = [outflow]
    elif which == "both":
        sphere = dict(inflow=True, velocity=(0.0, -0.5, 1.0), substep_emissions=0, constrained=False)
        sphere["vertices"], sphere["triangles"] = icosphere_mesh((0.6121, 0.7013, 0.3117), 0.0913, subdivisions=2)
        sources = [inflow, outflow, sphere]
    elif which == "inversed":
        inv = dict(inflow=False, inversed=True)
        inv["vertices"], inv["triangles"] = box_mesh((-0.05, -0.05, -0.05), (0.4913, 0.7219, 1.05))
        sources = [inv]
    else:
        raise ValueError(which)
    return Scene(n, n, n, dx, pos, np.zeros_like(pos), frame_dt=1.0 / 60.0, tolerance=1e-9, steps=steps,
                 name=f"fluid_sources_{which}_{n}", sources=sources, jitter_factor=0.001)


def plain_64(seed: int = 0) -> Scene:
    """Plain dam break, 64^3, dx=1/64, 10 steps of 1/120 s."""
    return dam_break(64, seed=seed, steps=10)


def plain_128(seed: int = 0) -> Scene:
    """Dam break plus falling sphere, 128^3, dx=1/128, 60 steps of 1/120 s."""
    return dam_break(128, seed=seed, sphere=True, steps=60)


def mixed_256(seed: int = 0) -> Scene:
    """256x128x128 at dx=1/128 (domain 2 x 1 x 1), fluid in the lower 45%."""
    return dam_break(256, jsize=128, ksize=128, dx=1.0 / 128, seed=seed,
                     fill=(2.0, 0.45, 1.0), steps=30, pic_ratio=0.02)


# -- the multi-scene sets: the batched (mixed-size) set and the served set

def mixed_scene_params(count: int = 64, seed: int = 1):
    """(edge, fill) of each scene of the mixed-size set, without its particles."""
    rng = np.random.default_rng(seed)
    edges = rng.choice([32, 48, 64, 80, 96], size=count)
    fills = rng.uniform(0.2, 0.6, size=count)
    return [(int(e), float(f)) for e, f in zip(edges, fills)]


def mixed_scene(q: int, count: int = 64, seed: int = 1) -> Scene:
    """Scene q of the mixed-size set: a cubic grid with its edge drawn from
    {32, 48, 64, 80, 96} (dx = 1/edge), a dam break whose x extent (the fill
    fraction) is drawn from [0.2, 0.6], y <= 0.6, full z, 8 jittered particles
    per cell, FLIP blend 0.95, PCG tolerance 1e-6."""
    e, f = mixed_scene_params(count, seed)[q]
    return dam_break(e, seed=seed * 1000 + q, fill=(f, 0.6, 1.0))


def served_scene_params(q: int, seed: int = 2):
    """(edge, fill, particles per cell) of scene q of the served set."""
    rng = np.random.default_rng([seed, q])
    edge = int(rng.integers(32, 161))
    fill = float(rng.uniform(0.2, 0.6))
    ppc = int(rng.integers(4, 9))
    return edge, fill, ppc


def served_scene(q: int, seed: int = 2) -> Scene:
    """Scene q of the served set: a cubic grid with its edge drawn uniformly
    from [32, 160] (dx = 1/edge), a dam break whose x extent is drawn from
    [0.2, 0.6], y <= 0.6, full z, 4-8 jittered particles per cell (drawn per
    scene), FLIP blend 0.95, PCG tolerance 1e-5."""
    edge, fill, ppc = served_scene_params(q, seed)
    return dam_break(edge, seed=seed * 100000 + q, fill=(fill, 0.6, 1.0), ppc=ppc, tolerance=1e-5)


def force_fields(n: int = 24, *, which: str = "point", seed: int = 0, steps: int = 4) -> Scene:
    """Point force fields over a dam break in an n^3 box (dx 1/n, 1/60 s
    frames, gravity -9.81): `point`: one attracting point field with a
    minimum and a maximum distance, and gravity scaled down around it;
    `two`: that field, a repelling one of falloff power 1 near the floor,
    and a disabled third, on a force-field grid of half the resolution."""
    L = 1.0
    dx = L / n
    rng = np.random.default_rng(seed)
    cells = _box_cells(n, n, n, dx, (0.0, 0.0, 0.0), (0.45, 0.55, 0.6))
    pos = _jittered_cells(cells, dx, rng, 8)
    attract = dict(params=dict(strength=-4.0, falloff_power=2.0, min_distance=0.1213, max_distance=0.6117,
                               gravity_scale=0.25, gravity_scale_width=0.3319))
    attract["vertices"], attract["triangles"] = icosphere_mesh((0.7013, 0.4121, 0.5217), 0.05, subdivisions=1)
    fields = [attract]
    reduction = 1
    if which == "two":
        repel = dict(params=dict(strength=1.5, falloff_power=1.0, max_force_limit_factor=2.0,
                                 gravity_scale=1.5, gravity_scale_width=0.2113))
        repel["vertices"], repel["triangles"] = box_mesh((0.2013, 0.0117, 0.7011), (0.3121, 0.0613, 0.8219))
        off = dict(params=dict(strength=50.0, enabled=False))
        off["vertices"], off["triangles"] = box_mesh((0.4, 0.4, 0.4), (0.5, 0.5, 0.5))
        fields = [attract, repel, off]
        reduction = 2
    elif which != "point":
        raise ValueError(which)
    return Scene(n, n, n, dx, pos, np.zeros_like(pos), frame_dt=1.0 / 60.0, tolerance=1e-9, steps=steps,
                 name=f"force_fields_{which}_{n}", force_fields=fields, force_field_reduction=reduction)

