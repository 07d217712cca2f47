"""ctypes binding of oracle/_ref/libflipref.so (test-only checker).

The library is the reference engine itself (jklae/FLIPEngine3D src/engine),
compiled by oracle/build_ref.sh; it exists only where the reference sources
are present.  Tests and tests/golden/make_golden.py use it to pin the C++
restatement in oracle/; the product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATHS = {"ref": _HERE / "_ref" / "libflipref.so", "orc": _HERE / "_build" / "libflip_oracle.so"}
_libs = {}


def available(prefix: str = "ref") -> bool:
    return _LIB_PATHS[prefix].exists()


class _Dump(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "phi", "u_p2g", "v_p2g", "w_p2g", "vu_p2g", "vv_p2g", "vw_p2g",
        "u_force", "v_force", "w_force", "pressure", "rhs",
        "u_press", "v_press", "w_press", "u_final", "v_final", "w_final",
        "u_saved", "v_saved", "w_saved", "vel_g2p", "pos_adv",
        "n_before", "pcg_iters", "pcg_error")]


class _Prefixed:
    """Attribute access with the symbol prefix ('ref_' or 'orc_') added."""

    def __init__(self, cdll, prefix):
        self._cdll, self._prefix = cdll, prefix

    def __getattr__(self, name):
        return getattr(self._cdll, name.replace("ref_", self._prefix + "_", 1))


def lib(prefix: str = "ref"):
    if prefix not in _libs:
        path = _LIB_PATHS[prefix]
        if not path.exists():
            raise FileNotFoundError(f"{path} missing: build it first")
        L = _Prefixed(C.CDLL(str(path)), prefix)
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double]
        for name, args in {
            "ref_destroy": [C.c_void_p], "ref_set_threads": [C.c_void_p, C.c_int],
            "ref_set_pic_ratio": [C.c_void_p, C.c_double],
            "ref_add_body_force": [C.c_void_p, C.c_double, C.c_double, C.c_double],
            "ref_set_cfl": [C.c_void_p, C.c_int], "ref_set_pressure_tol": [C.c_void_p, C.c_double],
            "ref_set_pressure_maxiter": [C.c_void_p, C.c_int],
            "ref_load_particles": [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
            "ref_initialize": [C.c_void_p], "ref_update": [C.c_void_p, C.c_double],
            "ref_get_particles": [C.c_void_p, C.c_void_p, C.c_void_p],
            "ref_get_liquid_phi": [C.c_void_p, C.c_void_p], "ref_get_solid_phi": [C.c_void_p, C.c_void_p],
            "ref_get_mac": [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p],
            "ref_get_weights": [C.c_void_p] + [C.c_void_p] * (4 if prefix == "ref" else 3),
            "ref_get_near_solid": [C.c_void_p, C.c_void_p, C.c_void_p],
        }.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = None
        if prefix == "ref":
            L.ref_set_particle_fragment_bytes.argtypes = [C.c_void_p, C.c_uint]
            L.ref_set_particle_fragment_bytes.restype = None
            L.ref_add_mesh_obstacle.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_float]
            L.ref_add_mesh_obstacle.restype = None
            L.ref_get_node_friction.argtypes = [C.c_void_p, C.c_void_p]
            L.ref_get_node_friction.restype = None
            L.ref_add_mesh_fluid_source.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                                    C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                                    C.c_int]
            L.ref_add_mesh_fluid_source.restype = None
            L.ref_fluid_source_setup.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_int,
                                                 C.c_void_p] + [C.c_void_p] * 5
            L.ref_fluid_source_setup.restype = None
            L.ref_set_viscosity.argtypes = [C.c_void_p, C.c_double]
            L.ref_set_viscosity.restype = None
            L.ref_viscosity_status.argtypes = [C.c_void_p]
            L.ref_viscosity_status.restype = C.c_char_p
            L.ref_set_surface_reconstruction.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int]
            L.ref_set_surface_reconstruction.restype = None
            L.ref_mesh_now.argtypes = [C.c_void_p]
            L.ref_mesh_now.restype = None
            L.ref_get_isomesh.argtypes = [C.c_void_p] + [C.c_void_p] * 4
            L.ref_get_isomesh.restype = None
            L.ref_add_mesh_fluid.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double,
                                             C.c_double, C.c_double]
            L.ref_add_mesh_fluid.restype = None
            L.ref_set_jitter_factor.argtypes = [C.c_void_p, C.c_double]
            L.ref_set_jitter_factor.restype = None
            L.ref_mesh_fluid_cells.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_int,
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
            L.ref_mesh_fluid_cells.restype = None
            L.ref_enable_force_fields.argtypes = [C.c_void_p, C.c_int]
            L.ref_enable_force_fields.restype = None
            L.ref_add_point_force_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
            L.ref_add_point_force_field.restype = None
            L.ref_point_force_grid.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int] + [C.c_void_p] * 9
            L.ref_point_force_grid.restype = None
        L.ref_num_particles.argtypes = [C.c_void_p]
        L.ref_num_particles.restype = C.c_int
        L.ref_frame_substeps.argtypes = [C.c_void_p]
        L.ref_frame_substeps.restype = C.c_int
        if prefix == "ref":
            L.ref_pressure_status.argtypes = [C.c_void_p]
            L.ref_pressure_status.restype = C.c_char_p
        else:
            L.ref_last_pcg_iters.argtypes = [C.c_void_p]
            L.ref_last_pcg_iters.restype = C.c_int
            L.ref_last_pcg_error.argtypes = [C.c_void_p]
            L.ref_last_pcg_error.restype = C.c_double
        L.ref_update_staged.argtypes = [C.c_void_p, C.c_double, C.POINTER(_Dump)]
        L.ref_update_staged.restype = C.c_int
        L.ref_mic0_factor.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 4
        L.ref_mic0_factor.restype = C.c_int
        L.ref_mic0_precondition_f32.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 4
        L.ref_mic0_precondition_f32.restype = C.c_int
        _libs[prefix] = L
    return _libs[prefix]


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def mic0_factor(fluid, rows7, prefix="ref"):
    """The MIC(0) factor of the 7-point system over the flagged cells
    (fluid: (K, J, I) uint8; rows7: (K, J, I, 4) float64 {diag, +x, +y, +z})
    by the reference's factorModifiedIncompleteColesky0 ('ref') or the
    oracle's restatement ('orc').  Returns (invdiag (K, J, I), lower
    (K, J, I, 3)): the inverse pivots and the scaled factor entries towards
    +x, +y, +z."""
    L = lib(prefix)
    K, J, I = fluid.shape
    fluid = np.ascontiguousarray(fluid, np.uint8)
    rows7 = np.ascontiguousarray(rows7, np.float64)
    inv = np.zeros((K, J, I), np.float64)
    low = np.zeros((K, J, I, 3), np.float64)
    L.ref_mic0_factor(I, J, K, _p(fluid), _p(rows7), _p(inv), _p(low))
    return inv, low


def mic0_precondition_f32(fluid, factor, r, prefix="ref"):
    """z = M^-1 r in FP32 by the reference's solveLower and
    solveLowerTransposeInPlace instantiated for float ('ref') or the oracle's
    restatement ('orc'); factor: (K, J, I, 4) float32 {invdiag, L+x, L+y, L+z}."""
    L = lib(prefix)
    K, J, I = fluid.shape
    fluid = np.ascontiguousarray(fluid, np.uint8)
    factor = np.ascontiguousarray(factor, np.float32)
    r = np.ascontiguousarray(r, np.float32)
    z = np.zeros((K, J, I), np.float32)
    L.ref_mic0_precondition_f32(I, J, K, _p(fluid), _p(factor), _p(r), _p(z))
    return z


def _hash_uniform(seed, stream, shape):
    """Uniform [0, 1) values from a splitmix64 hash of (seed, stream, index):
    the same on every host and numpy version, so fixtures need not store the
    inputs they were made from."""
    n = int(np.prod(shape))
    with np.errstate(over="ignore"):
        x = (np.arange(n, dtype=np.uint64) + np.uint64((seed * 1000003 + stream) * 0x9E3779B97F4A7C15 % (1 << 64)))
        x = (x + np.uint64(0x9E3779B97F4A7C15))
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return ((x >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))).reshape(shape)


def mesh_fluid_cells(isize, jsize, ksize, dx, vertices, triangles):
    """The reference's seeding inputs of a fluid mesh (ref_mesh_fluid_cells):
    flat cell indices of MeshObject::getCells and the mesh's nodal level set
    (k+1, j+1, i+1)."""
    L = lib("ref")
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    n = C.c_int()
    cells = np.zeros(isize * jsize * ksize, np.int32)
    phi = np.zeros((ksize + 1, jsize + 1, isize + 1), np.float32)
    L.ref_mesh_fluid_cells(isize, jsize, ksize, dx, len(v), _p(v), len(t), _p(t), C.byref(n), _p(cells), _p(phi))
    return cells[:n.value].copy(), phi


def force_field_params(q):
    """The 10 floats of the harness's point-field parameters from a dict as
    flipengine3d_gb300's PointForceFieldParams.make takes it."""
    mn, mx = q.get("min_distance"), q.get("max_distance")
    return np.array([q.get("strength", 0.0), q.get("falloff_power", 1.0), q.get("max_force_limit_factor", 3.0),
                     float(mn is not None), mn or 0.0, float(mx is not None), mx or 0.0,
                     q.get("gravity_scale", 1.0), q.get("gravity_scale_width", 0.0),
                     float(q.get("enabled", True))], np.float32)


def point_force_grid(ni, nj, nk, dx, fields, gravity):
    """The reference's ForceFieldGrid (a fresh one, updated once) for point
    fields given as (vertices, triangles, params dict): u, v, w (k, j, i)."""
    L = lib("ref")
    vs = [np.ascontiguousarray(v, np.float32).reshape(-1, 3) for v, _, _ in fields]
    ts = [np.ascontiguousarray(t, np.int32).reshape(-1, 3) for _, t, _ in fields]
    nv = np.array([len(v) for v in vs] or [0], np.int32)
    nt = np.array([len(t) for t in ts] or [0], np.int32)
    allv = np.ascontiguousarray(np.concatenate(vs) if vs else np.zeros((1, 3), np.float32))
    allt = np.ascontiguousarray(np.concatenate(ts) if ts else np.zeros((1, 3), np.int32))
    prm = np.ascontiguousarray(np.concatenate([force_field_params(q) for _, _, q in fields])
                               if fields else np.zeros(10, np.float32))
    g = np.ascontiguousarray(gravity, np.float32)
    u = np.zeros((nk, nj, ni + 1), np.float32)
    v = np.zeros((nk, nj + 1, ni), np.float32)
    w = np.zeros((nk + 1, nj, ni), np.float32)
    L.ref_point_force_grid(ni, nj, nk, float(dx), len(fields), _p(nv), _p(allv), _p(nt), _p(allt), _p(prm), _p(g),
                           _p(u), _p(v), _p(w))
    return u, v, w


def fluid_source_setup(isize, jsize, ksize, dx, vertices, triangles):
    """The reference's set-up of a static mesh fluid source: (nodes (i, j, k),
    offset xyz, level set (k, j, i) nodal, cells as flat indices)."""
    L = lib("ref")
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    nodes = np.zeros(3, np.int32)
    off = np.zeros(3, np.float32)
    n = C.c_int()
    phi = np.zeros((ksize + 2) * (jsize + 2) * (isize + 2), np.float32)
    cells = np.zeros(isize * jsize * ksize, np.int32)
    L.ref_fluid_source_setup(isize, jsize, ksize, dx, len(v), _p(v), len(t), _p(t), _p(nodes), _p(off), _p(phi),
                             C.byref(n), _p(cells))
    ni, nj, nk = (int(a) for a in nodes)
    return (ni, nj, nk), off, phi[: ni * nj * nk].reshape(nk, nj, ni).copy(), cells[: n.value].copy()


def random_mic0_system(shape, seed, weak_fraction=0.05, null_rows=2):
    """A random 7-point system of the pressure solve's shape: flagged cells
    (a union of balls, with holes) strictly inside the grid, negative
    couplings between flagged neighbours, a diagonal that dominates them by
    ghost-fluid terms towards unflagged neighbours, a fraction of weak rows
    (diagonal well below the couplings' sum, so pivots fall under the 0.25
    floor) and a few null rows (all zero).  Portable: the values depend on
    (shape, seed) only.  Returns (fluid (K, J, I) uint8, rows7 (K, J, I, 4))."""
    K, J, I = shape
    kk, jj, ii = np.meshgrid(np.arange(K), np.arange(J), np.arange(I), indexing="ij")
    inside = (ii >= 1) & (jj >= 1) & (kk >= 1) & (ii <= I - 2) & (jj <= J - 2) & (kk <= K - 2)
    balls = _hash_uniform(seed, 0, (4, 4))
    blob = np.zeros(shape, bool)
    for b in balls:
        c = b[:3] * np.array([K, J, I])
        rad = (0.25 + 0.25 * b[3]) * min(shape)
        blob |= (kk - c[0]) ** 2 + (jj - c[1]) ** 2 + (ii - c[2]) ** 2 <= rad * rad
    fluid = inside & blob & (_hash_uniform(seed, 1, shape) > 0.08)
    rows7 = np.zeros(shape + (4,), np.float64)
    nbr = np.zeros(shape + (3,), np.float64)
    offs = ((0, 0, 1), (0, 1, 0), (1, 0, 0))
    for q, (dk, dj, di) in enumerate(offs):
        shifted = np.zeros(shape, bool)
        shifted[: K - dk, : J - dj, : I - di] = fluid[dk:, dj:, di:]
        a = -(0.2 + 0.8 * _hash_uniform(seed, 2 + q, shape))
        nbr[..., q] = np.where(fluid & shifted, a, 0.0)
    rows7[..., 1:] = nbr
    coupled = np.abs(nbr).sum(-1)
    for q, (dk, dj, di) in enumerate(offs):   # the couplings mirrored from the lower neighbours
        back = np.zeros(shape)
        back[dk:, dj:, di:] = np.abs(nbr[: K - dk, : J - dj, : I - di, q])
        coupled += back
    diag = coupled + 2.0 * _hash_uniform(seed, 5, shape)
    weak = _hash_uniform(seed, 6, shape) < weak_fraction
    diag = np.where(weak, 0.3 * coupled + 1e-3, diag)
    rows7[..., 0] = np.where(fluid, diag, 0.0)
    cells = np.argwhere(fluid)
    if len(cells):
        picks = np.unique((_hash_uniform(seed, 7, (null_rows,)) * len(cells)).astype(np.int64))
        for q in picks:
            k, j, i = cells[q]
            rows7[k, j, i] = 0.0
            rows7[k, j, i - 1, 1] = 0.0
            rows7[k, j - 1, i, 2] = 0.0
            rows7[k - 1, j, i, 3] = 0.0
    return fluid.astype(np.uint8), rows7


class RefSimulation:
    """The reference FluidSimulation driven headless, as a test checker."""

    PREFIX = "ref"

    def __init__(self, isize, jsize, ksize, dx, *, threads=1, one_particle_fragment=False):
        """one_particle_fragment (reference only): hold the marker particles in
        one fragment of the reference's FragmentedVector, whose element access
        at some multiples of its default 208,333-element fragment returns the
        previous fragment's first element (ref_harness.cpp)."""
        self.L = lib(self.PREFIX)
        self.dims = (isize, jsize, ksize)
        self.dx = dx
        self.h = self.L.ref_create(isize, jsize, ksize, dx)
        self.L.ref_set_threads(self.h, threads)
        if one_particle_fragment and self.PREFIX == "ref":
            self.L.ref_set_particle_fragment_bytes(self.h, 2_000_000_000)

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup(self, scene, tolerance=None):
        obstacles = getattr(scene, "obstacles", [])
        fluids = getattr(scene, "fluid_meshes", [])
        if (obstacles or fluids or getattr(scene, "sources", []) or getattr(scene, "force_fields", [])) \
                and self.PREFIX != "ref":
            raise NotImplementedError("the oracle port restates the domain walls and loaded particles only; "
                                      "obstacle and fluid-mesh scenes are pinned by fixtures from the reference")
        if getattr(scene, "jitter_factor", None) is not None:
            self.L.ref_set_jitter_factor(self.h, float(scene.jitter_factor))
        if getattr(scene, "viscosity", None) is not None:
            self.L.ref_set_viscosity(self.h, float(scene.viscosity))
        for v, t, vel in fluids:
            v = np.ascontiguousarray(v, np.float32)
            t = np.ascontiguousarray(t, np.int32)
            self.L.ref_add_mesh_fluid(self.h, len(v), _p(v), len(t), _p(t), *(float(a) for a in vel))
        for v, t, fr in obstacles:
            v = np.ascontiguousarray(v, np.float32)
            t = np.ascontiguousarray(t, np.int32)
            self.L.ref_add_mesh_obstacle(self.h, len(v), _p(v), len(t), _p(t), float(fr))
        for src in getattr(scene, "sources", []):
            v = np.ascontiguousarray(src["vertices"], np.float32)
            t = np.ascontiguousarray(src["triangles"], np.int32)
            self.L.ref_add_mesh_fluid_source(self.h, len(v), _p(v), len(t), _p(t), int(src.get("inflow", True)),
                                             *(float(a) for a in src.get("velocity", (0.0, 0.0, 0.0))),
                                             int(src.get("substep_emissions", 1)), int(src.get("constrained", True)),
                                             int(src.get("fluid_outflow", True)), int(src.get("inversed", False)))
        if getattr(scene, "force_fields", []):
            self.L.ref_enable_force_fields(self.h, int(getattr(scene, "force_field_reduction", 1)))
            for ff in scene.force_fields:
                v = np.ascontiguousarray(ff["vertices"], np.float32)
                t = np.ascontiguousarray(ff["triangles"], np.int32)
                self.L.ref_add_point_force_field(self.h, len(v), _p(v), len(t), _p(t),
                                                 _p(force_field_params(ff["params"])))
        self.L.ref_set_pic_ratio(self.h, scene.pic_ratio)
        self.L.ref_add_body_force(self.h, *scene.gravity)
        self.L.ref_set_cfl(self.h, scene.cfl)
        self.L.ref_set_pressure_tol(self.h, scene.tolerance if tolerance is None else tolerance)
        pos = np.ascontiguousarray(scene.positions, dtype=np.float32)
        vel = np.ascontiguousarray(scene.velocities, dtype=np.float32)
        self.L.ref_load_particles(self.h, pos.shape[0], _p(pos), _p(vel))
        self.L.ref_initialize(self.h)
        return self

    def update(self, dt):
        self.L.ref_update(self.h, dt)

    def particles(self):
        n = self.L.ref_num_particles(self.h)
        pos = np.zeros((n, 3), np.float32)
        vel = np.zeros((n, 3), np.float32)
        self.L.ref_get_particles(self.h, _p(pos), _p(vel))
        return pos, vel

    def solid_phi(self):
        I, J, K = self.dims
        a = np.zeros((K + 1, J + 1, I + 1), np.float32)
        self.L.ref_get_solid_phi(self.h, _p(a))
        return a

    def liquid_phi(self):
        I, J, K = self.dims
        a = np.zeros((K, J, I), np.float32)
        self.L.ref_get_liquid_phi(self.h, _p(a))
        return a

    def weights(self):
        I, J, K = self.dims
        wu = np.zeros((K, J, I + 1), np.float32)
        wv = np.zeros((K, J + 1, I), np.float32)
        ww = np.zeros((K + 1, J, I), np.float32)
        if self.PREFIX == "ref":
            wc = np.zeros((K, J, I), np.float32)
            self.L.ref_get_weights(self.h, _p(wu), _p(wv), _p(ww), _p(wc))
        else:
            self.L.ref_get_weights(self.h, _p(wu), _p(wv), _p(ww))
        return wu, wv, ww

    def near_solid(self):
        dims = np.zeros(3, np.int32)
        self.L.ref_get_near_solid(self.h, _p(dims), None)
        out = np.zeros((dims[2], dims[1], dims[0]), np.uint8)
        self.L.ref_get_near_solid(self.h, _p(dims), _p(out))
        return out

    def pressure_status(self):
        return self.L.ref_pressure_status(self.h).decode()

    def node_friction(self):
        I, J, K = self.dims
        a = np.zeros((K + 1, J + 1, I + 1), np.float32)
        self.L.ref_get_node_friction(self.h, _p(a))
        return a

    def set_surface_reconstruction(self, enable=True, subdivisions=1, smooth_value=0.5, smooth_iterations=2):
        """Surface reconstruction on or off, with the mesher's settings
        (the reference's defaults: subdivision 1, smoothing 0.5 x 2)."""
        self.L.ref_set_surface_reconstruction(self.h, int(enable), int(subdivisions), float(smooth_value),
                                              int(smooth_iterations))

    def mesh_now(self):
        """Mesh the current particles as the first substep of a frame does."""
        self.L.ref_mesh_now(self.h)

    def isomesh(self):
        """getIsomesh(): (vertices (n, 3) float32, triangles (m, 3) int32)."""
        nv, nt = C.c_int(), C.c_int()
        self.L.ref_get_isomesh(self.h, C.byref(nv), C.byref(nt), None, None)
        v = np.zeros((nv.value, 3), np.float32)
        t = np.zeros((nt.value, 3), np.int32)
        self.L.ref_get_isomesh(self.h, C.byref(nv), C.byref(nt), _p(v), _p(t))
        return v, t

    def update_staged(self, dt):
        """One single-substep frame with the state between stages returned."""
        I, J, K = self.dims
        n = self.L.ref_num_particles(self.h)
        su, sv, sw = (K, J, I + 1), (K, J + 1, I), (K + 1, J, I)
        out = {}

        def mk(name, shape, dtype=np.float32):
            out[name] = np.zeros(shape, dtype)
            return out[name]

        d = _Dump()
        d.phi = _p(mk("phi", (K, J, I)))
        for stage in ("p2g", "force", "press", "final", "saved"):
            setattr(d, "u_" + stage, _p(mk("u_" + stage, su)))
            setattr(d, "v_" + stage, _p(mk("v_" + stage, sv)))
            setattr(d, "w_" + stage, _p(mk("w_" + stage, sw)))
        d.vu_p2g = _p(mk("vu_p2g", su, np.uint8))
        d.vv_p2g = _p(mk("vv_p2g", sv, np.uint8))
        d.vw_p2g = _p(mk("vw_p2g", sw, np.uint8))
        d.pressure = _p(mk("pressure", (K, J, I)))
        d.rhs = _p(mk("rhs", (K, J, I), np.float64))
        d.vel_g2p = _p(mk("vel_g2p", (n, 3)))
        d.pos_adv = _p(mk("pos_adv", (n, 3)))
        d.n_before = _p(mk("n_before", (1,), np.int32))
        d.pcg_iters = _p(mk("pcg_iters", (1,), np.int32))
        d.pcg_error = _p(mk("pcg_error", (1,), np.float64))
        rc = self.L.ref_update_staged(self.h, dt, C.byref(d))
        if rc != 0:
            raise RuntimeError(f"ref_update_staged returned {rc}")
        out["positions"], out["velocities"] = self.particles()
        return out


class OracleSimulation(RefSimulation):
    """The C++ restatement in oracle/flip_oracle.cpp (same interface)."""

    PREFIX = "orc"

    def pressure_status(self):
        return (f"Pressure Solver Iterations: {self.L.ref_last_pcg_iters(self.h)}\n"
                f"Estimated Error: {self.L.ref_last_pcg_error(self.h)}")
