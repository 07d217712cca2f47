"""Python mirror of the reference's FluidSimulation API over the C ABI.

Method names, argument meaning and error behaviour follow
jklae/FLIPEngine3D src/engine/fluidsimulation.h (FLIP Fluids 1.0.9b):
`std::runtime_error` becomes RuntimeError, `std::domain_error` ValueError,
`std::out_of_range` IndexError.  All work runs in libflip3d_gb300.so on the
GPU; there is no CPU path: without the built library or a CUDA device the
constructor raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

FLIP_OK = 0
FLIP_E_RUNTIME = -1
FLIP_E_DOMAIN = -2
FLIP_E_OUT_OF_RANGE = -3
FLIP_E_SOLVER_NOCONV = -4
FLIP_E_DEVICE_TIMEOUT = -5
FLIP_E_CUDA = -6
FLIP_E_NOMEM = -7
FLIP_E_NULL = -8


class FlipCudaError(RuntimeError):
    """A CUDA runtime failure inside the library."""


class FlipDeviceTimeout(RuntimeError):
    """A bounded device wait gave up (FLIP_E_DEVICE_TIMEOUT); the simulation
    stays usable and the next update() starts the frame afresh."""


class FrameStats(C.Structure):
    _fields_ = [("frame", C.c_int), ("substeps", C.c_int), ("delta_time", C.c_double),
                ("fluid_particles", C.c_int), ("pressure_iterations", C.c_int),
                ("pressure_error", C.c_double), ("pressure_status", C.c_int), ("pressure_cells", C.c_int)]


STAGE_NAMES = ("liquid_sdf", "p2g", "force", "pressure", "constrain", "advect", "binning")


class FluidSourceParams(C.Structure):
    """flip_fluid_source_params (include/flip3d.h)."""
    _fields_ = [("inflow", C.c_int), ("enabled", C.c_int), ("substep_emissions", C.c_int),
                ("constrained_velocity", C.c_int), ("fluid_outflow", C.c_int), ("outflow_inversed", C.c_int),
                ("velocity", C.c_double * 3)]


class PointForceFieldParams(C.Structure):
    """flip_point_force_field_params (include/flip3d.h); the defaults are
    ForceField's (forcefield.h:107-118)."""
    _fields_ = [("strength", C.c_float), ("falloff_power", C.c_float), ("max_force_limit_factor", C.c_float),
                ("min_distance_enabled", C.c_int), ("min_distance", C.c_float),
                ("max_distance_enabled", C.c_int), ("max_distance", C.c_float),
                ("gravity_scale", C.c_float), ("gravity_scale_width", C.c_float), ("enabled", C.c_int)]

    DEFAULTS = dict(strength=0.0, falloff_power=1.0, max_force_limit_factor=3.0, min_distance=None,
                    max_distance=None, gravity_scale=1.0, gravity_scale_width=0.0, enabled=True)

    @classmethod
    def make(cls, **kw):
        """From keyword arguments; min_distance / max_distance None keep the
        limit off."""
        unknown = set(kw) - set(cls.DEFAULTS)
        if unknown:
            raise TypeError(f"unknown force field parameters: {sorted(unknown)}")
        a = dict(cls.DEFAULTS, **kw)
        return cls(float(a["strength"]), float(a["falloff_power"]), float(a["max_force_limit_factor"]),
                   int(a["min_distance"] is not None), float(a["min_distance"] or 0.0),
                   int(a["max_distance"] is not None), float(a["max_distance"] or 0.0),
                   float(a["gravity_scale"]), float(a["gravity_scale_width"]), int(bool(a["enabled"])))


class Tuning(C.Structure):
    """flip_tuning (include/flip3d.h)."""
    _fields_ = [("sdf_threads", C.c_int), ("pcg_cells_per_cta", C.c_int), ("sweep_orientation", C.c_int)]


class StageDump(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in (
        "phi", "u_p2g", "v_p2g", "w_p2g", "vu_p2g", "vv_p2g", "vw_p2g",
        "u_force", "v_force", "w_force", "pressure", "rhs",
        "u_press", "v_press", "w_press", "u_final", "v_final", "w_final",
        "u_saved", "v_saved", "w_saved", "vel_g2p", "pos_adv",
        "n_before", "pcg_iters", "pcg_error")]


_lib = None

# (name, argtypes) of every exported entry point, as declared in include/flip3d.h
_P, _I, _D = C.c_void_p, C.c_int, C.c_double
SIGNATURES = {
    "flip_create": [_I, _I, _I, _D, C.POINTER(C.c_void_p)],
    "flip_destroy": [_P],
    "flip_set_stream": [_P, _P],
    "flip_set_pic_flip_ratio": [_P, _D],
    "flip_get_pic_flip_ratio": [_P, C.POINTER(C.c_double)],
    "flip_add_body_force": [_P, _D, _D, _D],
    "flip_reset_body_force": [_P],
    "flip_set_cfl_condition_number": [_P, _I],
    "flip_set_pressure_tolerance": [_P, _D],
    "flip_set_max_pressure_iterations": [_P, _I],
    "flip_load_marker_particle_data": [_P, _I, _P, _P],
    "flip_load_marker_particle_data_device": [_P, _I, _P, _P],
    "flip_initialize": [_P],
    "flip_is_initialized": [_P, C.POINTER(C.c_int)],
    "flip_update": [_P, _D],
    "flip_update_staged": [_P, _D, C.POINTER(StageDump)],
    "flip_get_num_marker_particles": [_P, C.POINTER(C.c_int)],
    "flip_get_marker_particle_position_data": [_P, _P],
    "flip_get_marker_particle_velocity_data": [_P, _P],
    "flip_get_marker_particle_position_data_range": [_P, _I, _I, _P],
    "flip_get_marker_particle_velocity_data_range": [_P, _I, _I, _P],
    "flip_get_marker_particle_data_device": [_P, _P, _P],
    "flip_get_frame_stats": [_P, C.POINTER(FrameStats)],
    "flip_get_current_frame": [_P, C.POINTER(C.c_int)],
    "flip_set_current_frame": [_P, _I],
    "flip_get_binned_particles": [_P, _P, _P, _P],
    "flip_set_device_wait_limit": [_P, C.c_uint],
    "flip_inject_sweep_stall": [_P, _I],
    "flip_get_liquid_sdf": [_P, _P],
    "flip_get_solid_sdf": [_P, _P],
    "flip_get_mac_velocity": [_P, _P, _P, _P],
    "flip_get_face_weights": [_P, _P, _P, _P],
    "flip_compute_domain_solid": [_I, _I, _I, _D, _I, _P, _P, _P, _P, _P, _P],
    "flip_add_mesh_obstacle": [_P, _I, _P, _I, _P, C.c_float],
    "flip_add_mesh_fluid": [_P, _I, _P, _I, _P, _D, _D, _D],
    "flip_set_marker_particle_jitter_factor": [_P, _D],
    "flip_get_marker_particle_jitter_factor": [_P, C.POINTER(C.c_double)],
    "flip_set_jitter_surface_marker_particles": [_P, _I],
    "flip_is_jitter_surface_marker_particles_enabled": [_P, C.POINTER(C.c_int)],
    "flip_mesh_fluid_cells": [_I, _I, _I, _D, _I, _P, _I, _P, C.POINTER(C.c_int), _P, _P],
    "flip_compute_solid": [_I, _I, _I, _D, _I, _I] + [_P] * 5 + [_P] * 9,
    "flip_set_stage_timing": [_P, _I],
    "flip_get_stage_times": [_P, _P, C.POINTER(C.c_longlong)],
    "flip_get_launch_count": [_P, C.POINTER(C.c_longlong)],
    "flip_get_host_sync_count": [_P, C.POINTER(C.c_longlong)],
    "flip_get_sweep_times": [_P, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
    "flip_set_sweep_orientation": [_P, _I],
    "flip_get_sweep_orientation": [_P, C.POINTER(C.c_int)],
    "flip_order_particles_by_id_noalloc": [_P, _P, _P, _P, _I, _I, _P, _P],
    "flip_mic0_factor": [_I, _I, _I, _P, _P, _P],
    "flip_mic0_precondition": [_I, _I, _I, _P, _P, _P, _P, _I],
    "flip_get_device_bytes": [_P, C.POINTER(C.c_longlong)],
    "flip_estimate_device_bytes": [_I, _I, _I, _I, C.POINTER(C.c_longlong)],
    "flip_runtime_create": [_I, C.c_longlong, C.POINTER(C.c_void_p)],
    "flip_runtime_destroy": [_P],
    "flip_runtime_submit": [_P, _P, _D, _I, C.POINTER(C.c_longlong)],
    "flip_runtime_wait": [_P, C.c_longlong, C.POINTER(C.c_double), C.POINTER(C.c_int)],
    "flip_runtime_update_all": [_P, C.POINTER(C.c_void_p), _I, _D],
    "flip_runtime_admit": [_P, C.c_longlong, C.POINTER(C.c_int)],
    "flip_runtime_pending": [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "flip_add_mesh_fluid_source": [_P, _I, _P, _I, _P, C.POINTER(FluidSourceParams), C.POINTER(C.c_int)],
    "flip_set_mesh_fluid_source_params": [_P, _I, C.POINTER(FluidSourceParams)],
    "flip_get_mesh_fluid_source_params": [_P, _I, C.POINTER(FluidSourceParams)],
    "flip_remove_mesh_fluid_source": [_P, _I],
    "flip_fluid_source_setup": [_I, _I, _I, _D, _I, _P, _I, _P, _P, _P, _P, C.POINTER(C.c_int), _P],
    "flip_set_viscosity": [_P, _D],
    "flip_enable_force_fields": [_P, _I],
    "flip_is_force_fields_enabled": [_P, C.POINTER(C.c_int)],
    "flip_set_force_field_reduction_level": [_P, _I],
    "flip_get_force_field_reduction_level": [_P, C.POINTER(C.c_int)],
    "flip_add_point_force_field": [_P, _I, _P, C.POINTER(PointForceFieldParams), C.POINTER(C.c_int)],
    "flip_set_point_force_field_params": [_P, _I, C.POINTER(PointForceFieldParams)],
    "flip_get_point_force_field_params": [_P, _I, C.POINTER(PointForceFieldParams)],
    "flip_point_force_grid": [_I, _I, _I, _D, _I, _P, _P, _P, _P, _P, _P, _P],
    "flip_get_viscosity": [_P, C.POINTER(C.c_double)],
    "flip_get_viscosity_solve": [_P, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_double)],
    "flip_set_tuning": [_P, C.POINTER(Tuning)],
    "flip_get_tuning": [_P, C.POINTER(Tuning)],
    "flip_enable_surface_reconstruction": [_P, _I],
    "flip_is_surface_reconstruction_enabled": [_P, C.POINTER(C.c_int)],
    "flip_set_surface_subdivision_level": [_P, _I],
    "flip_get_surface_subdivision_level": [_P, C.POINTER(C.c_int)],
    "flip_set_surface_smoothing_value": [_P, _D],
    "flip_get_surface_smoothing_value": [_P, C.POINTER(C.c_double)],
    "flip_set_surface_smoothing_iterations": [_P, _I],
    "flip_get_surface_smoothing_iterations": [_P, C.POINTER(C.c_int)],
    "flip_set_marker_particle_scale": [_P, _D],
    "flip_get_marker_particle_scale": [_P, C.POINTER(C.c_double)],
    "flip_build_isomesh": [_P],
    "flip_get_isomesh": [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), _P, _P],
}


def load_library(path: str | Path | None = None):
    """Load libflip3d_gb300.so (built by flipengine3d_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else _build.library_path()
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run flipengine3d_gb300.build.build_library() "
                                "(or __graft_entry__.build()) first")
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.flip_last_error.argtypes = []
    lib.flip_last_error.restype = C.c_char_p
    if path is None:
        _lib = lib
    return lib


def _check(lib, rc: int):
    if rc == FLIP_OK:
        return
    msg = (lib.flip_last_error() or b"").decode(errors="replace")
    if rc == FLIP_E_RUNTIME:
        raise RuntimeError(msg)
    if rc == FLIP_E_DOMAIN:
        raise ValueError(msg)
    if rc == FLIP_E_OUT_OF_RANGE:
        raise IndexError(msg)
    if rc == FLIP_E_CUDA or rc == FLIP_E_NOMEM:
        raise FlipCudaError(msg)
    if rc == FLIP_E_DEVICE_TIMEOUT:
        raise FlipDeviceTimeout(msg)
    raise RuntimeError(f"flip error {rc}: {msg}")


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def compute_domain_solid(isize, jsize, ksize, dx, cfl=5):
    """Static domain-wall set-up (no device needed): nodal solid SDF, face
    weights and the coarse near-solid grid, arrays shaped (k, j, i)."""
    lib = load_library()
    I, J, K = isize, jsize, ksize
    nodal = np.zeros((K + 1, J + 1, I + 1), np.float32)
    wu = np.zeros((K, J, I + 1), np.float32)
    wv = np.zeros((K, J + 1, I), np.float32)
    ww = np.zeros((K + 1, J, I), np.float32)
    dims = np.zeros(3, np.int32)
    _check(lib, lib.flip_compute_domain_solid(I, J, K, dx, cfl, None, None, None, None, _ptr(dims), None))
    near = np.zeros((dims[2], dims[1], dims[0]), np.uint8)
    _check(lib, lib.flip_compute_domain_solid(I, J, K, dx, cfl, _ptr(nodal), _ptr(wu), _ptr(wv), _ptr(ww),
                                              _ptr(dims), _ptr(near)))
    return nodal, (wu, wv, ww), near


def _obstacle_arrays(obstacles):
    """(n, nverts, verts, ntris, tris, friction) arrays of [(verts (m, 3),
    tris (t, 3), friction), ...]."""
    nv = np.array([len(o[0]) for o in obstacles], np.int32)
    nt = np.array([len(o[1]) for o in obstacles], np.int32)
    verts = np.ascontiguousarray(np.concatenate([np.asarray(o[0], np.float32).reshape(-1, 3) for o in obstacles])
                                 if obstacles else np.zeros((0, 3), np.float32), np.float32)
    tris = np.ascontiguousarray(np.concatenate([np.asarray(o[1], np.int32).reshape(-1, 3) for o in obstacles])
                                if obstacles else np.zeros((0, 3), np.int32), np.int32)
    fr = np.array([float(o[2]) if len(o) > 2 else 0.0 for o in obstacles], np.float32)
    return len(obstacles), nv, verts, nt, tris, fr


def mesh_fluid_cells(isize, jsize, ksize, dx, vertices, triangles):
    """Seeding inputs of a fluid mesh (no device needed): the flat indices of
    the cells around grid nodes inside the mesh (MeshObject::getCells), and
    the mesh's nodal level set (k+1, j+1, i+1), negative inside."""
    lib = load_library()
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    n = C.c_int()
    cells = np.zeros(isize * jsize * ksize, np.int32)
    phi = np.zeros((ksize + 1, jsize + 1, isize + 1), np.float32)
    _check(lib, lib.flip_mesh_fluid_cells(isize, jsize, ksize, dx, v.shape[0], _ptr(v), t.shape[0], _ptr(t),
                                          C.byref(n), _ptr(cells), _ptr(phi)))
    return cells[:n.value].copy(), phi


def point_force_grid(ni, nj, nk, dx, fields, gravity):
    """The force-field grid of point fields without a device: fields is a
    list of (vertices, params dict); returns u, v, w as (k, j, i) arrays."""
    lib = load_library()
    verts = [np.ascontiguousarray(v, np.float32).reshape(-1, 3) for v, _ in fields]
    nverts = np.array([len(v) for v in verts] or [0], np.int32)
    allv = np.ascontiguousarray(np.concatenate(verts) if verts else np.zeros((1, 3), np.float32))
    prm = (PointForceFieldParams * max(len(fields), 1))(*[PointForceFieldParams.make(**q) for _, q in fields])
    g = np.ascontiguousarray(gravity, np.float32)
    u = np.zeros((nk, nj, ni + 1), np.float32)
    v = np.zeros((nk, nj + 1, ni), np.float32)
    w = np.zeros((nk + 1, nj, ni), np.float32)
    _check(lib, lib.flip_point_force_grid(ni, nj, nk, float(dx), len(fields), _ptr(nverts), _ptr(allv),
                                          C.cast(prm, C.c_void_p), _ptr(g), _ptr(u), _ptr(v), _ptr(w)))
    return u, v, w


def fluid_source_setup(isize, jsize, ksize, dx, vertices, triangles):
    """A static mesh fluid source's set-up without a device: (nodes (i, j, k),
    offset xyz, level set (k, j, i) nodal, cells as flat indices)."""
    lib = load_library()
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
    nodes = np.zeros(3, np.int32)
    off = np.zeros(3, np.float32)
    n = C.c_int()
    _check(lib, lib.flip_fluid_source_setup(isize, jsize, ksize, dx, len(v), _ptr(v), len(t), _ptr(t), _ptr(nodes),
                                            _ptr(off), None, C.byref(n), None))
    ni, nj, nk = (int(a) for a in nodes)
    phi = np.zeros((nk, nj, ni), np.float32)
    cells = np.zeros(max(n.value, 1), np.int32)
    _check(lib, lib.flip_fluid_source_setup(isize, jsize, ksize, dx, len(v), _ptr(v), len(t), _ptr(t), _ptr(nodes),
                                            _ptr(off), _ptr(phi), C.byref(n), _ptr(cells)))
    return (ni, nj, nk), off, phi, cells[: n.value].copy()


def compute_solid(isize, jsize, ksize, dx, cfl=5, obstacles=()):
    """Static solid set-up with mesh obstacles [(verts, tris, friction), ...]
    (no device needed): nodal solid SDF, face weights (wu, wv, ww), the
    near-solid grid and the face friction (fu, fv, fw), arrays shaped (k, j, i)."""
    lib = load_library()
    I, J, K = isize, jsize, ksize
    n, nv, verts, nt, tris, fr = _obstacle_arrays(list(obstacles))
    nodal = np.zeros((K + 1, J + 1, I + 1), np.float32)
    wu, fu = np.zeros((K, J, I + 1), np.float32), np.zeros((K, J, I + 1), np.float32)
    wv, fv = np.zeros((K, J + 1, I), np.float32), np.zeros((K, J + 1, I), np.float32)
    ww, fw = np.zeros((K + 1, J, I), np.float32), np.zeros((K + 1, J, I), np.float32)
    dims = np.zeros(3, np.int32)
    args = (I, J, K, dx, cfl, n, _ptr(nv), _ptr(verts), _ptr(nt), _ptr(tris), _ptr(fr))
    _check(lib, lib.flip_compute_solid(*args, None, None, None, None, _ptr(dims), None, None, None, None))
    near = np.zeros((dims[2], dims[1], dims[0]), np.uint8)
    _check(lib, lib.flip_compute_solid(*args, _ptr(nodal), _ptr(wu), _ptr(wv), _ptr(ww), _ptr(dims), _ptr(near),
                                       _ptr(fu), _ptr(fv), _ptr(fw)))
    return nodal, (wu, wv, ww), near, (fu, fv, fw)


def order_particles_by_id_noalloc(d_px: int, d_py: int, d_pz: int, d_ids: int, n: int, id_space: int,
                                  d_out_xyz: int, cuda_stream_handle: int = 0) -> None:
    """Positions of n particles, in ascending id order, into caller memory
    (3*n floats, packed xyz); the library allocates nothing.  All pointers
    are device addresses (int); ids are distinct unsigned 32-bit values below
    id_space <= FLIP_NOALLOC_MAX_IDS.  Runs on the given stream."""
    lib = load_library()
    _check(lib, lib.flip_order_particles_by_id_noalloc(C.c_void_p(d_px), C.c_void_p(d_py), C.c_void_p(d_pz),
                                                       C.c_void_p(d_ids), int(n), int(id_space),
                                                       C.c_void_p(d_out_xyz), C.c_void_p(cuda_stream_handle)))


FLIP_NOALLOC_MAX_IDS = 1 << 20


def mic0_factor(fluid: np.ndarray, rows7: np.ndarray) -> np.ndarray:
    """The pressure solve's MIC(0) factor (factorModifiedIncompleteColesky0,
    pcgsolver.h:70-185) on the GPU for a 7-point system over the flagged
    cells: fluid (K, J, I) uint8, rows7 (K, J, I, 4) float64 {diag, +x, +y,
    +z}.  Returns the inverse pivots (K, J, I) float64, 0 off the system."""
    lib = load_library()
    K, J, I = fluid.shape
    f = np.ascontiguousarray(fluid, np.uint8)
    rows = np.ascontiguousarray(rows7, np.float64)
    inv = np.zeros((K, J, I), np.float64)
    _check(lib, lib.flip_mic0_factor(I, J, K, _ptr(f), _ptr(rows), _ptr(inv)))
    return inv


def mic0_precondition(fluid: np.ndarray, factor: np.ndarray, r: np.ndarray, orientation: int = 0) -> np.ndarray:
    """z = M^-1 r by the pressure solve's wavefront sweeps (solveLower then
    solveLowerTransposeInPlace, pcgsolver.h:192-221) on the GPU, in FP32:
    factor (K, J, I, 4) float32 {invdiag, L+x, L+y, L+z}, r (K, J, I)
    float32; orientation 0 or 1 picks the sweep tiles' lane axis."""
    lib = load_library()
    K, J, I = fluid.shape
    f = np.ascontiguousarray(fluid, np.uint8)
    L = np.ascontiguousarray(factor, np.float32)
    rr = np.ascontiguousarray(r, np.float32)
    z = np.zeros((K, J, I), np.float32)
    _check(lib, lib.flip_mic0_precondition(I, J, K, _ptr(f), _ptr(L), _ptr(rr), _ptr(z), int(orientation)))
    return z


def estimate_device_bytes(isize: int, jsize: int, ksize: int, particles: int) -> int:
    """Device memory a scene of this size needs (no device used)."""
    lib = load_library()
    b = C.c_longlong()
    _check(lib, lib.flip_estimate_device_bytes(int(isize), int(jsize), int(ksize), int(particles), C.byref(b)))
    return b.value


class FluidRuntime:
    """Many scenes on one GPU (C++ runtime behind the C ABI): `workers` host
    threads step FluidSimulation contexts concurrently, each on its own CUDA
    stream.  submit()/wait() serve step requests as they arrive (continuous
    batching; requests of one scene keep their order); update_all() steps a
    set of scenes once each.  A scene must not be used directly while it has
    requests in flight."""

    def __init__(self, workers: int = 8, reserve_bytes: int = 0):
        self._lib = load_library()
        self._h = C.c_void_p()
        _check(self._lib, self._lib.flip_runtime_create(int(workers), int(reserve_bytes), C.byref(self._h)))

    def close(self):
        if self._h:
            self._lib.flip_runtime_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, sim: "FluidSimulation", dt: float, steps: int = 1) -> int:
        rid = C.c_longlong()
        _check(self._lib, self._lib.flip_runtime_submit(self._h, sim._h, float(dt), int(steps), C.byref(rid)))
        return rid.value

    def wait(self, request_id: int):
        """(latency in ms from submission, status code of the request's updates)"""
        ms = C.c_double()
        st = C.c_int()
        _check(self._lib, self._lib.flip_runtime_wait(self._h, int(request_id), C.byref(ms), C.byref(st)))
        return ms.value, st.value

    def update_all(self, sims, dt: float) -> None:
        arr = (C.c_void_p * len(sims))(*[s._h.value for s in sims])
        rc = self._lib.flip_runtime_update_all(self._h, arr, len(sims), float(dt))
        if rc != FLIP_E_SOLVER_NOCONV:
            _check(self._lib, rc)

    def admit(self, nbytes: int) -> bool:
        ok = C.c_int()
        _check(self._lib, self._lib.flip_runtime_admit(self._h, int(nbytes), C.byref(ok)))
        return bool(ok.value)

    def pending(self):
        q, r = C.c_int(), C.c_int()
        _check(self._lib, self._lib.flip_runtime_pending(self._h, C.byref(q), C.byref(r)))
        return q.value, r.value


class FluidSimulation:
    """FluidSimulation(isize, jsize, ksize, dx) on one GB300 (current device)."""

    def __init__(self, isize: int, jsize: int, ksize: int, dx: float):
        self._lib = load_library()
        self._h = C.c_void_p()
        _check(self._lib, self._lib.flip_create(int(isize), int(jsize), int(ksize), float(dx), C.byref(self._h)))
        self.dims = (int(isize), int(jsize), int(ksize))
        self.dx = float(dx)

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.flip_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _c(self, rc):
        _check(self._lib, rc)

    # -- reference API
    def setStream(self, cuda_stream_handle: int):
        self._c(self._lib.flip_set_stream(self._h, C.c_void_p(int(cuda_stream_handle))))

    def setPICFLIPRatio(self, r: float):
        self._c(self._lib.flip_set_pic_flip_ratio(self._h, float(r)))

    def getPICFLIPRatio(self) -> float:
        v = C.c_double()
        self._c(self._lib.flip_get_pic_flip_ratio(self._h, C.byref(v)))
        return v.value

    def addBodyForce(self, fx, fy=None, fz=None):
        if fy is None:
            fx, fy, fz = fx
        self._c(self._lib.flip_add_body_force(self._h, float(fx), float(fy), float(fz)))

    def resetBodyForce(self):
        self._c(self._lib.flip_reset_body_force(self._h))

    def setCFLConditionNumber(self, n: int):
        self._c(self._lib.flip_set_cfl_condition_number(self._h, int(n)))

    def setPressureSolveTolerance(self, tol: float):
        self._c(self._lib.flip_set_pressure_tolerance(self._h, float(tol)))

    def setMaxPressureSolveIterations(self, n: int):
        self._c(self._lib.flip_set_max_pressure_iterations(self._h, int(n)))

    def addMeshObstacle(self, vertices, triangles, friction: float = 0.0):
        """addMeshObstacle (fluidsimulation.cpp:1994-2008) for a static mesh
        obstacle: vertices (m, 3), triangles (t, 3) vertex indices, surface
        friction in [0, 1]; copied on the call."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
        self._c(self._lib.flip_add_mesh_obstacle(self._h, v.shape[0], _ptr(v), t.shape[0], _ptr(t),
                                                 float(friction)))

    def addMeshFluid(self, vertices, triangles, velocity=(0.0, 0.0, 0.0)):
        """addMeshFluid (fluidsimulation.cpp:2038-2047): a static mesh,
        vertices (m, 3) and triangles (t, 3), filled with marker particles
        moving at `velocity` at the end of the next substep; copied on the
        call."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
        vx, vy, vz = (float(a) for a in velocity)
        self._c(self._lib.flip_add_mesh_fluid(self._h, v.shape[0], _ptr(v), t.shape[0], _ptr(t), vx, vy, vz))

    def setMarkerParticleJitterFactor(self, jitter: float):
        self._c(self._lib.flip_set_marker_particle_jitter_factor(self._h, float(jitter)))

    def getMarkerParticleJitterFactor(self) -> float:
        v = C.c_double()
        self._c(self._lib.flip_get_marker_particle_jitter_factor(self._h, C.byref(v)))
        return v.value

    def enableJitterSurfaceMarkerParticles(self):
        self._c(self._lib.flip_set_jitter_surface_marker_particles(self._h, 1))

    def disableJitterSurfaceMarkerParticles(self):
        self._c(self._lib.flip_set_jitter_surface_marker_particles(self._h, 0))

    def isJitterSurfaceMarkerParticlesEnabled(self) -> bool:
        v = C.c_int()
        self._c(self._lib.flip_is_jitter_surface_marker_particles_enabled(self._h, C.byref(v)))
        return bool(v.value)

    def loadMarkerParticleData(self, positions, velocities):
        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        vel = np.ascontiguousarray(velocities, dtype=np.float32).reshape(-1, 3)
        if pos.shape != vel.shape:
            raise ValueError("positions and velocities differ in size")
        self._c(self._lib.flip_load_marker_particle_data(self._h, pos.shape[0], _ptr(pos), _ptr(vel)))

    def loadMarkerParticleDataDevice(self, n: int, d_positions: int, d_velocities: int):
        self._c(self._lib.flip_load_marker_particle_data_device(self._h, int(n), C.c_void_p(d_positions),
                                                                C.c_void_p(d_velocities)))

    def initialize(self):
        self._c(self._lib.flip_initialize(self._h))

    def isInitialized(self) -> bool:
        v = C.c_int()
        self._c(self._lib.flip_is_initialized(self._h, C.byref(v)))
        return bool(v.value)

    def update(self, dt: float):
        self._c(self._lib.flip_update(self._h, float(dt)))

    def getNumMarkerParticles(self) -> int:
        v = C.c_int()
        self._c(self._lib.flip_get_num_marker_particles(self._h, C.byref(v)))
        return v.value

    def _readback_buffer(self, out) -> np.ndarray:
        n = self.getNumMarkerParticles()
        if out is None:
            return np.empty((n, 3), np.float32)
        if (not isinstance(out, np.ndarray) or out.dtype != np.float32 or not out.flags["C_CONTIGUOUS"]
                or out.size < 3 * n):
            raise ValueError(f"out must be a C-contiguous float32 array with room for {n} x 3 values")
        return out.reshape(-1)[: 3 * n].reshape(n, 3)

    def getMarkerParticlePositionData(self, out: np.ndarray | None = None) -> np.ndarray:
        """Positions in load order, 3 floats each (getMarkerParticlePositionData,
        fluidsimulation.cpp:2408-2420).  `out`, like the reference's caller
        buffer, is written in place (a pinned one avoids a staging copy)."""
        buf = self._readback_buffer(out)
        self._c(self._lib.flip_get_marker_particle_position_data(self._h, _ptr(buf)))
        return buf

    def getMarkerParticleVelocityData(self, out: np.ndarray | None = None) -> np.ndarray:
        buf = self._readback_buffer(out)
        self._c(self._lib.flip_get_marker_particle_velocity_data(self._h, _ptr(buf)))
        return buf

    def getMarkerParticlePositionDataRange(self, start: int, end: int) -> np.ndarray:
        out = np.zeros((max(end - start, 0), 3), np.float32)
        self._c(self._lib.flip_get_marker_particle_position_data_range(self._h, int(start), int(end), _ptr(out)))
        return out

    def getMarkerParticleVelocityDataRange(self, start: int, end: int) -> np.ndarray:
        out = np.zeros((max(end - start, 0), 3), np.float32)
        self._c(self._lib.flip_get_marker_particle_velocity_data_range(self._h, int(start), int(end), _ptr(out)))
        return out

    def getMarkerParticleDataDevice(self, d_positions: int, d_velocities: int):
        self._c(self._lib.flip_get_marker_particle_data_device(self._h, C.c_void_p(d_positions),
                                                               C.c_void_p(d_velocities)))

    def getCurrentFrame(self) -> int:
        v = C.c_int()
        self._c(self._lib.flip_get_current_frame(self._h, C.byref(v)))
        return v.value

    def setCurrentFrame(self, frame: int):
        """setCurrentFrame (fluidsimulation.cpp:98-103): resume numbering at
        `frame`; above 0 the first substep takes its CFL speed from the
        particles, as a run that reached this frame does."""
        self._c(self._lib.flip_set_current_frame(self._h, int(frame)))

    def getFrameStatsData(self) -> FrameStats:
        s = FrameStats()
        self._c(self._lib.flip_get_frame_stats(self._h, C.byref(s)))
        return s

    # -- viscosity (fluidsimulation.cpp:1650-1670, 3592-3640)
    # -- force fields (enableForceFields, getForceFieldGrid()->addForceField)
    def enableForceFields(self):
        self._c(self._lib.flip_enable_force_fields(self._h, 1))

    def disableForceFields(self):
        self._c(self._lib.flip_enable_force_fields(self._h, 0))

    def isForceFieldsEnabled(self) -> bool:
        v = C.c_int()
        self._c(self._lib.flip_is_force_fields_enabled(self._h, C.byref(v)))
        return bool(v.value)

    def setForceFieldReductionLevel(self, level: int):
        self._c(self._lib.flip_set_force_field_reduction_level(self._h, int(level)))

    def getForceFieldReductionLevel(self) -> int:
        v = C.c_int()
        self._c(self._lib.flip_get_force_field_reduction_level(self._h, C.byref(v)))
        return v.value

    def addPointForceField(self, vertices, **params) -> int:
        """A ForceFieldPoint at the centroid of a static mesh's vertices;
        params as PointForceFieldParams.make.  Returns the field's id."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        prm = PointForceFieldParams.make(**params)
        fid = C.c_int()
        self._c(self._lib.flip_add_point_force_field(self._h, len(v), _ptr(v), C.byref(prm), C.byref(fid)))
        return fid.value

    def setPointForceField(self, field_id: int, **params):
        prm = PointForceFieldParams.make(**params)
        self._c(self._lib.flip_set_point_force_field_params(self._h, int(field_id), C.byref(prm)))

    def getPointForceField(self, field_id: int) -> PointForceFieldParams:
        prm = PointForceFieldParams()
        self._c(self._lib.flip_get_point_force_field_params(self._h, int(field_id), C.byref(prm)))
        return prm

    def setViscosity(self, v: float):
        self._c(self._lib.flip_set_viscosity(self._h, float(v)))

    def getViscosity(self) -> float:
        v = C.c_double()
        self._c(self._lib.flip_get_viscosity(self._h, C.byref(v)))
        return v.value

    def viscosity_solve(self):
        """(rows, iterations, relative residual) of the last substep's viscosity solve."""
        rows, it, res = C.c_longlong(), C.c_int(), C.c_double()
        self._c(self._lib.flip_get_viscosity_solve(self._h, C.byref(rows), C.byref(it), C.byref(res)))
        return rows.value, it.value, res.value

    # -- tuning knobs (flip_set_tuning; flipengine3d_gb300.autotune)
    def setTuning(self, sdf_threads: int = 512, pcg_cells_per_cta: int = 4096, sweep_orientation: int = -1):
        t = Tuning(int(sdf_threads), int(pcg_cells_per_cta), int(sweep_orientation))
        self._c(self._lib.flip_set_tuning(self._h, C.byref(t)))

    def getTuning(self) -> dict:
        t = Tuning()
        self._c(self._lib.flip_get_tuning(self._h, C.byref(t)))
        return {"sdf_threads": t.sdf_threads, "pcg_cells_per_cta": t.pcg_cells_per_cta,
                "sweep_orientation": t.sweep_orientation}

    def applyTunedSettings(self):
        """The autotuner's settings for this grid (the nearest edge of
        flipengine3d_gb300/tuning_gb300.json; defaults without a table)."""
        from .autotune import lookup
        I, J, K = self.dims
        self.setTuning(**lookup(I, J, K))

    # -- mesh fluid sources (fluidsimulation.cpp:1953-1992)
    @staticmethod
    def _source_params(inflow=True, enabled=True, substep_emissions=1, constrained=True, fluid_outflow=True,
                       inversed=False, velocity=(0.0, 0.0, 0.0)):
        p = FluidSourceParams()
        p.inflow, p.enabled, p.substep_emissions = int(inflow), int(enabled), int(substep_emissions)
        p.constrained_velocity, p.fluid_outflow, p.outflow_inversed = int(constrained), int(fluid_outflow), int(inversed)
        for a in range(3):
            p.velocity[a] = float(velocity[a])
        return p

    def addMeshFluidSource(self, vertices, triangles, **params) -> int:
        """A static mesh fluid source; keyword settings as the reference's
        MeshFluidSource setters (inflow, enabled, substep_emissions,
        constrained, fluid_outflow, inversed, velocity).  Returns its id."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, np.int32).reshape(-1, 3)
        sid = C.c_int()
        p = self._source_params(**params)
        self._c(self._lib.flip_add_mesh_fluid_source(self._h, len(v), _ptr(v), len(t), _ptr(t), C.byref(p),
                                                     C.byref(sid)))
        return sid.value

    def setMeshFluidSource(self, source_id: int, **params):
        p = self._source_params(**params)
        self._c(self._lib.flip_set_mesh_fluid_source_params(self._h, int(source_id), C.byref(p)))

    def removeMeshFluidSource(self, source_id: int):
        self._c(self._lib.flip_remove_mesh_fluid_source(self._h, int(source_id)))

    # -- surface reconstruction (fluidsimulation.cpp:216-300, 367-380, 2543-2546)
    def enableSurfaceReconstruction(self):
        self._c(self._lib.flip_enable_surface_reconstruction(self._h, 1))

    def disableSurfaceReconstruction(self):
        self._c(self._lib.flip_enable_surface_reconstruction(self._h, 0))

    def isSurfaceReconstructionEnabled(self) -> bool:
        v = C.c_int()
        self._c(self._lib.flip_is_surface_reconstruction_enabled(self._h, C.byref(v)))
        return bool(v.value)

    def setSurfaceSubdivisionLevel(self, n: int):
        self._c(self._lib.flip_set_surface_subdivision_level(self._h, int(n)))

    def getSurfaceSubdivisionLevel(self) -> int:
        v = C.c_int()
        self._c(self._lib.flip_get_surface_subdivision_level(self._h, C.byref(v)))
        return v.value

    def setSurfaceSmoothingValue(self, s: float):
        self._c(self._lib.flip_set_surface_smoothing_value(self._h, float(s)))

    def getSurfaceSmoothingValue(self) -> float:
        v = C.c_double()
        self._c(self._lib.flip_get_surface_smoothing_value(self._h, C.byref(v)))
        return v.value

    def setSurfaceSmoothingIterations(self, n: int):
        self._c(self._lib.flip_set_surface_smoothing_iterations(self._h, int(n)))

    def getSurfaceSmoothingIterations(self) -> int:
        v = C.c_int()
        self._c(self._lib.flip_get_surface_smoothing_iterations(self._h, C.byref(v)))
        return v.value

    def setMarkerParticleScale(self, s: float):
        self._c(self._lib.flip_set_marker_particle_scale(self._h, float(s)))

    def getMarkerParticleScale(self) -> float:
        v = C.c_double()
        self._c(self._lib.flip_get_marker_particle_scale(self._h, C.byref(v)))
        return v.value

    def buildIsomesh(self):
        """Mesh the current particles now, as the first substep of a frame does."""
        self._c(self._lib.flip_build_isomesh(self._h))

    def getIsomesh(self):
        """The last frame's surface mesh: (vertices (n, 3) float32, triangles (m, 3) int32)."""
        nv, nt = C.c_int(), C.c_int()
        self._c(self._lib.flip_get_isomesh(self._h, C.byref(nv), C.byref(nt), None, None))
        v = np.zeros((nv.value, 3), np.float32)
        t = np.zeros((nt.value, 3), np.int32)
        self._c(self._lib.flip_get_isomesh(self._h, C.byref(nv), C.byref(nt), _ptr(v), _ptr(t)))
        return v, t

    # -- state readback for tests
    def liquid_sdf(self) -> np.ndarray:
        I, J, K = self.dims
        a = np.zeros((K, J, I), np.float32)
        self._c(self._lib.flip_get_liquid_sdf(self._h, _ptr(a)))
        return a

    def solid_sdf(self) -> np.ndarray:
        I, J, K = self.dims
        a = np.zeros((K + 1, J + 1, I + 1), np.float32)
        self._c(self._lib.flip_get_solid_sdf(self._h, _ptr(a)))
        return a

    def mac_velocity(self):
        I, J, K = self.dims
        u = np.zeros((K, J, I + 1), np.float32)
        v = np.zeros((K, J + 1, I), np.float32)
        w = np.zeros((K + 1, J, I), np.float32)
        self._c(self._lib.flip_get_mac_velocity(self._h, _ptr(u), _ptr(v), _ptr(w)))
        return u, v, w

    def binned_particles(self):
        """(positions (n, 3), ids (n,), cell_start (I*J*K + 1,)) as stored on
        the device: sorted by cell, then by id within a cell."""
        n = self.getNumMarkerParticles()
        I, J, K = self.dims
        pos = np.zeros((3, n), np.float32)
        ids = np.zeros(n, np.uint32)
        start = np.zeros(I * J * K + 1, np.int32)
        self._c(self._lib.flip_get_binned_particles(self._h, _ptr(pos), _ptr(ids), _ptr(start)))
        return pos.T.copy(), ids, start

    def set_device_wait_limit(self, polls: int):
        """Poll rounds before a bounded device wait gives up (0: default)."""
        self._c(self._lib.flip_set_device_wait_limit(self._h, int(polls)))

    def inject_sweep_stall(self, on: bool = True):
        """Fault injection: the sweeps' edge waits await terms no tile publishes."""
        self._c(self._lib.flip_inject_sweep_stall(self._h, 1 if on else 0))

    def set_stage_timing(self, enable: bool = True):
        self._c(self._lib.flip_set_stage_timing(self._h, 1 if enable else 0))

    def stage_times(self):
        """(dict stage -> summed device ms, substeps summed)"""
        ms = np.zeros(len(STAGE_NAMES), np.float64)
        n = C.c_longlong()
        self._c(self._lib.flip_get_stage_times(self._h, _ptr(ms), C.byref(n)))
        return dict(zip(STAGE_NAMES, ms.tolist())), n.value

    def sweep_times(self):
        """(summed device ms of the MIC(0) sweep kernels, kernels timed,
        pressure rows swept summed over them), while stage timing is on."""
        ms = C.c_double()
        n = C.c_longlong()
        cells = C.c_longlong()
        self._c(self._lib.flip_get_sweep_times(self._h, C.byref(ms), C.byref(n), C.byref(cells)))
        return ms.value, n.value, cells.value

    def set_sweep_orientation(self, mode: int):
        """Preconditioner sweep tile orientation: -1 chosen per solve (the
        default), 0 lanes along j, 1 lanes along k.  Results are the same."""
        self._c(self._lib.flip_set_sweep_orientation(self._h, int(mode)))

    def sweep_orientation(self) -> int:
        """Orientation used by the last pressure solve."""
        v = C.c_int()
        self._c(self._lib.flip_get_sweep_orientation(self._h, C.byref(v)))
        return v.value

    def device_bytes(self) -> int:
        b = C.c_longlong()
        self._c(self._lib.flip_get_device_bytes(self._h, C.byref(b)))
        return b.value

    def launch_count(self) -> int:
        v = C.c_longlong()
        self._c(self._lib.flip_get_launch_count(self._h, C.byref(v)))
        return v.value

    def host_sync_count(self) -> int:
        """Times this simulation's calls waited on the device so far."""
        v = C.c_longlong()
        self._c(self._lib.flip_get_host_sync_count(self._h, C.byref(v)))
        return v.value

    def update_staged(self, dt: float) -> dict:
        """One single-substep frame; returns the state between the stages."""
        I, J, K = self.dims
        n = self.getNumMarkerParticles()
        su, sv, sw = (K, J, I + 1), (K, J + 1, I), (K + 1, J, I)
        out = {}

        def mk(name, shape, dtype=np.float32):
            out[name] = np.zeros(shape, dtype)
            return _ptr(out[name])

        d = StageDump()
        d.phi = mk("phi", (K, J, I))
        for stage in ("p2g", "force", "press", "final", "saved"):
            setattr(d, "u_" + stage, mk("u_" + stage, su))
            setattr(d, "v_" + stage, mk("v_" + stage, sv))
            setattr(d, "w_" + stage, mk("w_" + stage, sw))
        d.vu_p2g = mk("vu_p2g", su, np.uint8)
        d.vv_p2g = mk("vv_p2g", sv, np.uint8)
        d.vw_p2g = mk("vw_p2g", sw, np.uint8)
        d.pressure = mk("pressure", (K, J, I))
        d.rhs = mk("rhs", (K, J, I), np.float64)
        d.vel_g2p = mk("vel_g2p", (n, 3))
        d.pos_adv = mk("pos_adv", (n, 3))
        d.n_before = mk("n_before", (1,), np.int32)
        d.pcg_iters = mk("pcg_iters", (1,), np.int32)
        d.pcg_error = mk("pcg_error", (1,), np.float64)
        self._c(self._lib.flip_update_staged(self._h, float(dt), C.byref(d)))
        out["positions"] = self.getMarkerParticlePositionData()
        out["velocities"] = self.getMarkerParticleVelocityData()
        return out

    @classmethod
    def from_scene(cls, scene, tolerance=None, surface_subdivisions=None, tuned=False):
        """Set up a seeded scene (flipengine3d_gb300.scenes) the way the
        reference's headless driver does: surface reconstruction off (or on
        at the given subdivision level), PIC ratio, gravity, CFL, tolerance,
        particles, initialize; `tuned` applies the autotuner's settings."""
        sim = cls(scene.isize, scene.jsize, scene.ksize, scene.dx)
        if tuned:
            sim.applyTunedSettings()
        if surface_subdivisions is None:
            sim.disableSurfaceReconstruction()
        else:
            sim.setSurfaceSubdivisionLevel(surface_subdivisions)
        sim.setPICFLIPRatio(scene.pic_ratio)
        sim.addBodyForce(*scene.gravity)
        sim.setCFLConditionNumber(scene.cfl)
        sim.setPressureSolveTolerance(scene.tolerance if tolerance is None else tolerance)
        for ob in getattr(scene, "obstacles", ()):
            sim.addMeshObstacle(*ob)
        if getattr(scene, "jitter_factor", None) is not None:
            sim.setMarkerParticleJitterFactor(scene.jitter_factor)
        if getattr(scene, "viscosity", None) is not None:
            sim.setViscosity(scene.viscosity)
        for fm in getattr(scene, "fluid_meshes", []):
            sim.addMeshFluid(*fm)
        for src in getattr(scene, "sources", []):
            sim.addMeshFluidSource(src["vertices"], src["triangles"],
                                   **{k: v for k, v in src.items() if k not in ("vertices", "triangles")})
        if getattr(scene, "force_fields", []):
            sim.enableForceFields()
            sim.setForceFieldReductionLevel(getattr(scene, "force_field_reduction", 1))
            for ff in scene.force_fields:
                sim.addPointForceField(ff["vertices"], **ff["params"])
        if len(scene.positions):
            sim.loadMarkerParticleData(scene.positions, scene.velocities)
        sim.initialize()
        return sim
