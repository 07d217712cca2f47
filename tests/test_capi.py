"""C ABI on the CPU: the library loads, exports every entry point that
include/*.h declares, validates arguments before touching a device, and its
device-free wall set-up equals the oracle's bit for bit."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT, cuda_device_count
from flipengine3d_gb300 import build, fluidsimulation as fs
from oracle import refsim


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(flip_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_api():
    names = declared_functions()
    for n in ("flip_create", "flip_update", "flip_initialize", "flip_load_marker_particle_data",
              "flip_get_marker_particle_position_data", "flip_set_pic_flip_ratio", "flip_add_body_force"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(str(build.library_path()))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header(built):
    declared = set(declared_functions()) - {"flip_last_error"}
    assert declared == set(fs.SIGNATURES), declared ^ set(fs.SIGNATURES)


def test_create_rejects_bad_dimensions_before_any_device_call(built):
    lib = fs.load_library()
    h = C.c_void_p()
    assert lib.flip_create(0, 8, 8, 0.1, C.byref(h)) == fs.FLIP_E_DOMAIN
    assert lib.flip_create(8, 8, 8, -1.0, C.byref(h)) == fs.FLIP_E_DOMAIN
    assert lib.flip_create(8, 8, 8, 0.1, None) == fs.FLIP_E_NULL
    with pytest.raises(ValueError):
        fs.FluidSimulation(4, -1, 4, 0.25)


@pytest.mark.skipif(cuda_device_count() > 0, reason="a CUDA device is present")
def test_create_without_device_fails_loudly(built):
    with pytest.raises(fs.FlipCudaError):
        fs.FluidSimulation(8, 8, 8, 1 / 8)


def test_null_context_is_rejected(built):
    lib = fs.load_library()
    assert lib.flip_update(None, 0.01) == fs.FLIP_E_NULL
    assert lib.flip_initialize(None) == fs.FLIP_E_NULL


@pytest.mark.parametrize("dims", [(32, 32, 32), (43, 43, 43), (24, 17, 30), (64, 48, 20)])
def test_domain_solid_setup_matches_oracle(built, dims):
    I, J, K = dims
    dx = 1.0 / I
    nodal, weights, near = fs.compute_domain_solid(I, J, K, dx, 5)
    orc = refsim.OracleSimulation(I, J, K, dx)
    assert np.array_equal(nodal, orc.solid_phi())
    for a, b in zip(weights, orc.weights()):
        assert np.array_equal(a, b)
    assert np.array_equal(near, orc.near_solid())


def test_runtime_and_estimate_checks_need_no_device(built):
    lib = fs.load_library()
    h = C.c_void_p()
    assert lib.flip_runtime_create(0, 0, C.byref(h)) == fs.FLIP_E_DOMAIN
    assert lib.flip_runtime_create(4, -1, C.byref(h)) == fs.FLIP_E_DOMAIN
    assert lib.flip_runtime_submit(None, None, 0.01, 1, None) == fs.FLIP_E_NULL
    b = C.c_longlong()
    assert lib.flip_estimate_device_bytes(0, 8, 8, 10, C.byref(b)) == fs.FLIP_E_DOMAIN
    small = fs.estimate_device_bytes(32, 32, 32, 100_000)
    big = fs.estimate_device_bytes(128, 128, 128, 4_000_000)
    assert 0 < small < big
    # 128^3 with 4M particles: grids + system + particles, between 0.5 and 2 GB
    assert 5e8 < big < 2e9
