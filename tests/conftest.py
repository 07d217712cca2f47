"""Shared test set-up.

Markers: `gpu` tests need a CUDA device and run the product library on it;
everything else runs on the CPU (oracle, host logic, C-ABI exports).
"""
from __future__ import annotations

import ctypes
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


def cuda_device_count() -> int:
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    else:
        return 0
    n = ctypes.c_int(0)
    if rt.cudaGetDeviceCount(ctypes.byref(n)) != 0:
        return 0
    return n.value


@pytest.fixture(scope="session")
def built():
    """Build the library and the oracle once (no-ops when up to date)."""
    from flipengine3d_gb300 import build as b
    b.build_library()
    b.build_oracle()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    if cuda_device_count() == 0:
        pytest.skip("no CUDA device")
    return True


def viscosity_cases():
    """Fixtures of scenes with viscosity (visc*.npz)."""
    return sorted(p.stem for p in GOLDEN.glob("visc*.npz"))


def surface_cases():
    """Fixtures of the reference's surface meshes (iso_*.npz)."""
    return sorted(p.stem for p in GOLDEN.glob("iso_*.npz"))


def golden_cases(stages=False):
    """Fixture names of simulation states (not the surface meshes); with
    stages, only those holding the first frame stage by stage (the
    fluid-mesh fixtures hold the particles after each frame)."""
    names = sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("iso_", "visc")))
    if stages:
        names = [n for n in names
                 if json.loads(str(np.load(GOLDEN / f"{n}.npz")["meta"])).get("builder") not in (
                     "mesh_fluid", "fluid_sources", "force_fields")]
    return names


def golden_scene(meta):
    """The scene a fixture was made from (scenes.dam_break, or the builder
    the fixture names, with its recorded arguments)."""
    from flipengine3d_gb300 import scenes
    return getattr(scenes, meta.get("builder", "dam_break"))(**meta["scene"])


def load_golden(name):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    return meta, {k: z[k] for k in z.files if k != "meta"}


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(initial=0.0), 1e-30)
    return float(np.abs(a - b).max(initial=0.0) / scale)


def aligned_rel_err(a, b, max_skips=3, tol=1e-4):
    """rel_err of two particle arrays in particle order that may each lack a
    few particles of the other (a particle on the solid boundary removed on
    one side only).  Matches the rows in order, skipping a row of either
    side where they disagree by more than `tol` (relative); returns (error
    over the matched rows, skips), or (inf, skips) past max_skips."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(initial=0.0), 1e-30)
    close = lambda x, y: float(np.abs(x - y).max()) / scale <= tol
    i = j = skips = 0
    err = 0.0
    while True:
        m = min(len(a) - i, len(b) - j)
        d = np.abs(a[i:i + m] - b[j:j + m]).max(axis=1, initial=0.0) / scale if m else np.zeros(0)
        bad = np.flatnonzero(d > tol)
        k = int(bad[0]) if len(bad) else m
        if k:
            err = max(err, float(d[:k].max()))
        i += k
        j += k
        if k == m:
            skips += (len(a) - i) + (len(b) - j)
            return (err if skips <= max_skips else float("inf")), skips
        if i + 1 < len(a) and close(a[i + 1], b[j]):
            i += 1
        elif j + 1 < len(b) and close(a[i], b[j + 1]):
            j += 1
        else:
            return float("inf"), skips
        skips += 1
        if skips > max_skips:
            return float("inf"), skips
