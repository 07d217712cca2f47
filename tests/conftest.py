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


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    return meta, {k: z[k] for k in z.files if k != "meta"}


def rel_err(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.abs(b).max(initial=0.0), 1e-30)
    return float(np.abs(a - b).max(initial=0.0) / scale)
