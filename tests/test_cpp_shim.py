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
