"""In-tree build of the CUDA library (sm_103a) and of the CPU oracle.

`build_library()` compiles flipengine3d_gb300/csrc/*.cu with nvcc for
sm_103a only and links flipengine3d_gb300/_lib/libflip3d_gb300.so.  The
translation units compile in parallel; nothing depends on torch.
`build_oracle()` compiles the test-only C++ oracle (oracle/flip_oracle.cpp)
into oracle/_build/libflip_oracle.so with -ffp-contract=off, so that it
gives the same bits on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIBNAME = "libflip3d_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-I", str(ROOT / "include")]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(out: Path, srcs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in srcs)


def library_path() -> Path:
    return LIBDIR / LIBNAME


def build_library(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = objdir / (src.stem + ".o")
        if force or _stale(obj, [src, *headers]):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = objdir / (src.stem + ".o")
        if force or _stale(obj, [src, *headers]):
            jobs.append(["g++", *CXX_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr)
    wanted = {objdir / (src.stem + ".o") for src in list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp"))}
    for stale in set(objdir.glob("*.o")) - wanted:   # objects of removed sources
        stale.unlink()
    objs = sorted(str(p) for p in wanted)
    out = library_path()
    if force or jobs or not out.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(out), *objs, "-lcudart"])
    return out


def oracle_path() -> Path:
    return ROOT / "oracle" / "_build" / "libflip_oracle.so"


def build_oracle(force: bool = False) -> Path:
    src = ROOT / "oracle" / "flip_oracle.cpp"
    out = oracle_path()
    out.parent.mkdir(parents=True, exist_ok=True)
    if force or _stale(out, [src, ROOT / "oracle" / "flip_oracle.h"]):
        _run(["g++", *CXX_FLAGS, "-shared", "-o", str(out), str(src)])
    return out


def build_reference_checker() -> Path | None:
    """oracle/_ref/libflipref.so from the reference sources, where present.

    oracle/build_ref.sh locates the sources (FLIP_REFERENCE_ROOT) and exits
    with status 2 when they are absent, as on a host without the reference
    tree; then nothing is built and None is returned."""
    script = ROOT / "oracle" / "build_ref.sh"
    r = subprocess.run(["bash", str(script)], capture_output=True, text=True)
    if r.returncode == 2:
        return None
    if r.returncode != 0:
        raise RuntimeError(f"oracle/build_ref.sh failed ({r.returncode}):\n{r.stdout}\n{r.stderr}")
    return ROOT / "oracle" / "_ref" / "libflipref.so"
