"""Generate tests/golden/units/mic0.npz from the reference's own MIC(0)
routines (pcgsolver.h: factorModifiedIncompleteColesky0, and solveLower /
solveLowerTransposeInPlace instantiated for float), compiled from the
reference sources by oracle/build_ref.sh.

The systems are oracle.refsim.random_mic0_system(shape, seed), which depends
on (shape, seed) only, so only the reference's outputs on the flagged cells
are stored: the inverse pivots, the scaled factor entries towards +x, +y, +z
and the FP32 preconditioned vector z for a right-hand side r drawn the same
portable way.

    python tests/golden/units/make_mic0_golden.py     # needs the reference sources
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[3]
sys.path.insert(0, str(ROOT))

from oracle import refsim  # noqa: E402

CASES = [((10, 12, 14), 0), ((20, 40, 36), 1)]   # (K, J, I) shape, seed


def rhs(shape, seed):
    return (2.0 * refsim._hash_uniform(seed, 9, shape) - 1.0).astype(np.float32)


def factor_rows(inv, lower):
    """{invdiag, L+x, L+y, L+z} per cell as floats, the FP32 rows the sweeps use."""
    return np.concatenate([inv[..., None], lower], -1).astype(np.float32)


def main():
    out = {}
    for q, (shape, seed) in enumerate(CASES):
        fluid, rows7 = refsim.random_mic0_system(shape, seed)
        inv, lower = refsim.mic0_factor(fluid, rows7, "ref")
        z = refsim.mic0_precondition_f32(fluid, factor_rows(inv, lower), rhs(shape, seed), "ref")
        m = fluid > 0
        out[f"c{q}_shape"] = np.array(shape)
        out[f"c{q}_seed"] = np.array(seed)
        out[f"c{q}_inv"] = inv[m]
        out[f"c{q}_lower"] = lower[m]
        out[f"c{q}_z"] = z[m]
    np.savez_compressed(Path(__file__).resolve().parent / "mic0.npz", **out)
    print("wrote mic0.npz")


if __name__ == "__main__":
    main()
