"""The MIC(0) preconditioner on its own: the factor and the two triangular
sweeps, on random 7-point systems of the pressure solve's shape (portable
generator: oracle.refsim.random_mic0_system).

* CPU: the oracle's restatement against the golden outputs of the reference's
  own factorModifiedIncompleteColesky0 and solveLower /
  solveLowerTransposeInPlace (tests/golden/units/mic0.npz), bit for bit; and
  against the compiled reference on further systems where it is built here.
* GPU: the library's factor (the solve's tiled wavefront) within 1e-12
  relative of the reference's inverse pivots (its FP64 operation order is
  regrouped, so the last bits may differ), and its FP32 wavefront sweeps
  bit-identical to the reference's sequential float sweeps, in both tile
  orientations.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import refsim

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden" / "units"))
import make_mic0_golden as gold  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "units" / "mic0.npz"
FACTOR_RTOL = 1e-12
# shapes (K, J, I): multi-tile in the sweep layout's lane and warp axes and
# in the factor's 16 x 16 pencil tiles, ragged edges, a long i axis
MORE = [((18, 37, 11), 3), ((12, 13, 70), 2), ((35, 34, 20), 4)]


def golden_cases():
    z = np.load(GOLDEN)
    out = []
    for q in range(len(gold.CASES)):
        shape = tuple(int(v) for v in z[f"c{q}_shape"])
        seed = int(z[f"c{q}_seed"])
        out.append((shape, seed, z[f"c{q}_inv"], z[f"c{q}_lower"], z[f"c{q}_z"]))
    return out


def test_oracle_matches_reference_golden(built):
    for shape, seed, inv_g, low_g, z_g in golden_cases():
        fluid, rows7 = refsim.random_mic0_system(shape, seed)
        m = fluid > 0
        inv, low = refsim.mic0_factor(fluid, rows7, "orc")
        assert np.array_equal(inv[m], inv_g) and np.array_equal(low[m], low_g), shape
        z = refsim.mic0_precondition_f32(fluid, gold.factor_rows(inv, low), gold.rhs(shape, seed), "orc")
        assert np.array_equal(z[m], z_g), shape


@pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")
def test_oracle_matches_reference_routines(built):
    for shape, seed in MORE:
        fluid, rows7 = refsim.random_mic0_system(shape, seed)
        inv_r, low_r = refsim.mic0_factor(fluid, rows7, "ref")
        inv_o, low_o = refsim.mic0_factor(fluid, rows7, "orc")
        assert np.array_equal(inv_r, inv_o) and np.array_equal(low_r, low_o), shape
        fac = gold.factor_rows(inv_r, low_r)
        r = gold.rhs(shape, seed)
        assert np.array_equal(refsim.mic0_precondition_f32(fluid, fac, r, "ref"),
                              refsim.mic0_precondition_f32(fluid, fac, r, "orc")), shape


def _cases_for_gpu():
    for shape, seed, inv_g, low_g, z_g in golden_cases():
        yield shape, seed, ("golden", inv_g, low_g, z_g)
    for shape, seed in MORE:
        yield shape, seed, None


@pytest.mark.gpu
def test_gpu_factor_matches_reference(gpu):
    import flipengine3d_gb300.fluidsimulation as fs
    for shape, seed, g in _cases_for_gpu():
        fluid, rows7 = refsim.random_mic0_system(shape, seed)
        m = fluid > 0
        if g is None:
            inv_ref, _ = refsim.mic0_factor(fluid, rows7, "orc")
            inv_ref = inv_ref[m]
        else:
            inv_ref = g[1]
        inv = fs.mic0_factor(fluid, rows7)
        assert (inv[~m] == 0).all()
        err = np.abs(inv[m] - inv_ref) / np.maximum(np.abs(inv_ref), 1e-300)
        assert err.max() <= FACTOR_RTOL, f"{shape}: inverse pivots differ by {err.max():.3g}"
        assert np.array_equal(inv[m] == 0, inv_ref == 0), f"{shape}: null rows"


@pytest.mark.gpu
@pytest.mark.parametrize("orientation", [0, 1])
def test_gpu_sweeps_bit_identical_to_reference(gpu, orientation):
    import flipengine3d_gb300.fluidsimulation as fs
    for shape, seed, g in _cases_for_gpu():
        fluid, rows7 = refsim.random_mic0_system(shape, seed)
        m = fluid > 0
        r = gold.rhs(shape, seed)
        if g is None:
            inv, low = refsim.mic0_factor(fluid, rows7, "orc")
            fac = gold.factor_rows(inv, low)
            z_ref = refsim.mic0_precondition_f32(fluid, fac, r, "orc")[m]
        else:
            inv = np.zeros(shape)
            low = np.zeros(shape + (3,))
            inv[m], low[m] = g[1], g[2]
            fac = gold.factor_rows(inv, low)
            z_ref = g[3]
        z = fs.mic0_precondition(fluid, fac, r, orientation)
        assert np.array_equal(z[m].view(np.uint32), z_ref.view(np.uint32)), \
            f"{shape}: {int((z[m] != z_ref).sum())} of {int(m.sum())} entries differ"
