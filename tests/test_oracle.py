"""The CPU oracle, pinned: against the golden fixtures made by the reference
engine (always), and against the reference engine itself where its sources
are present (oracle/_ref built by oracle/build_ref.sh)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, golden_scene, load_golden
from flipengine3d_gb300.scenes import dam_break
from oracle import refsim

STAGES = ("phi", "vu_p2g", "vv_p2g", "vw_p2g", "u_p2g", "v_p2g", "w_p2g", "pressure", "u_final", "v_final",
          "w_final", "vel_g2p", "pos_adv")


def wall_cases():
    """Fixtures of scenes with the domain walls only: the oracle port restates
    the walls; obstacle scenes are pinned by the reference's fixtures alone."""
    return [c for c in golden_cases() if load_golden(c)[0].get("builder", "dam_break") == "dam_break"]


@pytest.mark.parametrize("case", wall_cases())
def test_oracle_matches_golden_bit_exact(built, case):
    meta, g = load_golden(case)
    sc = golden_scene(meta)
    orc = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=meta["threads"])
    orc.setup(sc, tolerance=meta["tolerance"])
    st = orc.update_staged(meta["dt"])
    for k in STAGES:
        assert np.array_equal(st[k], g[k]), f"{case}: stage {k} differs from the reference"
    assert int(st["pcg_iters"][0]) == int(g["pcg_iters"][0])
    assert np.array_equal(st["positions"], g["positions_1"])
    assert np.array_equal(st["velocities"], g["velocities_1"])
    for _ in range(2, meta["frames"] + 1):
        orc.update(meta["dt"])
    pos, vel = orc.particles()
    f = meta["frames"]
    assert np.array_equal(pos, g[f"positions_{f}"])
    assert np.array_equal(vel, g[f"velocities_{f}"])


needs_ref = pytest.mark.skipif(not refsim.available("ref"), reason="reference checker (oracle/_ref) not built")


@needs_ref
@pytest.mark.parametrize("kw,threads,frames", [
    (dict(n=21, seed=11, sphere=True), 1, 3),
    (dict(n=18, jsize=23, ksize=14, dx=1 / 18, seed=4, fill=(0.7, 0.5, 0.8)), 3, 2),
])
def test_oracle_matches_reference_engine(built, kw, threads, frames):
    sc = dam_break(**kw)
    a = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=threads).setup(sc, tolerance=1e-9)
    b = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=threads).setup(sc, tolerance=1e-9)
    A = a.update_staged(sc.frame_dt)
    B = b.update_staged(sc.frame_dt)
    for k in STAGES + ("rhs", "positions", "velocities"):
        assert np.array_equal(A[k], B[k]), k
    for _ in range(frames - 1):
        a.update(sc.frame_dt)
        b.update(sc.frame_dt)
    pa, va = a.particles()
    pb, vb = b.particles()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    assert np.array_equal(a.solid_phi(), b.solid_phi())
    assert all(np.array_equal(x, y) for x, y in zip(a.weights()[:3], b.weights()))
    assert np.array_equal(a.near_solid(), b.near_solid())


@needs_ref
def test_oracle_matches_reference_empty_and_outside(built):
    """No particles inside the domain: both load nothing and step quietly."""
    n = 10
    sc = dam_break(n, seed=0)
    sc.positions = (sc.positions + 5.0).astype(np.float32)      # all outside the domain box
    a = refsim.RefSimulation(n, n, n, sc.dx).setup(sc)
    b = refsim.OracleSimulation(n, n, n, sc.dx).setup(sc)
    for _ in range(2):
        a.update(sc.frame_dt)
        b.update(sc.frame_dt)
    assert a.particles()[0].shape[0] == 0 and b.particles()[0].shape[0] == 0
    assert np.array_equal(a.liquid_phi(), b.liquid_phi())


def test_oracle_threads_do_not_change_results(built):
    """The port's threaded loops write disjoint outputs computed the same way,
    so below the reference's 500k-row dot partition the thread count changes
    no bit."""
    sc = dam_break(20, seed=6, sphere=True)
    out = []
    for threads in (1, 5):
        o = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=threads).setup(sc, tolerance=1e-9)
        st = o.update_staged(sc.frame_dt)
        o.update(sc.frame_dt)
        out.append((st, o.particles()))
    (a, pa), (b, pb) = out
    for k in STAGES + ("rhs", "positions", "velocities"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(pa[0], pb[0]) and np.array_equal(pa[1], pb[1])


@needs_ref
def test_oracle_matches_reference_engine_at_full_size(built):
    """128^3, ~4.2M particles, 8 threads: past the reference's 500k-row dot
    partition and its particle container's fragment boundaries.  With the
    reference's particles held in fragments larger than the particle count
    (see the next test), every stage dump is bit-identical."""
    from flipengine3d_gb300.scenes import plain_128
    sc = plain_128()
    a = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8, one_particle_fragment=True).setup(sc)
    b = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8).setup(sc)
    A = a.update_staged(sc.frame_dt)
    B = b.update_staged(sc.frame_dt)
    for k in A:
        assert A[k].shape == B[k].shape and np.array_equal(A[k], B[k]), k


@needs_ref
def test_reference_particle_container_aliases_fragment_starts(built):
    """The reference's FragmentedVector finds an element's fragment as
    (int)(i * (1.0 / n)) with n = 5e6 / 24 = 208,333 marker particles per
    fragment (fragmentedvector.h:141-153, 295-302).  For some multiples
    i = k n the product rounds below k, so element i reads as element
    (k - 1) n.  Loading goes through such a container, so with its default
    fragments the reference replaces exactly those particles by copies; this
    library and the oracle load every particle as given."""
    from flipengine3d_gb300.scenes import plain_128
    sc = plain_128()
    n = 5_000_000 // 24
    inv = 1.0 / n
    aliased = [k * n for k in range(1, sc.num_particles // n + 1) if int(k * n * inv) < k]
    assert aliased, "the seeded scene spans aliased fragment starts"
    r = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8).setup(sc)
    pos, _ = r.particles()
    differ = np.nonzero((pos != sc.positions).any(axis=1))[0].tolist()
    assert differ == aliased
    # each is a copy of an earlier fragment start (the readback reads through
    # the same index arithmetic, so a copy of a copy reaches back two)
    assert all(any(np.array_equal(pos[i], sc.positions[i - m * n]) for m in (1, 2)) for i in aliased)


@needs_ref
def test_oracle_tracks_reference_engine_ten_frames_at_64(built):
    """The 64^3 configuration at full size (486k particles), all 10 frames:
    particle positions and velocities bit-identical every frame."""
    from flipengine3d_gb300.scenes import plain_64
    sc = plain_64()
    a = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8, one_particle_fragment=True).setup(sc)
    b = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8).setup(sc)
    for f in range(sc.steps):
        a.update(sc.frame_dt)
        b.update(sc.frame_dt)
        pa, va = a.particles()
        pb, vb = b.particles()
        assert pa.shape == pb.shape, f"frame {f + 1}: particle count"
        assert np.array_equal(pa, pb) and np.array_equal(va, vb), f"frame {f + 1}"


@needs_ref
def test_oracle_matches_reference_engine_at_256x128x128(built):
    """The largest configuration (256x128x128, ~15M particles, FLIP blend
    0.98): every stage dump of the first frame bit-identical."""
    from flipengine3d_gb300.scenes import mixed_256
    sc = mixed_256()
    a = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8, one_particle_fragment=True).setup(sc)
    b = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=8).setup(sc)
    A = a.update_staged(sc.frame_dt)
    B = b.update_staged(sc.frame_dt)
    for k in A:
        assert A[k].shape == B[k].shape and np.array_equal(A[k], B[k]), k


@needs_ref
@pytest.mark.parametrize("kind,edge_or_index", [("mixed", 32), ("mixed", 48), ("mixed", 80), ("served", 6),
                                                ("served", 1)])
def test_oracle_matches_reference_engine_on_the_multi_scene_sets(built, kind, edge_or_index):
    """Scenes of the batched set (the first of each edge 32, 48, 80; fills
    0.2-0.6) and of the served set (4-8 particles per cell, tolerance 1e-5):
    two frames bit-identical."""
    from flipengine3d_gb300 import scenes
    if kind == "mixed":
        q = next(i for i, (e, _) in enumerate(scenes.mixed_scene_params(64)) if e == edge_or_index)
        sc = scenes.mixed_scene(q)
    else:
        sc = scenes.served_scene(edge_or_index)
    a = refsim.RefSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=4, one_particle_fragment=True).setup(sc)
    b = refsim.OracleSimulation(sc.isize, sc.jsize, sc.ksize, sc.dx, threads=4).setup(sc)
    for f in range(2):
        a.update(sc.frame_dt)
        b.update(sc.frame_dt)
        pa, va = a.particles()
        pb, vb = b.particles()
        assert pa.shape == pb.shape and np.array_equal(pa, pb) and np.array_equal(va, vb), f"{sc.name} frame {f + 1}"
