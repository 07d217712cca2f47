"""The allocation-free particle ordering entry point, through the C ABI.

flip_order_particles_by_id_noalloc works in a static device array instead of
context buffers; its output must equal the context readback's
(getMarkerParticlePositionData) for the same particles, call after call,
although every call reuses the same scratch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from flipengine3d_gb300 import FluidSimulation
from flipengine3d_gb300 import fluidsimulation as fs
from flipengine3d_gb300.scenes import dam_break


def _order_on_device(torch, pos, ids, id_space, stream):
    """Shuffle (pos, ids) consistently, upload as caller-owned device
    buffers, order them with the no-allocation entry point, return host xyz."""
    dev = torch.device("cuda:0")
    px = torch.from_numpy(np.ascontiguousarray(pos[:, 0])).to(dev)
    py = torch.from_numpy(np.ascontiguousarray(pos[:, 1])).to(dev)
    pz = torch.from_numpy(np.ascontiguousarray(pos[:, 2])).to(dev)
    di = torch.from_numpy(ids.astype(np.int32)).to(dev)   # bit pattern of the uint32 ids
    out = torch.full((3 * len(pos),), float("nan"), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    fs.order_particles_by_id_noalloc(px.data_ptr(), py.data_ptr(), pz.data_ptr(), di.data_ptr(), len(pos),
                                     id_space, out.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    return out.cpu().numpy().reshape(-1, 3)


@pytest.mark.gpu
def test_noalloc_order_matches_context_readback_twice(gpu):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(17)
    sc = dam_break(20, seed=11, sphere=True)
    with FluidSimulation.from_scene(sc) as sim:
        results = []
        for call, id_space in enumerate((200_000, fs.FLIP_NOALLOC_MAX_IDS)):
            sim.update(sc.frame_dt)
            ref = sim.getMarkerParticlePositionData()   # the context readback, in id order
            n = len(ref)
            ids = np.sort(rng.choice(id_space, size=n, replace=False)).astype(np.uint32)
            perm = rng.permutation(n)                     # any storage order
            got = _order_on_device(torch, ref[perm], ids[perm], id_space, stream)
            assert got.shape == ref.shape, f"call {call}"
            assert np.array_equal(got, ref), f"call {call}: differs from the context readback"
            results.append(n)
        assert results[0] > 0 and results[1] > 0


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_its_limit(gpu):
    lib = fs.load_library()
    rc = lib.flip_order_particles_by_id_noalloc(None, None, None, None, 1, fs.FLIP_NOALLOC_MAX_IDS + 1, None, None)
    assert rc == fs.FLIP_E_OUT_OF_RANGE
    assert b"no-allocation limit" in lib.flip_last_error()
    with pytest.raises(IndexError):
        fs.order_particles_by_id_noalloc(0, 0, 0, 0, 1, fs.FLIP_NOALLOC_MAX_IDS + 1, 0)


@pytest.mark.gpu
def test_noalloc_edge_cases(gpu):
    """n = 0 writes nothing; id_space = n (every rank used); an id at or
    above id_space is skipped and only the rows of the in-range ids are
    written, the rest of the caller's buffer keeps its contents."""
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(5)

    def run(pos, ids, id_space, rows):
        px, py, pz = (torch.from_numpy(np.ascontiguousarray(pos[:, c])).to(dev) for c in range(3))
        di = torch.from_numpy(np.asarray(ids, np.uint32).astype(np.int32)).to(dev)
        out = torch.full((3 * rows,), -7.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        fs.order_particles_by_id_noalloc(px.data_ptr(), py.data_ptr(), pz.data_ptr(), di.data_ptr(), len(pos),
                                         id_space, out.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        return out.cpu().numpy().reshape(-1, 3)

    # n = 0: the output is left untouched
    empty = run(np.zeros((1, 3), np.float32)[:0], [], 16, 4)
    assert (empty == -7.0).all()
    # id_space = n: a permutation of 0..n-1
    n = 4097
    pos = rng.random((n, 3), dtype=np.float32)
    ids = rng.permutation(n).astype(np.uint32)
    got = run(pos, ids, n, n)
    assert np.array_equal(got, pos[np.argsort(ids)])
    # one id at or above id_space: skipped; the first n-1 rows hold the others
    ids2 = ids.copy()
    far = int(np.argmax(ids2))
    ids2[far] = n + 3
    got = run(pos, ids2, n, n)
    keep = np.array([q for q in np.argsort(ids2) if q != far])
    assert np.array_equal(got[: n - 1], pos[keep])
    assert (got[n - 1] == -7.0).all()
