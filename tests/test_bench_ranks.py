"""bench.py's multi-rank path on CPU: two gloo ranks stand in for two GPU
replicas.  The whole-job figures are the slowest rank's time and the
particles of all ranks; the reference arm runs on rank 0 only."""
from __future__ import annotations

import argparse
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: its own time and particle count
        got = bench.combine_ranks(10.0 + rank, 2.0 * (rank + 1), 100 * (rank + 1), 7 * (rank + 1), world, "cpu")
        out[rank] = got
        # the reference arm does no work on ranks other than 0
        args = argparse.Namespace(steps=1, warmup=0, reference_max_steps=1, scene="plain_128")
        if rank != 0:
            assert bench.run_reference(args, rank, world) is None
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_max_time_and_summed_particles():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        ms, e2e, p, pe = out[rank]
        assert ms == 11.0 and e2e == 4.0        # slowest rank
        assert p == 300.0 and pe == 21.0         # all ranks' particles


def test_single_rank_is_identity():
    assert bench.combine_ranks(5.0, 1.5, 42, 40, 1, "cpu") == (5.0, 1.5, 42.0, 40.0)


def test_reference_arm_line_keeps_the_contract(built):
    """The reference arm on a small scene: one JSON-able line with the keys
    the bench contract names, the same metric and unit as the GPU arm, and a
    cpu_baseline and e2e block that describe this run."""
    import json
    args = argparse.Namespace(steps=1, warmup=1, reference_max_steps=60, scene="plain_64")
    line = bench.run_reference(args, 0, 1)
    assert line["config"]["frames_timed"] == [2, 2] and line["warmup"] == 1 and line["steps"] == 1
    json.dumps(line)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == bench.METRICS["plain_64"]
    assert line["unit"] == bench.UNIT and line["higher_is_better"] is True and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
