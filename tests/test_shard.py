"""Sharding a world batch across ranks (CPU; world_size 2 over gloo).

Each rank takes its contiguous world range of a batched scene (box2d-rs_gb300/shard.py), steps
it in the oracle, and the gathered results must equal the unsharded run bit for bit: worlds
never interact, so the split needs no collective on the data path.
"""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import shard

STEPS = 20


def test_world_range_partitions_the_batch():
    for n in (1, 5, 8, 4096, 4097):
        for ws in (1, 2, 3, 8):
            ranges = [shard.world_range(n, r, ws) for r in range(ws)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(ws - 1))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.world_range(4, 2, 2)


def test_shard_scene_keeps_each_world_intact():
    import scenes

    s = scenes.batched(num_worlds=7, lo=16, hi=64, seed=11)
    parts = [shard.shard_scene(s, r, 3) for r in range(3)]
    assert sum(p["num_worlds"] for p in parts) == 7
    assert np.array_equal(np.concatenate([p["body_ids"] for p in parts]), np.arange(len(s["bodies"])))
    assert np.array_equal(np.concatenate([p["fixture_ids"] for p in parts]), np.arange(len(s["fixtures"])))
    for p in parts:
        fb = p["fixtures"]["body"]
        assert fb.min() >= 0 and fb.max() < len(p["bodies"])
        # every fixture stays on the same body as in the full scene
        assert np.array_equal(p["body_ids"][fb], s["fixtures"]["body"][p["fixture_ids"]])
        assert p["bodies"]["world_index"].min() == 0
        assert p["bodies"]["world_index"].max() == p["num_worlds"] - 1


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _run_shard(rank, world_size, port, out_path):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [os.path.join(root, "box2d-rs_gb300"), os.path.join(root, "oracle")]
    import parity
    import scenes
    import shard as sh

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    try:
        s = scenes.batched(num_worlds=6, lo=16, hi=48, seed=5, steps=STEPS)
        part = sh.shard_scene(s, rank, world_size)
        ora = parity.MultiOracle(part, allow_sleep=False)
        for _ in range(STEPS):
            ora.step(s["dt"], s["vi"], s["pi"])
        states = ora.get_body_states()
        gathered = [None] * world_size
        dist.all_gather_object(gathered, (part["body_ids"], states))
        if rank == 0:
            ids = np.concatenate([g[0] for g in gathered])
            st = np.concatenate([g[1] for g in gathered])
            np.save(out_path, st[np.argsort(ids)])
    finally:
        dist.destroy_process_group()


def test_two_ranks_reproduce_the_unsharded_batch(tmp_path):
    import parity
    import scenes

    out = str(tmp_path / "sharded.npy")
    mp.spawn(_run_shard, args=(2, _free_port(), out), nprocs=2, join=True)
    s = scenes.batched(num_worlds=6, lo=16, hi=48, seed=5, steps=STEPS)
    ora = parity.MultiOracle(s, allow_sleep=False)
    for _ in range(STEPS):
        ora.step(s["dt"], s["vi"], s["pi"])
    full = ora.get_body_states()
    got = np.load(out)
    for f in parity.BODY_FIELDS:
        assert np.array_equal(got[f], full[f]), f
