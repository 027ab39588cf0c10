"""Sharding a batch of independent worlds across ranks (one GPU per rank).

Worlds of a batch never interact, so a batch splits by contiguous world ranges with no data-path
collective: rank r steps worlds [lo, hi) as its own batch and only the results are gathered. A
single world does not split (a spatial decomposition would exchange halos every colour sweep);
it runs as replicas.
"""
from __future__ import annotations

import numpy as np


def world_range(num_worlds: int, rank: int, world_size: int) -> tuple[int, int]:
    """[lo, hi) of rank's worlds: contiguous, disjoint, covering all, sizes differing by at most 1."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("need 0 <= rank < world_size")
    base, extra = divmod(num_worlds, world_size)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_scene(scene: dict, rank: int, world_size: int) -> dict:
    """The sub-scene with worlds [lo, hi) of a batched scene: bodies and fixtures of those worlds
    in their original order, world indices shifted to start at 0 and fixture body ids remapped.
    `body_ids` / `fixture_ids` give each entry's id in the full scene."""
    lo, hi = world_range(scene["num_worlds"], rank, world_size)
    bodies, fixtures = scene["bodies"], scene["fixtures"]
    wi = bodies["world_index"].astype(np.int64)
    bidx = np.nonzero((wi >= lo) & (wi < hi))[0]
    remap = np.full(len(bodies), -1, np.int64)
    remap[bidx] = np.arange(len(bidx))
    fidx = np.nonzero(remap[fixtures["body"].astype(np.int64)] >= 0)[0]
    bd = bodies[bidx].copy()
    bd["world_index"] = wi[bidx] - lo
    fx = fixtures[fidx].copy()
    fx["body"] = remap[fixtures["body"][fidx].astype(np.int64)]
    out = dict(scene)
    out.update(bodies=bd, fixtures=fx, num_worlds=hi - lo, world_lo=lo, world_hi=hi, body_ids=bidx,
               fixture_ids=fidx, n_dynamic=int((bd["type"] == 2).sum()))
    if "world_body_counts" in scene:
        out["world_body_counts"] = np.asarray(scene["world_body_counts"])[lo:hi]
    return out
