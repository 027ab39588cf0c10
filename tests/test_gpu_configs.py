"""Lockstep parity at the benchmark configurations' stated sizes.

Each test steps the full-size scene on the GPU and checks windows of it against the oracle (the CPU
restatement of box2d-rs's step) solved in the GPU's constraint order:

  mixed 100k    50k circles + 50k 3-8-gons in a 1000 x 1000 m walled box: steps 1-20 from the start,
                and steps 301-320 after the GPU has run 300 steps alone and the oracle has imported
                its state (bodies, fat AABBs, the contact table with manifolds and impulses);
  pile 250k     250k boxes dropped into a 100 x 400 m walled container: steps 981-983 of the
                1000-step scene, from the GPU's state at step 980 (about 2.4 million contact points;
                the falling column's stretched fat AABBs push the table past 16M entries on the way,
                and the world grows its capacities as it steps);
  batch 4096    4096 worlds of 16-2048 bodies (log-uniform, 1.7M bodies): the GPU steps the whole
                batch; 64 worlds of every log2 size bucket (7 buckets) are restated one oracle world
                each, for steps 1-10 and for steps 151-160 from the GPU's state at step 150.

Bar on every checked step: bodies bit-exact (position, angle, velocities, centre), fat AABBs
bit-exact, the broadphase's pair set equal, every live contact present on both sides with the same
touching flag, manifold type and feature ids, and manifold geometry and impulses within 1e-5
(observed: equal). The differentiable configuration at its stated size (240 steps, one world and
512 worlds) is in test_gpu_adjoint.py.
"""
import numpy as np
import pytest

import parity
import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _check(recs):
    assert recs, "no steps checked"
    for r in recs:
        assert r["hook_misses"] == 0, r
        assert r["bitexact_bodies"] and r["body_rel"] <= TOL, r
        assert r["fat_aabb_equal"], r
        assert r.get("pairs_equal", True), r
        assert r["contact_key_mismatch"] == 0 and r["contact_id_mismatch"] == 0, r
        assert r["manifold_max_diff"] <= TOL, r


def test_mixed_100k_opening_window(built, oracle_lib):
    scene = scenes.mixed()
    assert scene["n_dynamic"] == 100_000
    recs = parity.lockstep_window(scene, 20, skip=0)
    _check(recs)
    assert recs[-1]["contacts"] > 1000


def test_mixed_100k_window_at_step_300(built, oracle_lib):
    scene = scenes.mixed()
    recs = parity.lockstep_window(scene, 20, skip=300)
    _check(recs)
    assert recs[-1]["constraints"] > 20_000, "expected the floor's resting contacts"


def test_pile_250k_settled_window(built, oracle_lib):
    scene = scenes.pile()
    assert scene["n_dynamic"] == 250_000
    scene["contact_capacity"] = 16_000_000
    scene["pair_capacity"] = 4_000_000
    scene["auto_grow"] = True
    recs = parity.lockstep_window(scene, 3, skip=980)
    _check(recs)
    assert recs[-1]["constraints"] > 200_000, recs[-1]


def _bucket_sample(scene, per_bucket=64):
    sizes = np.asarray(scene["world_body_counts"])
    bucket = np.floor(np.log2(sizes)).astype(int)
    pick = []
    for b in np.unique(bucket):
        members = np.nonzero(bucket == b)[0]
        pick.extend(members[np.linspace(0, len(members) - 1, min(per_bucket, len(members))).astype(int)].tolist())
    return sorted(set(pick)), len(np.unique(bucket))


@pytest.mark.parametrize("skip,steps", [(0, 10), (150, 10)])
def test_batch_4096_bucket_sample(built, oracle_lib, skip, steps):
    scene = scenes.batched()
    assert scene["num_worlds"] == 4096
    worlds, buckets = _bucket_sample(scene)
    assert buckets == 7 and len(worlds) >= 64 * 7
    recs = parity.lockstep_window(scene, steps, skip=skip, worlds=worlds)
    _check(recs)
