"""The broadphase hierarchy kept between passes (moved leaves updated in place, ancestors grown)
against a hierarchy rebuilt every pass.

With the grid-wide solve order (part-local solve off) nothing downstream of the broadphase depends on
the hierarchy's shape, so a world that keeps its hierarchy and one that rebuilds it every pass must
stay bit for bit equal: bodies, the pair set of every pass, the whole contact table, and the world
queries that walk the kept hierarchy. The default (part-local) order is covered by the lockstep
tests against the oracle, which compare the pair set of every pass."""
import numpy as np
import pytest

import b2g
import scenes

pytestmark = pytest.mark.gpu


def _world(s, max_age):
    w = b2g.B2world(gravity=s["gravity"])
    w.set_allow_sleeping(False)
    w.set_part_solve(False)
    w.set_record_pairs(True)
    w.set_hierarchy_max_age(max_age)
    scenes.build_world(w, s)
    return w


def _pairs(w):
    p = w.get_pairs()
    return set(map(tuple, np.sort(p, axis=1).tolist()))


@pytest.mark.parametrize("seed", [2, 9])
def test_kept_hierarchy_equals_rebuilt(built, seed):
    size = 45.0
    s = scenes.mixed(n_circles=1500, n_polygons=1500, size=size, seed=seed, steps=150)
    kept, fresh = _world(s, 16), _world(s, 0)
    rng = np.random.default_rng(seed)
    ages = []
    for k in range(150):
        for w in (kept, fresh):
            w.step(s["dt"], s["vi"], s["pi"])
        ages.append(kept.get_step_stats()["hierarchy_age"])
        assert fresh.get_step_stats()["hierarchy_age"] == 0
        a, b = kept.get_body_states(), fresh.get_body_states()
        for f in b2g.BODY_STATE.names:
            assert np.array_equal(a[f], b[f]), (k, f)
        assert _pairs(kept) == _pairs(fresh), k
        ca, cb = kept.get_contacts(), fresh.get_contacts()
        assert len(ca) == len(cb), k
        for f in ca.dtype.names:
            assert np.array_equal(ca[f], cb[f]), (k, f)
        if k % 10 == 9:  # the queries walk the kept hierarchy too
            lo = rng.uniform(0.0, size, (64, 2)).astype(np.float32)
            boxes = np.concatenate([lo, lo + rng.uniform(0.5, 6.0, (64, 2)).astype(np.float32)], axis=1)
            qa = set(map(tuple, kept.query_aabb(boxes).tolist()))
            qb = set(map(tuple, fresh.query_aabb(boxes).tolist()))
            assert qa == qb, k
            rays = np.concatenate([lo, lo + rng.uniform(-10.0, 10.0, (64, 2)).astype(np.float32)], axis=1)
            ra, rb = kept.ray_cast_closest(rays), fresh.ray_cast_closest(rays)
            assert np.array_equal(ra["fraction"], rb["fraction"]), k
    ages = np.array(ages)
    assert (ages > 0).sum() >= 50, "expected many passes to keep the hierarchy"
    assert (ages == 0).sum() >= 150 // 17, "expected periodic rebuilds"
    kept.close()
    fresh.close()


def test_kept_hierarchy_after_host_edits(built):
    """Host edits between steps (a teleported body, destroyed bodies, new bodies); the worlds stay
    equal through them."""
    s = scenes.mixed(n_circles=600, n_polygons=600, size=30.0, seed=4, steps=60)
    kept, fresh = _world(s, 16), _world(s, 0)
    nb = len(s["bodies"])
    for k in range(60):
        if k == 20:
            for w in (kept, fresh):
                w.set_transform(7, (0.0, 0.0), 0.3)
                w.set_linear_velocity(8, (30.0, 0.0))
        if k == 30:
            for w in (kept, fresh):
                w.destroy_bodies([11, 12, 300])
        if k == 40:
            bd = b2g.body_defs(4)
            bd["type"] = b2g.DYNAMIC
            bd["position"][:, 0] = 12.0 + np.arange(4) * 1.5
            bd["position"][:, 1] = 27.0
            fx = np.concatenate([b2g.circle_fixture(nb + i, 0.4, density=1.0) for i in range(4)])
            for w in (kept, fresh):
                w.create_bodies(bd)
                w.create_fixtures(fx)
            nb += 4
        for w in (kept, fresh):
            w.step(s["dt"], s["vi"], s["pi"])
        # destroyed proxies rebuild the hierarchy at the step's pass; new proxies at the step's first
        # pass (of the new fixtures), which the step's own pass then keeps; a teleport moves a leaf
        if k == 30:
            assert kept.get_step_stats()["hierarchy_age"] == 0, k
        if k == 40:
            assert kept.get_step_stats()["hierarchy_age"] == 1, k
        a, b = kept.get_body_states(), fresh.get_body_states()
        for f in b2g.BODY_STATE.names:
            assert np.array_equal(a[f], b[f]), (k, f)
        assert _pairs(kept) == _pairs(fresh), k
    kept.close()
    fresh.close()
