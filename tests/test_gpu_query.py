"""World queries on the GPU (b2g_query_aabb, b2g_ray_cast_closest) against the oracle's
restatement of B2world::query_aabb / ray_cast (its own dynamic tree and the reference's shape ray
casts), on states that are bit-identical (lockstep with the ordering hook).

Bar: the set of fixtures per box equal; per ray the same closest fixture and bit-identical
fraction, point and normal (when two fixtures are hit at exactly the same fraction, either may be
reported: the hierarchies meet them in different orders)."""
import numpy as np
import pytest

import b2g
import parity
import scenes

pytestmark = pytest.mark.gpu


def _random_boxes(rng, n, lo, hi, size):
    c = rng.uniform(lo, hi, (n, 2))
    e = rng.uniform(0.05, size, (n, 2))
    return np.concatenate([c - e, c + e], 1).astype(np.float32)


def _random_rays(rng, n, lo, hi):
    p1 = rng.uniform(lo, hi, (n, 2))
    p2 = rng.uniform(lo, hi, (n, 2))
    return np.concatenate([p1, p2], 1).astype(np.float32)


def _compare_rays(g, o):
    assert len(g) == len(o)
    same = g["fixture"] == o["fixture"]
    for i in np.nonzero(~same)[0]:
        # a tie at exactly the same fraction
        assert g["fixture"][i] >= 0 and o["fixture"][i] >= 0 and g["fraction"][i] == o["fraction"][i], (g[i], o[i])
    for f in ("point", "normal", "fraction"):
        assert np.array_equal(g[f][same], o[f][same]), f
    return int((g["fixture"] >= 0).sum())


def test_queries_match_the_reference_on_a_mixed_pile(built):
    s = scenes.mixed(n_circles=300, n_polygons=300, size=25.0, seed=31)
    recs, gpu, ora = parity.lockstep(s, 80, check_pairs=False, check_contacts=False)
    assert recs[-1]["bitexact_bodies"] and recs[-1]["fat_aabb_equal"]
    rng = np.random.default_rng(7)
    boxes = _random_boxes(rng, 300, -2.0, 27.0, 2.0)
    gq, oq = gpu.query_aabb(boxes), ora.query_aabb(boxes)
    assert len(gq) > 300
    assert np.array_equal(gq, oq)
    rays = _random_rays(rng, 2000, -3.0, 28.0)
    hits = _compare_rays(gpu.ray_cast_closest(rays), ora.ray_cast_closest(rays))
    assert hits > 1000


def test_ray_casts_on_all_shape_kinds(built):
    """Pyramid of boxes on an edge ground plus the throw-and-stack circle: rays from above and
    from the side hit polygons, circles and the edge; polygons ignore hits before fraction
    0.032 (the reference's polygon ray cast starts its entering bound there)."""
    s = scenes.throw_stack(steps=30)
    recs, gpu, ora = parity.lockstep(s, 30, check_pairs=False, check_contacts=False)
    assert recs[-1]["bitexact_bodies"]
    rng = np.random.default_rng(11)
    down = np.stack([rng.uniform(-6, 10, 500), np.full(500, 8.0), rng.uniform(-6, 10, 500), np.full(500, -1.0)], 1)
    side = np.stack([np.full(300, -10.0), rng.uniform(0, 5, 300), np.full(300, 15.0), rng.uniform(0, 5, 300)], 1)
    rays = np.concatenate([down, side]).astype(np.float32)
    g, o = gpu.ray_cast_closest(rays), ora.ray_cast_closest(rays)
    _compare_rays(g, o)
    kinds = set(int(s["fixtures"]["shape_type"][f]) for f in g["fixture"] if f >= 0)
    assert kinds == {b2g.CIRCLE, b2g.EDGE, b2g.POLYGON} or kinds >= {b2g.EDGE, b2g.POLYGON}


def test_batched_worlds_queries_respect_the_world(built):
    s = scenes.batched(num_worlds=4, lo=32, hi=96, seed=9)
    recs, gpu, ora = parity.lockstep(s, 20, check_pairs=False, check_contacts=False)
    rng = np.random.default_rng(3)
    boxes = _random_boxes(rng, 200, -5.0, 15.0, 3.0)
    wi = rng.integers(0, 4, 200).astype(np.uint32)
    q = gpu.query_aabb(boxes, wi)
    world_of_fixture = s["bodies"]["world_index"][s["fixtures"]["body"]]
    assert len(q) > 0
    assert np.all(world_of_fixture[q[:, 1]] == wi[q[:, 0]])


def test_queries_need_a_step(built):
    s = scenes.pyramid(rows=3)
    w = b2g.B2world(gravity=s["gravity"])
    scenes.build_world(w, s)
    with pytest.raises(b2g.B2GError):
        w.ray_cast_closest(np.zeros((1, 4), np.float32) + [0, 5, 0, -5])
    w.close()
