"""Time of impact (b2_time_of_impact with its GJK distance): the oracle's restatement on cases with
analytic answers (CPU), and the GPU's b2g_time_of_impact against the oracle bit for bit on random
pairs of moving circles, polygons and edges."""
import numpy as np
import pytest

import b2g
import oracle

SLOP = 0.005


def _sweep(c0, c, a0=0.0, a=0.0, lc=(0.0, 0.0)):
    s = np.zeros(1, b2g.SWEEP)
    s["local_center"] = lc
    s["c0"] = c0
    s["c"] = c
    s["a0"] = a0
    s["a"] = a
    return s


def _circle(r, p=(0.0, 0.0)):
    return np.atleast_1d(b2g.circle_fixture(0, r, center=p))


def _box(hx, hy):
    return np.atleast_1d(b2g.box_fixture(0, hx, hy))


def test_head_on_circles_touch_at_the_target_distance(oracle_lib):
    """Two circles of radius 0.5: the core distance (between centres) reaches the target
    1 - 3 slop when the moving centre is at x = -0.985, i.e. t = (5 - 0.985) / 10 (the root finder
    stops within 0.25 slop of the target)."""
    out = oracle.time_of_impact(_circle(0.5), _sweep((-5.0, 0.0), (5.0, 0.0)), _circle(0.5), _sweep((0.0, 0.0), (0.0, 0.0)))
    assert out["state"][0] == b2g.TOI_TOUCHING
    target = 1.0 - 3 * SLOP
    x = -5.0 + 10.0 * float(out["t"][0])
    assert abs(-x - target) < 0.25 * SLOP + 1e-6


def test_separated_overlapped_and_late_contact(oracle_lib):
    # never closer than 2 m: separated, t = t_max
    out = oracle.time_of_impact(_circle(0.5), _sweep((-5.0, 3.0), (5.0, 3.0)), _circle(0.5), _sweep((0.0, 0.0), (0.0, 0.0)),
                                t_max=np.array([0.75], np.float32))
    assert out["state"][0] == b2g.TOI_SEPARATED and out["t"][0] == np.float32(0.75)
    # cores overlap at the start: overlapped, t = 0
    out = oracle.time_of_impact(_box(1.0, 1.0), _sweep((0.0, 0.0), (1.0, 0.0)), _box(1.0, 1.0), _sweep((0.5, 0.0), (0.5, 0.0)))
    assert out["state"][0] == b2g.TOI_OVERLAPPED and out["t"][0] == 0.0
    # a box falling onto an edge while turning: touching, with the box's lowest corner at the
    # target distance from the edge (polygon radius + edge radius - 3 slop = 0.005)
    edge = np.atleast_1d(b2g.edge_fixture(0, (-10.0, 0.0), (10.0, 0.0)))
    out = oracle.time_of_impact(_box(0.5, 0.5), _sweep((0.0, 3.0), (0.0, -1.0), 0.0, 0.8), edge, _sweep((0.0, 0.0), (0.0, 0.0)))
    assert out["state"][0] == b2g.TOI_TOUCHING
    t = float(out["t"][0])
    y = 3.0 - 4.0 * t
    ang = 0.8 * t
    lowest = y - 0.5 * (abs(np.cos(ang)) + abs(np.sin(ang)))
    assert abs(lowest - max(SLOP, 2 * 0.01 - 3 * SLOP)) < 0.25 * SLOP + 1e-4


def _random_pairs(n, seed):
    rng = np.random.default_rng(seed)
    da = b2g.fixture_defs(n)
    db = b2g.fixture_defs(n)
    for d in (da, db):
        kind = rng.integers(0, 3, n)
        for i in range(n):
            if kind[i] == 0:
                d[i] = b2g.circle_fixture(0, float(rng.uniform(0.1, 0.6)), center=tuple(rng.uniform(-0.2, 0.2, 2)))
            elif kind[i] == 1:
                k = int(rng.integers(3, 9))
                ang = np.sort(rng.uniform(0, 2 * np.pi, k))
                r = rng.uniform(0.2, 0.7, k)
                d[i] = b2g.polygon_fixture(0, np.stack([r * np.cos(ang), r * np.sin(ang)], 1).astype(np.float32))
            else:
                a = rng.uniform(-2, 2, 2)
                d[i] = b2g.edge_fixture(0, tuple(a), tuple(a + rng.uniform(-3, 3, 2)))
    sa = np.zeros(n, b2g.SWEEP)
    sb = np.zeros(n, b2g.SWEEP)
    for s, spread in ((sa, 4.0), (sb, 1.0)):
        s["local_center"] = rng.uniform(-0.1, 0.1, (n, 2))
        s["c0"] = rng.uniform(-spread, spread, (n, 2))
        s["c"] = s["c0"] + rng.uniform(-spread, spread, (n, 2))
        s["a0"] = rng.uniform(-10, 10, n)
        s["a"] = s["a0"] + rng.uniform(-3, 3, n)
    return da, sa, db, sb


@pytest.mark.gpu
def test_gpu_time_of_impact_matches_the_oracle(built, oracle_lib):
    da, sa, db, sb = _random_pairs(20000, 7)
    t_max = np.random.default_rng(8).uniform(0.5, 1.0, len(da)).astype(np.float32)
    oracle.set_trig(False)  # the project's sin/cos, which the GPU uses
    try:
        ref = oracle.time_of_impact(da, sa, db, sb, t_max)
    finally:
        oracle.set_trig(True)
    got = b2g.time_of_impact(da, sa, db, sb, t_max)
    assert np.array_equal(got["state"], ref["state"])
    assert np.array_equal(got["t"].view(np.uint32), ref["t"].view(np.uint32))
    states = np.bincount(ref["state"], minlength=5)
    assert states[b2g.TOI_TOUCHING] > 1000 and states[b2g.TOI_SEPARATED] > 1000 and states[b2g.TOI_OVERLAPPED] > 100


def _rain_below_plate(continuous):
    import scenes

    s = scenes.toi_rain(n=64, seed=7, steps=120)
    o = oracle.OracleWorld(gravity=s["gravity"], continuous=continuous)
    o.set_key_order(True)
    scenes.build_world(o, s)
    o.steps(s["dt"], s["vi"], s["pi"], s["steps"])
    st = o.get_body_states()
    dyn = s["bodies"]["type"] == b2g.DYNAMIC
    x, y = st["position"][dyn, 0], st["position"][dyn, 1]
    return int(((np.abs(x) < 19.5) & (y < 0.0)).sum()), o.toi_events()


def test_oracle_solve_toi_stops_tunnelling(oracle_lib):
    """B2world::solve_toi in the oracle: bodies at 60-250 m/s pass a 0.1 m static plate in a
    discrete step, and none does with continuous physics on (hundreds of time-of-impact events)."""
    oracle.set_trig(False)
    passed, events = _rain_below_plate(False)
    assert passed > 10 and events == 0
    passed, events = _rain_below_plate(True)
    assert passed == 0 and events > 100
