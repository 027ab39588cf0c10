"""The oracle (CPU restatement of box2d-rs's step path) against the reference's own
known-answer tests, plus properties the rest of the suite relies on. CPU only."""
import math
import os

import numpy as np
import pytest

import b2g
import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(params=[True, False], ids=["libm", "b2g_trig"])
def trig(request, oracle_lib):
    oracle_lib.set_trig(request.param)
    yield request.param
    oracle_lib.set_trig(True)


def test_hello_world(oracle_lib, trig):
    """box2d-rs tests/test.rs:26-102: the box settles at y = 1.01 +- 0.01 after 60 steps of 6/2."""
    s = scenes.hello_world()
    w = oracle_lib.OracleWorld(gravity=s["gravity"], allow_sleep=True)
    scenes.build_world(w, s)
    for _ in range(60):
        w.step(np.float32(1.0 / 60.0), 6, 2)
    st = w.get_body_states()[1]
    assert abs(st["position"][0]) < 0.01
    assert abs(st["position"][1] - 1.01) < 0.01
    assert abs(st["angle"]) < 0.01


def test_begin_contact(oracle_lib):
    """box2d-rs tests/world_test.rs:51-87: no contact while apart, begin_contact after overlap."""
    w = oracle_lib.OracleWorld(gravity=(0.0, -10.0), allow_sleep=True, record_events=True)
    bd = b2g.body_defs(2)
    bd["type"] = b2g.DYNAMIC
    w.create_bodies(bd)
    w.create_fixtures(np.concatenate([b2g.circle_fixture(0, 5.0), b2g.circle_fixture(1, 5.0)]))
    w.set_transform(0, (0.0, 0.0), 0.0)
    w.set_transform(1, (100.0, 0.0), 0.0)
    w.step(np.float32(1.0 / 60.0), 6, 2)
    assert w.get_counts()["contacts"] == 0
    assert not any(e["kind"] == 0 for e in w.get_events())
    w.set_transform(1, (1.0, 0.0), 0.0)
    w.step(np.float32(1.0 / 60.0), 6, 2)
    assert w.get_counts()["contacts"] > 0
    assert any(e["kind"] == 0 for e in w.get_events())


def test_polygon_mass_data(oracle_lib):
    """box2d-rs tests/collision_test.rs:30-81: set_as_box_angle and set() agree with the analytic mass."""
    center = np.array([100.0, -50.0], np.float32)
    hx, hy, angle = np.float32(0.5), np.float32(1.5), np.float32(0.25)
    eps = np.finfo(np.float32).eps
    abs_tol = 2.0 * eps
    rel_tol = 2.0 * eps
    p1 = b2g.box_fixture(0, hx, hy, center=center, angle=angle, density=1.0)
    verts = [(center[0] - hx, center[1] - hy), (center[0] + hx, center[1] - hy),
             (center[0] - hx, center[1] + hy), (center[0] + hx, center[1] + hy)]
    p2 = b2g.polygon_fixture(0, verts, density=1.0)
    mass = 4.0 * hx * hy
    inertia = (mass / 3.0) * (hx * hx + hy * hy) + mass * float(np.dot(center, center))
    for fd in (p1, p2):
        md = oracle_lib.polygon_mass(fd)
        assert md["count"] == 4
        for i in range(2):
            assert abs(md["centroid"][i] - center[i]) < abs_tol + rel_tol * abs(center[i])
            assert abs(md["center"][i] - center[i]) < abs_tol + rel_tol * abs(center[i])
        assert abs(md["mass"] - mass) < 20.0 * (abs_tol + rel_tol * mass)
        assert abs(md["I"] - inertia) < 40.0 * (abs_tol + rel_tol * inertia)


def test_project_sincos_is_correctly_rounded(oracle_lib):
    """The project's sin/cos (used by the GPU and by the oracle in parity mode) rounds the exact
    value once: compare with float64 sin/cos rounded to f32 over 2M angles of physics magnitudes."""
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.uniform(-200, 200, 500_000), rng.uniform(-2, 2, 500_000),
                        rng.uniform(-1e-3, 1e-3, 500_000), rng.uniform(-1e4, 1e4, 500_000)]).astype(np.float32)
    oracle_lib.set_trig(False)
    s, c = oracle_lib.sincos(x)
    oracle_lib.set_trig(True)
    xd = x.astype(np.float64)
    assert np.array_equal(s, np.sin(xd).astype(np.float32))
    assert np.array_equal(c, np.cos(xd).astype(np.float32))
    assert s[0] == s[0]


def test_project_sincos_vs_libm(oracle_lib):
    """How often the platform libm sinf/cosf (what Rust's f32::sin calls) differs from the
    correctly rounded value: a 1-ulp difference on a small fraction of inputs, never more."""
    rng = np.random.default_rng(8)
    x = rng.uniform(-50, 50, 200_000).astype(np.float32)
    oracle_lib.set_trig(False)
    s1, c1 = oracle_lib.sincos(x)
    oracle_lib.set_trig(True)
    s2, c2 = oracle_lib.sincos(x)
    ulp = lambda a, b: np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))
    assert ulp(s1, s2).max() <= 1 and ulp(c1, c2).max() <= 1
    assert (s1 != s2).mean() < 0.05


def test_sweep_transform_exact(oracle_lib):
    """box2d-rs tests/math_test.rs:25-49: the rotation of an angle is exactly (cos a, sin a)."""
    for mode in (True, False):
        oracle_lib.set_trig(mode)
        a = np.array([0.5, 5.0], np.float32)
        s, c = oracle_lib.sincos(a)
        if mode:
            assert s[0] == np.float32(math.sin(np.float32(0.5))) or abs(s[0] - math.sin(0.5)) < 1e-7
        assert np.all(s * s + c * c > 0.9999)
    oracle_lib.set_trig(True)


def test_pyramid_stands(oracle_lib):
    """The 20-row, 210-box pyramid is still standing after 600 steps of 8/3 (its top box stays
    near the stacked height of 19.75 m)."""
    s = scenes.pyramid()
    w = oracle_lib.OracleWorld(gravity=s["gravity"])
    scenes.build_world(w, s)
    w.steps(s["dt"], 8, 3, 600)
    st = w.get_body_states()
    top = st["position"][1:, 1].max()
    assert 19.6 < top < 19.9
    assert np.abs(st["linear_velocity"][1:]).max() < 0.05


def test_pair_rule_unique(oracle_lib):
    """update_pairs emits each overlapping pair with a moved proxy once per pass (no duplicates
    without repeated moves), the property the GPU broadphase relies on."""
    s = scenes.mixed(n_circles=300, n_polygons=300, size=30.0, seed=11)
    w = oracle_lib.OracleWorld(gravity=s["gravity"])
    scenes.build_world(w, s)
    for _ in range(5):
        w.step(s["dt"], 8, 3)
        p = w.get_pairs()
        assert len(np.unique(p, axis=0)) == len(p)


def test_golden_oracle(oracle_lib):
    """The oracle reproduces the committed golden outputs bit for bit (made on x86-64 by
    tests/golden/make_golden.py); on the Arm GPU host this pins the oracle's f32 discipline
    (no fused multiply-add) across machines."""
    import sys

    sys.path.insert(0, GOLDEN)
    import make_golden

    g = np.load(os.path.join(GOLDEN, "golden_oracle.npz"))
    fresh = make_golden.compute()
    assert set(g.files) == set(fresh)
    for k in g.files:
        assert np.array_equal(g[k], fresh[k]), k


def test_state_import_continues_exactly(oracle_lib):
    """A world rebuilt from a post-step snapshot (bodies, fat AABBs, contacts with manifolds and
    impulses) continues bit for bit when solved in the same island order."""
    s = scenes.mixed(n_circles=250, n_polygons=250, size=22.0, seed=4)
    a = oracle_lib.OracleWorld(gravity=s["gravity"])
    scenes.build_world(a, s)
    a.steps(s["dt"], 8, 3, 40)
    b = oracle_lib.OracleWorld(gravity=s["gravity"])
    scenes.build_world(b, s)
    aabbs, _, _ = a.get_proxies()
    b.import_state(a.get_body_states(), aabbs, a.get_contacts(), np.float32(1.0) / s["dt"])
    for _ in range(5):
        a.step(s["dt"], 8, 3)
        b.set_solver_order(a.get_solver_order())
        b.step(s["dt"], 8, 3)
        assert b.hook_misses() == 0
        sa, sb = a.get_body_states(), b.get_body_states()
        for f in ("position", "angle", "linear_velocity", "angular_velocity"):
            assert np.array_equal(sa[f], sb[f]), f


def test_scene_sizes():
    s = scenes.pyramid()
    assert s["n_dynamic"] == 210
    m = scenes.mixed(n_circles=1000, n_polygons=1000, size=100.0)
    assert m["n_dynamic"] == 2000
    assert (m["fixtures"]["shape_type"] == b2g.CIRCLE).sum() == 1000
    nv = m["fixtures"]["vertex_count"][m["fixtures"]["shape_type"] == b2g.POLYGON]
    assert nv.min() >= 3 and nv.max() <= 8
    b = scenes.batched(num_worlds=64)
    counts = b["world_body_counts"]
    assert counts.min() >= 16 and counts.max() <= 2048
    assert b["n_dynamic"] == int(counts.sum())
