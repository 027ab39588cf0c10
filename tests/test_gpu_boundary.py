"""The rest of the B2world boundary on the GPU, in lockstep with the oracle: destroying bodies,
fixtures and joints mid-run (with the dynamic tree's proxy-id reuse), creating new bodies into the
freed proxy ids, and changing fixtures' filter data (set_filter_data / refilter).

Every step: bodies bit-exact, awake flags equal, fat AABBs bit-exact, proxy ids equal, the
broadphase's pair set equal, every live contact equal (feature ids exact, geometry and impulses
within 1e-5, observed equal), begin/end events equal as sets, joint impulses bit-exact."""
import numpy as np
import pytest

import b2g
import parity
import scenes

pytestmark = pytest.mark.gpu


def _events(w):
    ev = w.get_events() if hasattr(w, "get_events") else []
    return sorted((int(e["kind"]), int(e["fixture_a"]), int(e["fixture_b"])) for e in ev)


def _compare(gpu, ora, k, joints=False):
    gs, os_ = gpu.get_body_states(), ora.get_body_states()
    for f in parity.BODY_FIELDS:
        assert np.array_equal(gs[f], os_[f]), (k, f)
    assert np.array_equal(gpu.get_awake(), ora.get_awake()), k
    ga, _ = gpu.get_proxies()
    oa, _, oids = ora.get_proxies()
    assert np.array_equal(ga, oa), k
    assert np.array_equal(gpu.get_proxy_ids(), oids), k
    assert parity.pair_set(gpu.get_pairs()) == parity.pair_set(ora.get_pairs()), k
    km, im, worst = parity.manifold_diff_fast(gpu.get_contacts(), ora.get_contacts())
    assert km == 0 and im == 0 and worst <= 1e-5, (k, km, im, worst)
    assert _events(gpu) == _events(ora), k
    if joints:
        gi, oi = gpu.get_joint_impulses(), ora.get_joint_impulses()
        assert np.array_equal(gi, oi), k


def _new_boxes(first_body, n, x0, y0, seed):
    rng = np.random.default_rng(seed)
    bodies = b2g.body_defs(n)
    bodies["type"] = b2g.DYNAMIC
    bodies["allow_sleep"] = 0
    bodies["position"][:, 0] = x0 + np.arange(n) * 1.1
    bodies["position"][:, 1] = y0
    bodies["angle"] = rng.uniform(0, 1, n).astype(np.float32)
    fix = np.concatenate([b2g.box_fixture(first_body + i, 0.4, 0.3, density=1.0, friction=0.5) for i in range(n)])
    return bodies, fix


def _step_both(gpu, ora, s):
    gpu.step(s["dt"], s["vi"], s["pi"])
    ora.set_solver_order(gpu.get_solver_order())
    ora.step(s["dt"], s["vi"], s["pi"])


def test_destroy_recreate_and_refilter_lockstep(built, oracle_lib):
    s = scenes.mixed(n_circles=250, n_polygons=250, size=25.0, seed=11, steps=90)
    gpu, ora = parity.make_pair(s, record_pairs=True, record_events=True)
    body_of = s["fixtures"]["body"]
    live_fix = lambda body: int(np.nonzero(body_of == body)[0][0])  # noqa: E731
    nb = len(s["bodies"])
    for k in range(90):
        if k == 10:  # bodies with their contacts and proxies
            for w in (gpu, ora):
                w.destroy_bodies([5, 17, 33, 120])
        if k == 15:  # fixtures of live bodies: contacts, proxies, mass data
            for w in (gpu, ora):
                w.destroy_fixtures([live_fix(40), live_fix(41)])
        if k == 20:  # new bodies take the freed proxy ids, most recently freed first
            bd, fx = _new_boxes(nb, 6, -10.0, 20.0, 1)
            for w in (gpu, ora):
                w.create_bodies(bd)
                w.create_fixtures(fx)
            nb += 6
            ids = gpu.get_proxy_ids()
            assert len(np.unique(ids[ids >= 0])) == int((ids >= 0).sum())
        if k == 30:  # filter data: these fixtures stop colliding with everything
            for f in (live_fix(60), live_fix(61), live_fix(62)):
                for w in (gpu, ora):
                    w.set_filter_data(f, 0x0002, 0x0000, 0)
        if k == 45:  # and collide again (refilter touches the proxy: the next broadphase finds them)
            for f in (live_fix(60), live_fix(61)):
                for w in (gpu, ora):
                    w.set_filter_data(f, 0x0001, 0xffff, 0)
            for w in (gpu, ora):
                w.set_filter_data(live_fix(62), 0x0001, 0xffff, -3)
        if k == 60:  # a body destroyed after its fixture, and one more recreation round
            for w in (gpu, ora):
                w.destroy_bodies([40])
            bd, fx = _new_boxes(nb, 3, 5.0, 22.0, 2)
            for w in (gpu, ora):
                w.create_bodies(bd)
                w.create_fixtures(fx)
            nb += 3
        _step_both(gpu, ora, s)
        assert ora.hook_misses() == 0, k
        _compare(gpu, ora, k)
    with pytest.raises(b2g.B2GError):
        gpu.destroy_bodies([5])
    with pytest.raises(b2g.B2GError):
        gpu.set_linear_velocity(17, (1.0, 0.0))
    gpu.close()
    ora.close()


def test_destroy_joints_and_plank_lockstep(built, oracle_lib):
    """The bridge: a joint destroyed mid-run (the bridge breaks), then a plank body with its two
    joints; the joints' colouring changes and the oracle takes the GPU's new joint order."""
    s = scenes.bridge(steps=120)
    gpu, ora = parity.make_pair(s, record_pairs=True, record_events=True)
    for k in range(120):
        if k == 30:
            for w in (gpu, ora):
                w.destroy_joints([12])
            ora.set_joint_order(gpu.get_joint_order())
        if k == 70:
            for w in (gpu, ora):
                w.destroy_bodies([20])
            ora.set_joint_order(gpu.get_joint_order())
        _step_both(gpu, ora, s)
        assert ora.hook_misses() == 0, k
        _compare(gpu, ora, k, joints=True)
    gpu.close()
    ora.close()


def test_checkpoint_keeps_destroyed_objects_and_mouse_targets(built):
    """A state saved after destructions and a moved mouse target loads into a world built without
    them, and both continue bit for bit; a target set again after the load to the saved value is
    not skipped as unchanged."""
    s = scenes.bridge(steps=60)
    mouse = b2g.mouse_joint(0, 40, (3.0, 12.0), max_force=500.0, stiffness=5.0, damping=0.7)

    def make():
        w = b2g.B2world(gravity=s["gravity"])
        w.set_allow_sleeping(False)
        scenes.build_world(w, s)
        w.create_joints(mouse)
        return w

    a = make()
    for _ in range(10):
        a.step(s["dt"], s["vi"], s["pi"])
    a.destroy_joints([12])
    a.destroy_bodies([44])
    a.set_mouse_target(len(s["joints"]), (4.0, 13.0))
    for _ in range(5):
        a.step(s["dt"], s["vi"], s["pi"])
    state = a.save_state()
    a.set_mouse_target(len(s["joints"]), (-2.0, 9.0))
    a.load_state(state)
    a.set_mouse_target(len(s["joints"]), (-2.0, 9.0))  # must take effect: the loaded target is (4, 13)
    ref = []
    for _ in range(20):
        a.step(s["dt"], s["vi"], s["pi"])
    ref = a.get_body_states().copy()

    b = make()
    b.load_state(state)
    assert np.array_equal(b.get_proxy_ids(), a.get_proxy_ids())
    b.set_mouse_target(len(s["joints"]), (-2.0, 9.0))
    for _ in range(20):
        b.step(s["dt"], s["vi"], s["pi"])
    got = b.get_body_states()
    for f in b2g.BODY_STATE.names:
        assert np.array_equal(ref[f], got[f]), f
    with pytest.raises(b2g.B2GError):
        b.destroy_bodies([44])


def _post_solve_sorted(w):
    r = w.get_post_solve()
    key = (r["fixture_a"].astype(np.int64) << 32) | r["fixture_b"].astype(np.int64)
    return r[np.argsort(key, kind="stable")]


def test_post_solve_reports_match_oracle(built, oracle_lib):
    """B2island::report: every solved contact's impulses after the velocity iterations and its solved
    point count, the same bits as the oracle's reports, on a pyramid settling onto its ground."""
    s = scenes.pyramid(rows=12, steps=80)
    gpu, ora = parity.make_pair(s, record_pairs=False)
    seen2 = 0
    for k in range(80):
        _step_both(gpu, ora, s)
        g, o = _post_solve_sorted(gpu), _post_solve_sorted(ora)
        assert len(g) == len(o) == len(gpu.get_solver_order()), k
        for f in ("fixture_a", "fixture_b", "count", "normal_impulses", "tangent_impulses"):
            assert np.array_equal(g[f], o[f]), (k, f)
        seen2 += int((g["count"] == 2).sum())
    assert seen2 > 0
    gpu.close()
    ora.close()


def test_contact_filter_and_pre_solve_lockstep(built, oracle_lib):
    """A host contact filter replacing the default one (asked about new pairs and about flagged
    contacts) and a pre_solve listener that disables some contacts and changes the friction and
    restitution of others; both run the same Python functions on the GPU world and on the oracle."""
    s = scenes.mixed(n_circles=200, n_polygons=200, size=22.0, seed=5, steps=80)
    gpu, ora = parity.make_pair(s, record_pairs=True, record_events=True)
    calls = {"gpu": 0, "ora": 0}

    def filt(a, b):
        return (a * 7 + b * 7) % 11 != 0

    def pre_solve(tag):
        def fn(c, old, edit):
            calls[tag] += 1
            key = int(c["fixture_a"]) + int(c["fixture_b"])
            if key % 9 == 0:
                edit.enabled = 0
            elif key % 4 == 0:
                edit.friction = 0.05
                edit.restitution = 0.3
            assert int(c["touching"]) == 1
        return fn

    gpu.set_contact_filter(filt)
    ora.set_contact_filter(filt)
    gpu.set_pre_solve(pre_solve("gpu"))
    ora.set_pre_solve(pre_solve("ora"))
    body_of = s["fixtures"]["body"]
    for k in range(80):
        if k == 40:  # flagged contacts go through the host filter before collide
            f = int(np.nonzero(body_of == 30)[0][0])
            for w in (gpu, ora):
                w.set_filter_data(f, 0x0001, 0xffff, 0)
        _step_both(gpu, ora, s)
        assert ora.hook_misses() == 0, k
        _compare(gpu, ora, k)
        g, o = _post_solve_sorted(gpu), _post_solve_sorted(ora)
        for fld in ("fixture_a", "fixture_b", "count", "normal_impulses", "tangent_impulses"):
            assert np.array_equal(g[fld], o[fld]), (k, fld)
        assert calls["gpu"] == calls["ora"], (k, calls)
    assert calls["gpu"] > 100
    with pytest.raises(b2g.B2GError):
        gpu.set_continuous_physics(True)
    gpu.close()
    ora.close()
