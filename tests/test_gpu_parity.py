"""GPU path vs the oracle (CPU restatement of box2d-rs) through the C ABI.

Bar: broadphase pair sets equal (bit-exact fat AABBs), manifold feature ids exact and
points/normals/impulses within 1e-5, bodies within 1e-5 per step with the oracle solved
in the GPU's constraint-colour order. With identical IEEE f32 operations the GPU is
expected to be bit-exact, and most checks assert exactly that.
"""
import os

import numpy as np
import pytest

import b2g
import oracle
import parity
import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-5
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _assert_step(r, bitexact=True):
    assert r["hook_misses"] == 0, r
    assert r["pairs_equal"], r
    assert r["fat_aabb_equal"], r
    assert r["contact_key_mismatch"] == 0, r
    assert r["contact_id_mismatch"] == 0, r
    assert r["manifold_max_diff"] <= TOL, r
    assert r["body_rel"] <= TOL, r
    if bitexact:
        assert r["bitexact_bodies"], r
        assert r["awake_equal"], r


def test_narrowphase_golden(built):
    """All five manifold routines on 3000 posed shape pairs: ids exact, geometry bit-exact."""
    g = np.load(os.path.join(GOLDEN, "golden_oracle.npz"))
    da = g["narrow_def_a"].view(b2g.FIXTURE_DEF)
    db = g["narrow_def_b"].view(b2g.FIXTURE_DEF)
    ref = g["narrow_out"].view(b2g.CONTACT_INFO)
    out = b2g.collide_pairs(da, g["narrow_xf_a"], db, g["narrow_xf_b"])
    assert np.array_equal(out["point_count"], ref["point_count"])
    t = ref["point_count"] > 0
    assert np.array_equal(out["manifold_type"][t], ref["manifold_type"][t])
    for i in np.nonzero(t)[0]:
        n = ref["point_count"][i]
        assert list(out["point_id"][i][:n]) == list(ref["point_id"][i][:n]), i
        for f in ("local_normal", "local_point"):
            assert np.array_equal(out[f][i], ref[f][i]), (i, f)
        assert np.array_equal(out["point_local"][i][:n], ref["point_local"][i][:n]), i


def test_narrowphase_vs_live_oracle(built):
    """Same check against the oracle evaluated in this process (random poses, new seed)."""
    import sys

    sys.path.insert(0, GOLDEN)
    import make_golden

    oracle.set_trig(False)
    try:
        da, xa, db, xb = make_golden.random_shape_pairs(n=2000, seed=77)
        ref = make_golden.run_narrow(da, xa, db, xb)
    finally:
        oracle.set_trig(True)
    out = b2g.collide_pairs(da, xa, db, xb)
    assert np.array_equal(out["point_count"], ref["point_count"])
    t = ref["point_count"] > 0
    assert np.array_equal(out["point_id"][t], ref["point_id"][t]) or all(
        list(out["point_id"][i][: ref["point_count"][i]]) == list(ref["point_id"][i][: ref["point_count"][i]])
        for i in np.nonzero(t)[0])
    assert np.array_equal(out["local_normal"][t], ref["local_normal"][t])


def test_pyramid_lockstep(built):
    """20-row pyramid, 120 steps of 8/3: bit-exact bodies, equal pair sets, every step."""
    s = scenes.pyramid()
    recs, gpu, _ = parity.lockstep(s, 120)
    for r in recs:
        _assert_step(r)
    assert recs[-1]["constraints"] > 200


def test_first_step_matches_golden(built):
    """The committed oracle trajectories are solved in the reference's own island order, so a
    GPU trajectory matches them only while no island holds two or more constraints; the first
    step of the 8-row pyramid (no contacts yet: bodies free-fall) must match bit for bit."""
    s = scenes.pyramid(rows=8, steps=1)
    w = b2g.B2world(gravity=s["gravity"])
    w.set_allow_sleeping(False)
    scenes.build_world(w, s)
    ora = oracle.OracleWorld(gravity=s["gravity"])
    oracle.set_trig(False)
    try:
        scenes.build_world(ora, s)
        for _ in range(2):
            w.step(s["dt"], s["vi"], s["pi"])
            ora.step(s["dt"], s["vi"], s["pi"])
    finally:
        oracle.set_trig(True)
    got, ref = w.get_body_states(), ora.get_body_states()
    for f in parity.BODY_FIELDS:
        assert np.array_equal(got[f], ref[f]), f


def test_mixed_small_lockstep(built):
    """400 circles and polygons (3-8 vertices) in a 20 m walled box under gravity: 60 steps."""
    s = scenes.mixed(n_circles=200, n_polygons=200, size=20.0, seed=9)
    recs, gpu, ora = parity.lockstep(s, 60)
    for r in recs:
        _assert_step(r)
    assert max(r["constraints"] for r in recs) > 50


def test_mixed_dense_lockstep(built):
    """A denser pile of 3000 mixed bodies in a 40 m box (hundreds of multi-body islands)."""
    s = scenes.mixed(n_circles=1500, n_polygons=1500, size=40.0, seed=13)
    recs, _, _ = parity.lockstep(s, 40)
    for r in recs:
        _assert_step(r)
    assert max(r["constraints"] for r in recs) > 500


def test_many_parts_lockstep(built):
    """40 000 bodies: the part-local solve splits the constraint bodies into one part per SM, and
    constraints between parts run in the grid-wide boundary colours; the oracle solved in the
    exported order must agree bit for bit."""
    s = scenes.mixed(n_circles=20000, n_polygons=20000, size=200.0, seed=21)
    recs, _, _ = parity.lockstep(s, 12)
    for r in recs:
        _assert_step(r)
    assert max(r["constraints"] for r in recs) > 5000


def test_grid_colour_schedule_lockstep(built):
    """With the part-local solve off every constraint is solved in grid-wide colours."""
    s = scenes.mixed(n_circles=1500, n_polygons=1500, size=40.0, seed=13)
    s["part_solve"] = False
    recs, _, _ = parity.lockstep(s, 40)
    for r in recs:
        _assert_step(r)
    assert max(r["constraints"] for r in recs) > 500


def test_batched_worlds_lockstep(built):
    """Several independent worlds in one batch: never any cross-world pair."""
    s = scenes.batched(num_worlds=6, lo=16, hi=200, seed=5)
    recs, gpu, _ = parity.lockstep(s, 30)
    for r in recs:
        _assert_step(r)
    world = s["bodies"]["world_index"]
    fb = s["fixtures"]["body"]
    for a, b in gpu.get_pairs():
        assert world[fb[a]] == world[fb[b]]


def test_pile_boxes_lockstep(built):
    """Small boxes dropped into a walled container settle into a pile (2-point manifolds,
    block solver, warm starting through many steps)."""
    s = scenes.pile(n_boxes=2000, width=12.0, height=40.0, seed=3, spacing=0.6)
    recs, _, _ = parity.lockstep(s, 150, check_pairs=True)
    for r in recs:
        _assert_step(r)


def test_one_sided_edges_and_kinematic(built):
    """One-sided edge chain, a kinematic paddle and circles/polygons dropped on them."""
    bodies = b2g.body_defs(40)
    bodies["allow_sleep"] = 0
    bodies[1]["type"] = b2g.KINEMATIC
    bodies[1]["position"] = (0.0, 3.0)
    bodies[1]["angular_velocity"] = 1.0
    bodies[2:]["type"] = b2g.DYNAMIC
    rng = np.random.default_rng(3)
    bodies[2:]["position"][:, 0] = rng.uniform(-4, 4, 38)
    bodies[2:]["position"][:, 1] = rng.uniform(5, 15, 38)
    fx = [b2g.edge_fixture(0, (-5.0, 0.0), (0.0, -1.0), v0=(-6.0, 1.0), v3=(5.0, 0.0)),
          b2g.edge_fixture(0, (0.0, -1.0), (5.0, 0.0), v0=(-5.0, 0.0), v3=(6.0, 1.0)),
          b2g.box_fixture(1, 2.0, 0.1, density=1.0)]
    for i in range(2, 40):
        if i % 2:
            fx.append(b2g.circle_fixture(i, 0.3, density=1.0, friction=0.5))
        else:
            fx.append(b2g.polygon_fixture(i, [(-0.3, -0.2), (0.3, -0.25), (0.35, 0.2), (0.0, 0.4), (-0.3, 0.2)],
                                          density=1.0, friction=0.5))
    s = {"bodies": bodies, "fixtures": np.concatenate(fx), "gravity": (0.0, -10.0), "dt": np.float32(1 / 60),
         "vi": 8, "pi": 3, "num_worlds": 1, "allow_sleep": False}
    recs, _, _ = parity.lockstep(s, 200)
    for r in recs:
        _assert_step(r)


def test_kinematic_bodies_across_parts_lockstep(built):
    """3000 mixed bodies (several parts of the part-local solve) with six kinematic paddles
    sweeping through them: kinematic bodies are in no part (their velocities are read, never
    written), and the constraints at them follow their dynamic body's part."""
    s = scenes.mixed(n_circles=1500, n_polygons=1500, size=40.0, seed=17)
    nb = len(s["bodies"])
    kin = b2g.body_defs(6)
    kin["type"] = b2g.KINEMATIC
    kin["allow_sleep"] = 0
    kin["position"][:, 0] = np.linspace(6.0, 34.0, 6)
    kin["position"][:, 1] = 5.0
    kin["linear_velocity"][:, 0] = np.array([1.5, -1.5] * 3)
    kin["angular_velocity"] = np.array([0.7, -0.7] * 3)
    fx = np.concatenate([b2g.box_fixture(nb + i, 2.0, 0.15, density=1.0) for i in range(6)])
    s = dict(s, bodies=np.concatenate([s["bodies"], kin]), fixtures=np.concatenate([s["fixtures"], fx]))
    recs, _, _ = parity.lockstep(s, 60)
    for r in recs:
        _assert_step(r)
    assert max(r["constraints"] for r in recs) > 500


def test_compound_bodies_lockstep(built):
    """1500 bodies with two fixtures each (a box and an offset circle): a body's Morton rank is its
    first fixture's, its fixtures may lie far apart in that order, and pairs within a body are
    never made."""
    rng = np.random.default_rng(23)
    n = 1500
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1:]["position"][:, 0] = rng.uniform(2.0, 48.0, n)
    bodies[1:]["position"][:, 1] = rng.uniform(2.0, 60.0, n)
    bodies[1:]["angle"] = rng.uniform(0.0, 6.28, n)
    walls = [b2g.edge_fixture(0, (0.0, 0.0), (50.0, 0.0)), b2g.edge_fixture(0, (0.0, 0.0), (0.0, 80.0)),
             b2g.edge_fixture(0, (50.0, 0.0), (50.0, 80.0))]
    fx = []
    for i in range(n):
        fx.append(b2g.box_fixture(i + 1, 0.3, 0.15, density=1.0, friction=0.5))
        fx.append(b2g.circle_fixture(i + 1, 0.2, center=(0.45, 0.0), density=1.0, friction=0.5))
    s = {"name": "compound", "bodies": bodies, "fixtures": np.concatenate(walls + fx), "gravity": (0.0, -10.0),
         "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 60, "num_worlds": 1, "allow_sleep": False,
         "n_dynamic": n}
    recs, _, _ = parity.lockstep(s, 60)
    for r in recs:
        _assert_step(r)
    assert max(r["constraints"] for r in recs) > 300


def _toi_lockstep(s, steps, schedule=b2g.TOI_SIDE_BY_SIDE):
    recs, gpu, ora = parity.lockstep(dict(s, toi_schedule=schedule), steps)
    for r in recs:
        _assert_step(r)
    events, _, restarts = gpu.get_toi_stats()
    assert events == ora.toi_events()
    return recs, gpu, ora, events


@pytest.mark.parametrize("schedule", [b2g.TOI_ONE_AT_A_TIME, b2g.TOI_RESTART_ON_ADVANCE])
def test_continuous_rain_schedules_lockstep(built, schedule):
    """The same rain, every event alone, and side by side with a restart at the first sweep
    advance (the path a conflict takes): the same bits as the oracle each step."""
    s = scenes.toi_rain(n=64, seed=7, steps=80)
    _, gpu, _, _ = _toi_lockstep(s, 80, schedule)
    if schedule == b2g.TOI_RESTART_ON_ADVANCE:
        assert gpu.get_toi_stats()[2] > 0


def test_continuous_rain_lockstep(built):
    """Continuous physics: fast circles, boxes and polygons (2 bullets) onto thin static plates and
    a kinematic plate. Every step bit-exact with the oracle's solve_toi, the same number of
    time-of-impact events, and no body passes the plate."""
    s = scenes.toi_rain(n=64, seed=7, steps=120)
    _, gpu, _, events = _toi_lockstep(s, 120)
    assert events > 100
    st = gpu.get_body_states()
    dyn = s["bodies"]["type"] == b2g.DYNAMIC
    x, y = st["position"][dyn, 0], st["position"][dyn, 1]
    assert not np.any((np.abs(x) < 19.5) & (y < 0.0))


def test_continuous_equal_times_lockstep(built):
    """A row of identical boxes with identical velocities meets the plate at identical times: the
    event among equal times of impact is the smallest contact key on both sides."""
    n = 12
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[0]["position"] = (0.0, 0.0)
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1:]["position"][:, 0] = np.linspace(-9.0, 9.0, n).astype(np.float32)
    bodies[1:]["position"][:, 1] = 6.0
    bodies[1:]["linear_velocity"] = (0.0, -150.0)
    fx = [b2g.box_fixture(0, 12.0, 0.05, friction=0.5)]
    fx += [b2g.box_fixture(i + 1, 0.3, 0.2, density=1.0, friction=0.5) for i in range(n)]
    s = {"name": "toi_row", "bodies": bodies, "fixtures": np.concatenate(fx), "gravity": (0.0, -10.0),
         "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 40, "num_worlds": 1, "allow_sleep": False,
         "n_dynamic": n, "continuous": True}
    _, gpu, _, events = _toi_lockstep(s, 40)
    assert events >= n
    assert np.all(gpu.get_body_states()["position"][1:, 1] > 0.0)


def test_continuous_batched_worlds_lockstep(built):
    """Four toi_rain worlds in one batch: events of different worlds are solved side by side."""
    s = scenes.toi_rain_batch(seeds=(7, 8, 9, 10), n=32, steps=90)
    _, _, _, events = _toi_lockstep(s, 90)
    assert events > 100


def test_continuous_pyramid_lockstep(built):
    """A settling pyramid with continuous physics on: every box-ground contact gets a time of impact
    each step (slow landings may make events); bit-exact with the oracle's solve_toi."""
    s = dict(scenes.pyramid(rows=8), continuous=True)
    _toi_lockstep(s, 120)


def test_continuous_mixed_side_by_side_lockstep(built):
    """3000 circles and polygons falling in a 60 x 60 m box of one-sided-free edges: many bodies
    cross an edge within a step at once, so most iterations of the pass solve many events side by
    side. Bit-exact with the oracle's one-event-at-a-time solve_toi."""
    s = dict(scenes.mixed(n_circles=1500, n_polygons=1500, size=60.0, seed=29), continuous=True)
    _, gpu, _, events = _toi_lockstep(s, 150)
    assert events > 50


def _sleepy(s):
    s = dict(s, allow_sleep=True)
    b = s["bodies"].copy()
    b["allow_sleep"] = 1
    return dict(s, bodies=b)


def test_sleeping_pyramid_lockstep(built):
    """Sleeping on: a 10-row pyramid settles and falls asleep island by island (sleep timers,
    the per-island position-solved test, set_awake(false) zeroing velocities); bodies and awake
    flags bit-exact with the oracle every step."""
    s = _sleepy(scenes.pyramid(rows=10))
    recs, gpu, _ = parity.lockstep(s, 300)
    for r in recs:
        _assert_step(r)
    assert recs[-1]["awake"] == 0


def _woken_pile():
    """40 boxes that fall asleep in a pile, and a heavy box dropped from 145 m onto them."""
    s = scenes.pile(n_boxes=40, width=4.0, height=4.0, seed=11, spacing=0.45)
    nb = len(s["bodies"])
    drop = b2g.body_defs(1)
    drop["type"] = b2g.DYNAMIC
    drop["position"] = (0.3, 145.0)
    fx = b2g.box_fixture(nb, 0.6, 0.6, density=20.0, friction=0.6)
    return _sleepy(dict(s, bodies=np.concatenate([s["bodies"], drop]), fixtures=np.concatenate([s["fixtures"], fx]),
                        n_dynamic=s["n_dynamic"] + 1))


def test_sleeping_pile_woken_lockstep(built):
    """A pile of 40 boxes falls asleep, then a heavy box dropped from 145 m lands on it: the
    sleeping pile's contacts become active as the wake spreads, in the reference's order within
    each collide pass (its list order, here the key order on both sides)."""
    recs, gpu, _ = parity.lockstep(_woken_pile(), 440)
    for r in recs:
        _assert_step(r)
    awake = [r["awake"] for r in recs]
    assert min(awake[230:320]) <= 1      # the pile slept before the box arrived
    assert max(awake[340:]) > 30         # and woke up


def _collide_group(group):
    """a lockstep before_step hook that sets the GPU world's narrowphase pairs per warp batch"""
    def hook(k, gpu, ora):
        if k == 0:
            gpu.set_launch_config(collide_group=group)
    return hook


@pytest.mark.parametrize("group", [8, 32])
def test_segment_narrowphase_lockstep(built, group):
    """Polygon pairs evaluated eight lanes to a pair (collide_polygons_group) in every warp batch
    holding at most `group` of them: a settling box pile (nearly every contact a polygon pair) and a
    dense mixed pile, bit-exact with the oracle every step."""
    for s, steps in ((scenes.pile(n_boxes=2000, width=12.0, height=40.0, seed=3, spacing=0.6), 100),
                     (scenes.mixed(n_circles=1500, n_polygons=1500, size=40.0, seed=13), 40)):
        recs, gpu, _ = parity.lockstep(s, steps, before_step=_collide_group(group))
        assert gpu.get_launch_config()["collide_group"] == group
        for r in recs:
            _assert_step(r)
        assert max(r["constraints"] for r in recs) > 200


def test_segment_narrowphase_wake_cascade_lockstep(built):
    """The wake cascade of a sleeping world (contacts collided in rounds as a wake spreads along the
    table) with every polygon pair evaluated eight lanes to a pair."""
    recs, gpu, _ = parity.lockstep(_woken_pile(), 440, before_step=_collide_group(32))
    for r in recs:
        _assert_step(r)
    awake = [r["awake"] for r in recs]
    assert min(awake[230:320]) <= 1
    assert max(awake[340:]) > 30


def test_revolute_bridge_lockstep(built):
    """Revolute joints: a 30-plank bridge between static posts with bodies dropped on it, a
    motorised bar and a hinged flap with limits and a weak motor. Joints solve before the contacts
    in each velocity iteration and after them in each position iteration, in the joint colouring's
    order on both sides; bodies, manifolds and joint impulses bit-exact every step. Joined planks
    never collide (collide_connected off)."""
    s = scenes.bridge()
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    planks = set(range(1, 31))
    fb = s["fixtures"]["body"]
    for c in gpu.get_contacts():
        a, b = int(fb[c["fixture_a"]]), int(fb[c["fixture_b"]])
        assert not (a in planks and b in planks and abs(a - b) == 1)
    st = gpu.get_body_states()
    assert abs(float(st["angular_velocity"][1 + 30 + 24]) - 2.0) < 1e-3  # the motor holds its speed


def test_revolute_chain_sleeps_lockstep(built):
    """Sleeping on: a hanging chain of 8 links (revolute joints, the first to a static hook) is
    set swinging, comes to rest and falls asleep as one island (the joints keep it together)."""
    n = 8
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 1
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1:]["position"][:, 1] = 19.5 - np.arange(n, dtype=np.float32)
    bodies[1:]["angle"] = np.float32(-np.pi / 2)
    bodies[1:]["angular_damping"] = 4.0
    bodies[1:]["linear_damping"] = 4.0
    bodies[n]["linear_velocity"] = (3.0, 0.0)
    fx = [b2g.edge_fixture(0, (-30.0, 0.0), (30.0, 0.0))]
    fx += [b2g.box_fixture(i + 1, 0.5, 0.1, density=1.0, friction=0.2) for i in range(n)]
    joints = [b2g.revolute_joint(0, 1, (0.0, 20.0), (-0.5, 0.0))]
    joints += [b2g.revolute_joint(i, i + 1, (0.5, 0.0), (-0.5, 0.0)) for i in range(1, n)]
    s = {"name": "chain", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 480, "num_worlds": 1,
         "allow_sleep": True, "n_dynamic": n}
    recs, _, _ = parity.lockstep(s, 480)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    assert recs[-1]["awake"] == 0


def test_joint_created_mid_run_filters_contacts(built):
    """Two overlapping boxes collide; a revolute joint between them (collide_connected off) made
    after 20 steps flags their contact, which the next collide destroys (B2world::create_joint's
    filtering), on the GPU as in the oracle."""
    bodies = b2g.body_defs(3)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1]["position"] = (0.0, 1.0)
    bodies[2]["position"] = (0.8, 2.1)
    fx = np.concatenate([b2g.edge_fixture(0, (-10.0, 0.0), (10.0, 0.0)),
                         b2g.box_fixture(1, 0.5, 0.5, density=1.0, friction=0.5),
                         b2g.box_fixture(2, 0.5, 0.5, density=1.0, friction=0.5)])
    s = {"name": "mid_joint", "bodies": bodies, "fixtures": fx, "gravity": (0.0, -10.0), "dt": np.float32(1 / 60),
         "vi": 8, "pi": 3, "steps": 60, "num_worlds": 1, "allow_sleep": False, "n_dynamic": 2}
    gpu, ora = parity.make_pair(s, record_pairs=False)
    dt, vi, pi = s["dt"], s["vi"], s["pi"]

    def step_both(k):
        for _ in range(k):
            gpu.step(dt, vi, pi)
            ora.set_solver_order(gpu.get_solver_order())
            ora.step(dt, vi, pi)
            for f in parity.BODY_FIELDS:
                assert np.array_equal(gpu.get_body_states()[f], ora.get_body_states()[f]), f
            km, im, _ = parity.manifold_diff(gpu.get_contacts(), ora.get_contacts())
            assert not km and im == 0

    step_both(20)
    pair = (1, 2)
    assert any(tuple(sorted((int(c["fixture_a"]), int(c["fixture_b"])))) == pair for c in gpu.get_contacts())
    j = b2g.revolute_joint(1, 2, (0.4, 0.5), (-0.4, -0.6))
    gpu.create_joints(j)
    ora.create_joints(j)
    ora.set_joint_order(gpu.get_joint_order())
    step_both(40)
    assert not any(tuple(sorted((int(c["fixture_a"]), int(c["fixture_b"])))) == pair for c in gpu.get_contacts())
    assert np.array_equal(gpu.get_joint_impulses(), ora.get_joint_impulses())


def test_distance_joints_lockstep(built):
    """Distance joints: a rigid pendulum, a damped spring with min and max length, a rope (max
    length only), and a chain of boxes hung on rigid distance joints with bodies dropped on it;
    bodies, manifolds and joint impulses bit-exact every step."""
    n_chain, n_drop = 10, 12
    nb = 1 + 3 + n_chain + n_drop
    bodies = b2g.body_defs(nb)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1]["position"] = (-10.0, 7.0)
    bodies[2]["position"] = (-6.0, 9.0)
    bodies[3]["position"] = (-2.0, 12.0)
    bodies[3]["linear_velocity"] = (4.0, 0.0)
    fx = [b2g.edge_fixture(0, (-30.0, 0.0), (30.0, 0.0)),
          b2g.box_fixture(1, 0.3, 0.3, density=2.0), b2g.circle_fixture(2, 0.4, density=2.0),
          b2g.box_fixture(3, 0.4, 0.2, density=2.0)]
    joints = [b2g.distance_joint(0, 1, (-10.0, 10.0), (0.0, 0.3), 3.0),
              b2g.distance_joint(0, 2, (-6.0, 12.0), (0.0, 0.0), 3.0, min_length=1.0, max_length=5.0,
                                 stiffness=20.0, damping=0.5),
              b2g.distance_joint(0, 3, (-2.0, 14.0), (-0.4, 0.0), 4.0, min_length=0.0, max_length=4.0)]
    first = 4
    for i in range(n_chain):
        b = first + i
        bodies[b]["position"] = (2.0 + 1.0 * i, 8.0)
        fx.append(b2g.box_fixture(b, 0.4, 0.1, density=5.0, friction=0.3))
        if i == 0:
            joints.append(b2g.distance_joint(0, b, (1.0, 8.0), (-0.4, 0.0), 0.6))
        else:
            joints.append(b2g.distance_joint(b - 1, b, (0.4, 0.0), (-0.4, 0.0), 0.2))
    joints.append(b2g.distance_joint(first + n_chain - 1, 0, (0.4, 0.0), (12.0, 8.0), 0.6))
    rng = np.random.default_rng(31)
    for k in range(n_drop):
        b = first + n_chain + k
        bodies[b]["position"] = (rng.uniform(2.5, 11.0), rng.uniform(10.0, 16.0))
        fx.append(b2g.circle_fixture(b, 0.25, density=1.0, friction=0.4) if k % 2 else
                  b2g.box_fixture(b, 0.25, 0.2, density=1.0, friction=0.4))
    s = {"name": "distance", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 200, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": nb - 1}
    recs, gpu, _ = parity.lockstep(s, 200)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert abs(float(np.linalg.norm(st["position"][1] + np.array([10.0, -10.0]) - [0.0, 0.0]) ) - 3.0) < 0.35


def test_weld_joints_lockstep(built):
    """Weld joints: a rigid cantilever of 8 welded boxes from a static wall, and a soft-welded
    beam (angular spring, stiffness 30, damping 1) on a revolute hinge, with bodies dropped on both;
    bodies, manifolds and joint impulses bit-exact every step."""
    n, n_drop = 8, 10
    nb = 1 + 2 * n + n_drop
    bodies = b2g.body_defs(nb)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    fx = [b2g.edge_fixture(0, (-30.0, 0.0), (30.0, 0.0))]
    joints = []
    for i in range(n):
        a, b = 1 + i, 1 + n + i
        bodies[a]["position"] = (-12.0 + 1.0 * i, 8.0)
        bodies[b]["position"] = (3.0 + 1.0 * i, 8.0)
        fx.append(b2g.box_fixture(a, 0.5, 0.125, density=5.0, friction=0.4))
        fx.append(b2g.box_fixture(b, 0.5, 0.125, density=5.0, friction=0.4))
        if i == 0:
            joints.append(b2g.weld_joint(0, a, (-12.5, 8.0), (-0.5, 0.0)))
            joints.append(b2g.revolute_joint(0, b, (2.5, 8.0), (-0.5, 0.0)))
        else:
            joints.append(b2g.weld_joint(a - 1, a, (0.5, 0.0), (-0.5, 0.0)))
            joints.append(b2g.weld_joint(b - 1, b, (0.5, 0.0), (-0.5, 0.0), stiffness=30.0, damping=1.0))
    rng = np.random.default_rng(37)
    for k in range(n_drop):
        b = 1 + 2 * n + k
        bodies[b]["position"] = (rng.uniform(-12.0, 10.0), rng.uniform(10.0, 16.0))
        fx.append(b2g.circle_fixture(b, 0.3, density=1.0, friction=0.4) if k % 2 else
                  b2g.box_fixture(b, 0.3, 0.2, density=1.0, friction=0.4))
    s = {"name": "weld", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 200, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": nb - 1}
    recs, gpu, _ = parity.lockstep(s, 200)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert float(st["position"][n, 1]) > 4.5  # the rigid cantilever holds up (welds sag a little)


def test_friction_joints_lockstep(built):
    """Friction joints (top-down friction): boxes and circles sliding and spinning over a static
    body with no gravity are slowed by friction joints to it, one pair drags each other through a
    friction joint, and they collide with each other and the walls; bit-exact every step."""
    n = 16
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    rng = np.random.default_rng(41)
    bodies[1:]["position"][:, 0] = rng.uniform(-8.0, 8.0, n)
    bodies[1:]["position"][:, 1] = rng.uniform(-8.0, 8.0, n)
    bodies[1:]["linear_velocity"][:, 0] = rng.uniform(-6.0, 6.0, n)
    bodies[1:]["linear_velocity"][:, 1] = rng.uniform(-6.0, 6.0, n)
    bodies[1:]["angular_velocity"] = rng.uniform(-4.0, 4.0, n)
    corners = [(-10.0, -10.0), (10.0, -10.0), (10.0, 10.0), (-10.0, 10.0)]
    fx = [b2g.edge_fixture(0, corners[i], corners[(i + 1) % 4]) for i in range(4)]
    joints = []
    for i in range(n):
        b = i + 1
        fx.append(b2g.box_fixture(b, 0.5, 0.3, density=1.0, friction=0.3) if i % 2 else
                  b2g.circle_fixture(b, 0.4, density=1.0, friction=0.3))
        if i < n - 2:
            joints.append(b2g.friction_joint(0, b, (0.0, 0.0), (0.0, 0.0), max_force=2.0, max_torque=0.5,
                                             collide_connected=True))
    joints.append(b2g.friction_joint(n - 1, n, (0.0, 0.0), (0.0, 0.0), max_force=4.0, max_torque=1.0))
    s = {"name": "friction", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, 0.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 240, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": n}
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    v = gpu.get_body_states()["linear_velocity"][1:n - 1]
    assert float(np.abs(v).max()) < 1.0  # friction stopped them


@pytest.mark.gpu
def test_motor_joints_lockstep(built):
    """Motor joints: boxes hanging under gravity are driven by motor joints to offsets from a static
    body and to angles, two dynamic bodies are held apart by a motor joint between them, and the
    driven boxes collide with each other on the way; bit-exact every step."""
    n = 12
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    rng = np.random.default_rng(43)
    bodies[1:]["position"][:, 0] = rng.uniform(-6.0, 6.0, n)
    bodies[1:]["position"][:, 1] = rng.uniform(1.0, 8.0, n)
    bodies[1:]["angle"] = rng.uniform(-1.0, 1.0, n)
    fx = [b2g.edge_fixture(0, (-20.0, 0.0), (20.0, 0.0))]
    joints = []
    for i in range(n):
        b = i + 1
        fx.append(b2g.box_fixture(b, 0.5, 0.3, center=(0.1, 0.0), density=1.0, friction=0.3) if i % 2 else
                  b2g.circle_fixture(b, 0.4, density=1.0, friction=0.3))
        if i < n - 2:
            joints.append(b2g.motor_joint(0, b, linear_offset=(-5.0 + i, 4.0), angular_offset=0.25 * i,
                                          max_force=float(60 + 10 * i), max_torque=float(5 + i),
                                          correction_factor=0.2 + 0.05 * i))
    joints.append(b2g.motor_joint(n - 1, n, linear_offset=(1.5, 0.5), angular_offset=0.5, max_force=40.0,
                                  max_torque=10.0, collide_connected=True))
    s = {"name": "motor", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 240, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": n}
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert abs(float(st["position"][1, 0]) + 5.0) < 0.2 and abs(float(st["position"][1, 1]) - 4.0) < 0.2


@pytest.mark.gpu
def test_mouse_joints_lockstep(built):
    """Mouse joints: boxes resting on the ground, some held by soft mouse joints at a point of their
    own; the free ones fall asleep, then new targets drag jointed boxes up and sideways (each new
    target wakes its body) and back down onto the others; bit-exact bodies, impulses and awake flags
    every step."""
    n = 8
    bodies = b2g.body_defs(n + 1)
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1:]["position"][:, 0] = np.arange(n) * 2.0 - 7.0
    bodies[1:]["position"][:, 1] = 0.5
    fx = [b2g.edge_fixture(0, (-20.0, 0.0), (20.0, 0.0))]
    fx += [b2g.box_fixture(i + 1, 0.5, 0.5, density=1.0, friction=0.6) for i in range(n)]
    held = [1, 3, 4, 6]
    joints = [b2g.mouse_joint(0, b, (float(bodies[b]["position"][0]) + 0.2, 0.8), max_force=400.0,
                              stiffness=150.0, damping=12.0 + b) for b in held]
    moves = {90: [(0, (-5.5, 3.0)), (2, (-2.0, 4.0))], 150: [(1, (-1.0, 2.5)), (0, (-4.0, 1.2))],
             200: [(3, (4.0, 5.0)), (2, (-2.5, 1.0))]}

    def before_step(k, gpu, ora):
        for j, t in moves.get(k, []):
            gpu.set_mouse_target(j, t)
            ora.set_mouse_target(j, t)

    s = {"name": "mouse", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 260, "num_worlds": 1,
         "allow_sleep": True, "n_dynamic": n}
    recs, gpu, _ = parity.lockstep(s, 260, before_step=before_step)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    assert min(r["awake"] for r in recs[60:90]) < n  # free boxes slept before the drags
    st = gpu.get_body_states()
    assert st["position"][held[3], 1] > 3.5  # dragged up to its last target


@pytest.mark.gpu
def test_prismatic_joints_lockstep(built):
    """Prismatic joints: boxes on slides at several angles to a static body (limits, motors, a
    locked slide with equal limits, a free slide), a dynamic pair on a motorised slide, and the
    sliders collide with one another and a falling box; bit-exact every step."""
    n = 10
    bodies = b2g.body_defs(n + 1)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    bodies[1:]["position"][:, 0] = np.arange(n) * 1.3 - 6.0
    bodies[1:]["position"][:, 1] = 3.0 + 0.4 * (np.arange(n) % 3)
    bodies[1:]["angle"] = 0.1 * np.arange(n)
    bodies[n]["position"] = (0.2, 8.0)
    fx = [b2g.edge_fixture(0, (-20.0, 0.0), (20.0, 0.0))]
    fx += [b2g.box_fixture(i + 1, 0.5, 0.25, density=1.0, friction=0.4) for i in range(n)]
    joints = []
    for i in range(n - 3):
        b = i + 1
        ang = -0.6 + 0.2 * i
        p = bodies[b]["position"]
        limits = [(-1.0, 1.5), None, (0.0, 0.0), (-0.5, 2.0), (-2.0, 0.3), None, (-1.0, 1.0)][i]
        motor = [None, (1.0, 30.0), None, (-2.0, 50.0), (3.0, 5.0), None, (0.5, 100.0)][i]
        joints.append(b2g.prismatic_joint(0, b, (float(p[0]), float(p[1])), (0.0, 0.0), (np.cos(ang), np.sin(ang)),
                                          reference_angle=float(bodies[b]["angle"]), limits=limits, motor=motor))
    joints.append(b2g.prismatic_joint(n - 2, n - 1, (0.6, 0.0), (-0.6, 0.0), (1.0, 0.5), reference_angle=-0.1,
                                      limits=(-0.5, 0.8), motor=(-1.5, 20.0)))
    s = {"name": "prismatic", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 240, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": n}
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert np.all(np.isfinite(st["position"]))
    locked = st["position"][3] - bodies[3]["position"]
    assert float(np.abs(locked).max()) < 0.05  # equal limits hold the slide in place


@pytest.mark.gpu
def test_wheel_joints_lockstep(built):
    """Wheel joints: two cars (a chassis on two sprung wheels, rear wheel motorised, one car with
    suspension limits and an axis not of unit length) drive over bumps and into each other; bit-exact
    bodies and joint impulses every step."""
    bodies = b2g.body_defs(7)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    pos = [(-6.0, 1.2), (-7.0, 0.6), (-5.0, 0.6), (6.0, 1.3), (5.0, 0.65), (7.0, 0.65)]
    for i, p in enumerate(pos):
        bodies[i + 1]["position"] = p
    fx = [b2g.edge_fixture(0, (-20.0, 0.0), (-2.0, 0.0)), b2g.edge_fixture(0, (-2.0, 0.0), (-1.0, 0.3)),
          b2g.edge_fixture(0, (-1.0, 0.3), (1.0, 0.0)), b2g.edge_fixture(0, (1.0, 0.0), (20.0, 0.0))]
    for c in (1, 4):
        fx.append(b2g.box_fixture(c, 1.5, 0.25, density=1.0, friction=0.4))
        fx.append(b2g.circle_fixture(c + 1, 0.4, density=1.0, friction=0.9))
        fx.append(b2g.circle_fixture(c + 2, 0.4, density=1.0, friction=0.9))
    joints = [
        b2g.wheel_joint(1, 2, (-1.0, -0.6), (0.0, 0.0), (0.0, 1.0), stiffness=40.0, damping=2.0, motor=(-12.0, 40.0)),
        b2g.wheel_joint(1, 3, (1.0, -0.6), (0.0, 0.0), (0.0, 1.0), stiffness=40.0, damping=2.0),
        b2g.wheel_joint(4, 5, (-1.0, -0.65), (0.0, 0.0), (0.3, 1.2), stiffness=25.0, damping=1.0,
                        limits=(-0.15, 0.1)),
        b2g.wheel_joint(4, 6, (1.0, -0.65), (0.0, 0.0), (0.0, 1.0), stiffness=25.0, damping=1.0, limits=(-0.15, 0.1),
                        motor=(10.0, 30.0)),
    ]
    s = {"name": "wheel", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 240, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": 6}
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert np.all(np.isfinite(st["position"]))
    assert float(st["position"][1, 0]) > -6.0  # the motorised car moved forward


@pytest.mark.gpu
def test_pulley_joints_lockstep(built):
    """Pulley joints: two unequal loads on a 1:1 pulley, a block-and-tackle with ratio 2, and a load
    dropped onto one side; bit-exact bodies and joint impulses every step."""
    bodies = b2g.body_defs(6)
    bodies["allow_sleep"] = 0
    bodies[1:]["type"] = b2g.DYNAMIC
    pos = [(-3.0, 4.0), (3.0, 5.0), (-8.0, 3.0), (-5.0, 5.0), (3.1, 9.0)]
    for i, p in enumerate(pos):
        bodies[i + 1]["position"] = p
    fx = [b2g.edge_fixture(0, (-20.0, 0.0), (20.0, 0.0))]
    fx += [b2g.box_fixture(1, 0.5, 0.5, density=1.0), b2g.box_fixture(2, 0.5, 0.5, density=1.5),
           b2g.circle_fixture(3, 0.4, density=1.0), b2g.box_fixture(4, 0.3, 0.6, density=1.0),
           b2g.box_fixture(5, 0.4, 0.4, density=2.0)]
    joints = [
        b2g.pulley_joint(1, 2, (-3.0, 10.0), (3.0, 10.0), (0.0, 0.5), (0.2, 0.5), 5.5, 4.5, ratio=1.0),
        b2g.pulley_joint(3, 4, (-8.0, 9.0), (-5.0, 9.0), (0.0, 0.0), (0.0, 0.6), 6.0, 3.4, ratio=2.0),
    ]
    s = {"name": "pulley", "bodies": bodies, "fixtures": np.concatenate(fx), "joints": np.concatenate(joints),
         "gravity": (0.0, -10.0), "dt": np.float32(1.0 / 60.0), "vi": 8, "pi": 3, "steps": 240, "num_worlds": 1,
         "allow_sleep": False, "n_dynamic": 5}
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert np.all(np.isfinite(st["position"]))
    assert float(st["position"][2, 1]) < 5.0  # the heavier side went down


def test_gear_joints_lockstep(built):
    """Gear joints (B2gearJoint): a disc geared to the box it hangs from (the box is both bodies A and D
    of that gear), two discs geared 2:1 on ground hinges, and the larger disc geared to a box on a
    limited vertical slider (a revolute-prismatic gear); bodies and joint impulses bit-exact every step,
    and the gear constraints hold: a4 + 2 a5 and a5 - 0.5 (y6 - 12) stay at their initial values."""
    s = scenes.gears(steps=240)
    recs, gpu, _ = parity.lockstep(s, 240)
    for r in recs:
        _assert_step(r)
        assert r["joint_impulses_equal"], r
    st = gpu.get_body_states()
    assert abs(st["angle"][4] + 2.0 * st["angle"][5]) < 1e-3
    assert abs(st["angle"][5] - 0.5 * (st["position"][6, 1] - 12.0)) < 1e-3
    assert abs(st["angle"][4]) > 1.0, "the geared train should have turned"
    with pytest.raises(b2g.B2GError):  # a gear whose body_a is not its first joint's second body
        gpu.create_joints(b2g.gear_joint(0, 1, 1, 3))
