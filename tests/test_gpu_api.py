"""Reference behaviours through the GPU path's B2world-shaped API (the reference's own KATs
re-expressed on the GPU, listener events, flags and error handling)."""
import numpy as np
import pytest

import b2g
import scenes

pytestmark = pytest.mark.gpu


def test_hello_world_gpu(built):
    """box2d-rs tests/test.rs:26-102 on the GPU: y = 1.01 +- 0.01 after 60 steps of 6/2."""
    s = scenes.hello_world()
    w = b2g.B2world(gravity=s["gravity"])
    scenes.build_world(w, s)
    for _ in range(60):
        w.step(np.float32(1.0 / 60.0), 6, 2)
    st = w.get_body_states()[1]
    assert abs(st["position"][0]) < 0.01
    assert abs(st["position"][1] - 1.01) < 0.01
    assert abs(st["angle"]) < 0.01


class Listener:
    def __init__(self):
        self.begin = []
        self.end = []

    def begin_contact(self, fa, fb):
        self.begin.append((fa, fb))

    def end_contact(self, fa, fb):
        self.end.append((fa, fb))


def test_begin_contact_gpu(built):
    """box2d-rs tests/world_test.rs:51-87 on the GPU, with events replayed to a listener."""
    w = b2g.B2world(gravity=(0.0, -10.0))
    lst = Listener()
    w.set_contact_listener(lst)
    bd = b2g.body_defs(2)
    bd["type"] = b2g.DYNAMIC
    w.create_bodies(bd)
    w.create_fixtures(np.concatenate([b2g.circle_fixture(0, 5.0), b2g.circle_fixture(1, 5.0)]))
    w.set_transform(0, (0.0, 0.0), 0.0)
    w.set_transform(1, (100.0, 0.0), 0.0)
    w.step(np.float32(1.0 / 60.0), 6, 2)
    assert w.get_counts()["contacts"] == 0
    assert lst.begin == []
    w.set_transform(1, (1.0, 0.0), 0.0)
    w.step(np.float32(1.0 / 60.0), 6, 2)
    assert w.get_counts()["contacts"] > 0
    assert lst.begin == [(0, 1)]
    w.set_transform(1, (100.0, 0.0), 0.0)
    w.step(np.float32(1.0 / 60.0), 6, 2)
    assert lst.end == [(0, 1)]


def test_empty_and_zero_dt(built):
    w = b2g.B2world()
    w.step(np.float32(1 / 60), 8, 3)  # no bodies: a no-op
    s = scenes.pyramid(rows=3)
    scenes.build_world(w, s)
    before = w.get_body_states()
    w.step(np.float32(0.0), 8, 3)  # dt = 0: collide only, bodies do not move
    after = w.get_body_states()
    assert np.array_equal(before["position"], after["position"])


def test_continuous_physics_refused_while_taping(built):
    """The tape does not record the continuous pass: stepping with both on is refused (-6), and
    the world steps again once continuous physics is off."""
    w = b2g.B2world()
    w.set_allow_sleeping(False)
    scenes.build_world(w, scenes.pyramid(rows=2))
    w.step(np.float32(1 / 60), 8, 3)
    w.tape_begin(4)
    w.set_continuous_physics(True)
    with pytest.raises(b2g.B2GError) as e:
        w.step(np.float32(1 / 60), 8, 3)
    assert e.value.code == -6
    w.set_continuous_physics(False)
    w.step(np.float32(1 / 60), 8, 3)
    w.tape_end()


def test_contact_capacity_overflow_reports(built):
    """A too-small contact table reports B2G_ERR_CAPACITY instead of writing out of bounds."""
    s = scenes.pile(n_boxes=600, width=6.0, height=30.0, seed=1, spacing=0.45)
    w = b2g.B2world(gravity=s["gravity"], contact_capacity=64, pair_capacity=64)
    w.set_allow_sleeping(False)
    scenes.build_world(w, s)
    with pytest.raises(b2g.B2GError) as e:
        for _ in range(200):
            w.step(s["dt"], 8, 3)
        w.synchronize()
    assert e.value.code == -3


def test_forces_and_impulses(built):
    w = b2g.B2world(gravity=(0.0, 0.0))
    bd = b2g.body_defs(1)
    bd["type"] = b2g.DYNAMIC
    w.create_bodies(bd)
    w.create_fixture(b2g.circle_fixture(0, 0.5, density=1.0))
    w.step(np.float32(1 / 60), 8, 3)
    w.apply_linear_impulse(0, (1.0, 0.0), (0.0, 0.0))
    st = w.get_body_states()[0]
    mass = np.float32(np.pi) * 0.25
    assert abs(st["linear_velocity"][0] - 1.0 / mass) < 1e-5
    w.set_linear_velocity(0, (0.0, 2.0))
    w.step(np.float32(0.5), 8, 3)
    assert abs(w.get_body_states()[0]["position"][1] - 1.0) < 1e-5


def test_center_force_torque_and_angular_impulse(built):
    """apply_force_to_center / apply_torque act over one step (v += h/m F, w += h/I T);
    the impulse forms change the velocity at once; set_awake(False) zeroes the motion."""
    h = np.float32(1 / 60)
    for device_first in (False, True):
        w = b2g.B2world(gravity=(0.0, 0.0))
        w.set_allow_sleeping(False)
        bd = b2g.body_defs(1)
        bd["type"] = b2g.DYNAMIC
        w.create_bodies(bd)
        w.create_fixture(b2g.box_fixture(0, 0.5, 0.5, density=2.0))
        if device_first:
            w.step(h, 8, 3)  # the device copy becomes authoritative
            w.set_linear_velocity(0, (0.0, 0.0))
        md = w.get_mass_data()[0]
        inv_m, inv_i = np.float32(md[1]), np.float32(md[3])
        w.apply_force_to_center(0, (3.0, 0.0))
        w.apply_torque(0, 2.0)
        w.step(h, 8, 3)
        st = w.get_body_states()[0]
        assert st["linear_velocity"][0] == np.float32(np.float32(h * inv_m) * np.float32(3.0))
        assert st["angular_velocity"] == np.float32(np.float32(h * inv_i) * np.float32(2.0))
        v0, w0 = st["linear_velocity"].copy(), np.float32(st["angular_velocity"])
        w.apply_linear_impulse_to_center(0, (0.0, 1.0))
        w.apply_angular_impulse(0, 0.5)
        st = w.get_body_states()[0]
        assert st["linear_velocity"][1] == np.float32(v0[1] + inv_m * np.float32(1.0))
        assert st["angular_velocity"] == np.float32(w0 + inv_i * np.float32(0.5))
        w.set_awake(0, False)
        st = w.get_body_states()[0]
        assert np.all(st["linear_velocity"] == 0.0) and st["angular_velocity"] == 0.0
        w.close()


def test_sleeping_bodies_stop(built):
    """With sleep allowed, a resting pyramid falls asleep (velocities zeroed) like the reference."""
    s = scenes.pyramid(rows=4)
    s["bodies"]["allow_sleep"] = 1
    w = b2g.B2world(gravity=s["gravity"])
    w.set_allow_sleeping(True)
    scenes.build_world(w, s)
    for _ in range(400):
        w.step(s["dt"], 8, 3)
    st = w.get_body_states()
    assert np.abs(st["linear_velocity"][1:]).max() == 0.0


def test_async_body_state_readback(built):
    """b2g_get_body_states_async: pipelined read-back (two requests in flight, alternating
    buffers) gives every step's states exactly as the blocking read-back does."""
    s = scenes.mixed(n_circles=300, n_polygons=300, size=30.0, seed=4)
    a, b = b2g.B2world(gravity=s["gravity"]), b2g.B2world(gravity=s["gravity"])
    for w in (a, b):
        w.set_allow_sleeping(False)
        scenes.build_world(w, s)
    ref = []
    for _ in range(12):
        a.step(s["dt"], s["vi"], s["pi"])
        ref.append(a.get_body_states().copy())
    bufs = [np.zeros(b.body_count, b2g.BODY_STATE) for _ in range(12)]
    for k in range(12):
        b.step(s["dt"], s["vi"], s["pi"])
        b.get_body_states_async(bufs[k])
    b.wait_body_states()
    for k in range(12):
        for f in ("position", "angle", "linear_velocity", "angular_velocity", "world_center"):
            assert np.array_equal(bufs[k][f], ref[k][f]), (k, f)
    # a sub-range, and a request before any step (the host still holds the state)
    c = b2g.B2world(gravity=s["gravity"])
    scenes.build_world(c, s)
    part = np.zeros(10, b2g.BODY_STATE)
    c.get_body_states_async(part, first=5)
    c.wait_body_states()
    assert np.array_equal(part["position"], c.get_body_states()[5:15]["position"])
    for w in (a, b, c):
        w.close()


def _continue(w, s, steps):
    for _ in range(steps):
        w.step(s["dt"], s["vi"], s["pi"])
    c = w.get_contacts()
    c = c[np.lexsort((c["fixture_b"], c["fixture_a"]))]
    return w.get_body_states().copy(), c.copy(), w.get_awake().copy()


def test_state_checkpoint_with_joints(built):
    """A bridge of revolute joints resumes bit for bit from a checkpoint, joint impulses included."""
    s = scenes.bridge(steps=60)

    def make():
        w = b2g.B2world(gravity=s["gravity"])
        w.set_allow_sleeping(False)
        scenes.build_world(w, s)
        return w

    a = make()
    _continue(a, s, 25)
    state = a.save_state()
    ref = _continue(a, s, 20) + (a.get_joint_impulses(),)
    b = make()
    b.load_state(state)
    got = _continue(b, s, 20) + (b.get_joint_impulses(),)
    for f in b2g.BODY_STATE.names:
        assert np.array_equal(ref[0][f], got[0][f]), f
    assert np.array_equal(ref[1], got[1]) and np.array_equal(ref[3], got[3])


@pytest.mark.parametrize("continuous,sleep", [(False, False), (True, True)])
def test_state_checkpoint_resumes_bit_for_bit(built, continuous, sleep):
    """b2g_state_save / b2g_state_load: after a checkpoint at step 25, the next 30 steps are the
    same bits whether the world runs on, is loaded back, or a second world built the same way is
    loaded from it (contact table, colouring and partition state included)."""
    s = scenes.mixed(n_circles=600, n_polygons=600, size=30.0, seed=8)

    def make():
        w = b2g.B2world(gravity=s["gravity"])
        w.set_allow_sleeping(sleep)
        w.set_continuous_physics(continuous)
        scenes.build_world(w, s)
        return w

    a = make()
    _continue(a, s, 25)
    state = a.save_state()
    ref = _continue(a, s, 30)
    a.load_state(state)
    again = _continue(a, s, 30)
    b = make()
    b.load_state(state)
    other = _continue(b, s, 30)
    for got in (again, other):
        for f in b2g.BODY_STATE.names:
            assert np.array_equal(ref[0][f], got[0][f]), f
        assert np.array_equal(ref[1], got[1])
        assert np.array_equal(ref[2], got[2])
    with pytest.raises(b2g.B2GError):
        small = b2g.B2world(gravity=s["gravity"])
        scenes.build_world(small, scenes.pyramid(rows=3))
        small.load_state(state)


def test_barrier_timeout_reports_and_world_recovers(built):
    """A grid-barrier wait that runs out returns B2G_ERR_TIMEOUT instead of hanging: the world's
    barriers are made to wait for arrivals that never come (b2g_debug_hold_barriers) under a short
    limit (~0.5 ms); every block leaves its kernel and the host reports the timeout. The world is
    then restored from a checkpoint and its next steps equal those of a world that never failed."""
    s = scenes.mixed(n_circles=1500, n_polygons=1500, size=60.0, seed=3)

    def make():
        w = b2g.B2world(gravity=s["gravity"])
        w.set_allow_sleeping(False)
        scenes.build_world(w, s)
        return w

    a = make()
    _continue(a, s, 10)
    state = a.save_state()
    ref = _continue(a, s, 10)

    b = make()
    b.load_state(state)
    b.set_barrier_limit(1 << 20)
    b.debug_hold_barriers(1)
    b.step(s["dt"], s["vi"], s["pi"])
    with pytest.raises(b2g.B2GError) as err:
        b.synchronize()
    assert err.value.code == b2g.ERR_TIMEOUT
    b.debug_hold_barriers(0)
    b.set_barrier_limit(0)
    b.load_state(state)
    got = _continue(b, s, 10)
    for f in b2g.BODY_STATE.names:
        assert np.array_equal(ref[0][f], got[0][f]), f
    assert np.array_equal(ref[1], got[1])


def test_auto_grow_continues_bit_for_bit(built):
    """Contact and pair capacities far too small for the scene, with automatic growth on: every
    overflow doubles the capacity and repeats the step's broadphase pass, and the world stays bit for
    bit equal to one created with ample capacity (bodies and the whole contact table, every step); a
    checkpoint taken after the growth loads into a world created with the grown capacities."""
    s = scenes.mixed(n_circles=1500, n_polygons=1500, size=40.0, seed=13)

    def make(**kw):
        w = b2g.B2world(gravity=s["gravity"], **kw)
        w.set_allow_sleeping(False)
        scenes.build_world(w, s)
        return w

    small = make(contact_capacity=1500, pair_capacity=300)
    small.set_auto_grow(True)
    big = make()
    for k in range(60):
        small.step(s["dt"], s["vi"], s["pi"])
        big.step(s["dt"], s["vi"], s["pi"])
        a, b = small.get_body_states(), big.get_body_states()
        for f in b2g.BODY_STATE.names:
            assert np.array_equal(a[f], b[f]), (k, f)
        ca, cb = small.get_contacts(), big.get_contacts()
        assert np.array_equal(ca, cb), k
    st = small.get_step_stats()
    assert st["capacity_grows"] >= 2 and st["contact_capacity"] > 1500, st
    # without growth the same small world reports the overflow
    fixed = make(contact_capacity=1500, pair_capacity=300)
    with pytest.raises(b2g.B2GError) as e:
        for _ in range(10):
            fixed.step(s["dt"], s["vi"], s["pi"])
        fixed.synchronize()
    assert e.value.code == b2g.ERR_CAPACITY
