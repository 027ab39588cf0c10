"""ctypes binding of the oracle (liboracle.so) — TEST INFRASTRUCTURE ONLY.

The oracle is a CPU restatement of box2d-rs 0.0.4's `B2world::step` path (see the
header of b2_oracle_world.cpp for the reference lines it follows). Only tests,
`__graft_entry__.smoke()` and bench.py's CPU-baseline / reference legs use it, as
the checker; the product never imports it.

`OracleWorld` has the same method names as `b2g.B2world`, so a parity test can
build one scene into both and step them side by side.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
sys.path.insert(0, os.path.join(os.path.dirname(_HERE), "box2d-rs_gb300"))
import b2g  # noqa: E402  (struct layouts of include/b2g.h)

_lib = None
CONTACT_FILTER_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32)


def build(force=False):
    """Compile liboracle.so with the Makefile beside this file (-ffp-contract=off)."""
    if force and os.path.exists(LIB_PATH):
        os.remove(LIB_PATH)
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ctypes.CDLL(LIB_PATH)
    vp, i32, u32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_float
    pi32 = ctypes.POINTER(ctypes.c_int)
    sig = {
        "ora_set_trig_libm": [i32],
        "ora_world_create": [f32, f32, ctypes.POINTER(vp)],
        "ora_world_destroy": [vp],
        "ora_set_flags": [vp, i32, i32, i32, i32],
        "ora_set_record_events": [vp, i32],
        "ora_create_bodies": [vp, vp, i32, vp],
        "ora_create_fixtures": [vp, vp, i32, vp],
        "ora_step": [vp, f32, i32, i32],
        "ora_steps": [vp, f32, i32, i32, i32],
        "ora_get_body_states": [vp, u32, u32, vp],
        "ora_set_transform": [vp, u32, b2g.Vec2, f32],
        "ora_set_velocity": [vp, u32, b2g.Vec2, f32],
        "ora_get_counts": [vp, ctypes.POINTER(b2g.Counts)],
        "ora_get_profile": [vp, ctypes.POINTER(b2g.Profile)],
        "ora_get_contacts": [vp, vp, i32, pi32],
        "ora_query_aabb": [vp, f32, f32, f32, f32, vp, i32],
        "ora_ray_cast_closest": [vp, f32, f32, f32, f32, vp],
        "ora_get_pairs": [vp, vp, i32, pi32],
        "ora_get_proxies": [vp, vp, vp, vp, i32],
        "ora_set_solver_order": [vp, vp, i32],
        "ora_get_hook_misses": [vp],
        "ora_get_toi_events": [vp],
        "ora_create_joints": [vp, vp, i32, vp],
        "ora_get_joint_impulses": [vp, u32, u32, vp],
        "ora_set_joint_order": [vp, vp, i32],
        "ora_set_mouse_target": [vp, u32, f32, f32],
        "ora_set_key_order": [vp, i32],
        "ora_get_awake": [vp, u32, u32, vp],
        "ora_get_solver_order": [vp, vp, i32, pi32],
        "ora_get_events": [vp, vp, i32, pi32],
        "ora_polygon_mass": [vp, vp],
        "ora_sincos": [vp, vp, vp, i32],
        "ora_collide": [vp, vp, vp, vp, vp],
        "ora_time_of_impact": [vp, vp, vp, vp, vp, i32, vp],
        "ora_import_state": [vp, vp, i32, vp, i32, vp, i32, f32],
        "ora_destroy_bodies": [vp, vp, i32],
        "ora_destroy_fixtures": [vp, vp, i32],
        "ora_destroy_joints": [vp, vp, i32],
        "ora_set_filter_data": [vp, u32, i32, i32, i32],
        "ora_set_contact_filter": [vp, vp, vp],
        "ora_get_post_solve": [vp, vp, i32, pi32],
        "ora_set_pre_solve": [vp, vp, vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_trig(libm: bool):
    """libm=True: sin/cos from the platform libm (what the Rust reference calls).
    libm=False: the project's correctly rounded sin/cos, identical to the GPU's."""
    load().ora_set_trig_libm(int(libm))


def sincos(x):
    x = np.ascontiguousarray(x, np.float32)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    load().ora_sincos(_ptr(x), _ptr(s), _ptr(c), len(x))
    return s, c


def polygon_mass(fixture_def):
    out = np.zeros(6, np.float32)
    d = np.ascontiguousarray(fixture_def, b2g.FIXTURE_DEF)
    count = load().ora_polygon_mass(_ptr(d), _ptr(out))
    return {"centroid": out[0:2].copy(), "mass": out[2], "center": out[3:5].copy(), "I": out[5], "count": count}


def collide(def_a, xf_a, def_b, xf_b):
    """Manifold of two standalone shapes; xf = (x, y, angle)."""
    da = np.ascontiguousarray(def_a, b2g.FIXTURE_DEF)
    db = np.ascontiguousarray(def_b, b2g.FIXTURE_DEF)
    xa = np.asarray(xf_a, np.float32)
    xb = np.asarray(xf_b, np.float32)
    out = np.zeros(1, b2g.CONTACT_INFO)
    rc = load().ora_collide(_ptr(da), _ptr(xa), _ptr(db), _ptr(xb), _ptr(out))
    if rc != 0:
        raise ValueError("unsupported shape pair")
    return out[0]


def time_of_impact(defs_a, sweeps_a, defs_b, sweeps_b, t_max=None):
    """Time of impact of independent pairs of moving shapes (b2_time_of_impact), same layout as
    b2g.time_of_impact."""
    da = np.ascontiguousarray(defs_a, b2g.FIXTURE_DEF)
    db = np.ascontiguousarray(defs_b, b2g.FIXTURE_DEF)
    sa = np.ascontiguousarray(sweeps_a, b2g.SWEEP)
    sb = np.ascontiguousarray(sweeps_b, b2g.SWEEP)
    tm = None if t_max is None else np.ascontiguousarray(t_max, np.float32)
    out = np.zeros(len(da), b2g.TOI_OUTPUT)
    load().ora_time_of_impact(_ptr(da), _ptr(sa), _ptr(db), _ptr(sb), None if tm is None else _ptr(tm), len(da),
                              _ptr(out))
    return out


class OracleWorld:
    """The CPU restatement of B2world; same method names as b2g.B2world."""

    def __init__(self, gravity=(0.0, -10.0), allow_sleep=False, warm_starting=True, record_events=False,
                 continuous=False):
        self._lib = load()
        self._continuous = continuous
        h = ctypes.c_void_p()
        self._lib.ora_world_create(gravity[0], gravity[1], ctypes.byref(h))
        self._h = h
        self.body_count = 0
        self.fixture_count = 0
        self._allow_sleep = allow_sleep
        self._warm = warm_starting
        self._apply_flags()
        self._lib.ora_set_record_events(self._h, int(record_events))

    def _apply_flags(self):
        rc = self._lib.ora_set_flags(self._h, int(self._allow_sleep), int(self._warm), int(self._continuous), 1)
        assert rc == 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ora_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_allow_sleeping(self, flag):
        self._allow_sleep = bool(flag)
        self._apply_flags()

    def set_warm_starting(self, flag):
        self._warm = bool(flag)
        self._apply_flags()

    def set_continuous_physics(self, flag):
        self._continuous = bool(flag)
        self._apply_flags()

    def set_key_order(self, flag):
        """collide and solve_toi take contacts in key order (the GPU's table order) instead of the
        contact-list order: ties of solve_toi's first time of impact, an event's island order, and
        which contacts see the bodies woken by collide's earlier updates."""
        self._lib.ora_set_key_order(self._h, int(bool(flag)))

    def get_awake(self, first=0, count=None):
        if count is None:
            count = self.body_count - first
        out = np.zeros(count, np.uint8)
        self._lib.ora_get_awake(self._h, first, count, _ptr(out))
        return out

    def toi_events(self):
        """Solid time-of-impact events solved since the world was made."""
        return self._lib.ora_get_toi_events(self._h)

    def create_bodies(self, defs):
        defs = np.ascontiguousarray(defs, b2g.BODY_DEF)
        ids = np.zeros(len(defs), np.uint32)
        self._lib.ora_create_bodies(self._h, _ptr(defs), len(defs), _ptr(ids))
        self.body_count += len(defs)
        return ids

    def create_fixtures(self, defs):
        defs = np.ascontiguousarray(defs, b2g.FIXTURE_DEF)
        ids = np.zeros(len(defs), np.uint32)
        rc = self._lib.ora_create_fixtures(self._h, _ptr(defs), len(defs), _ptr(ids))
        assert rc == 0, rc
        self.fixture_count += len(defs)
        return ids

    def create_joints(self, defs):
        defs = np.ascontiguousarray(defs, b2g.JOINT_DEF)
        ids = np.zeros(len(defs), np.uint32)
        rc = self._lib.ora_create_joints(self._h, _ptr(defs), len(defs), _ptr(ids))
        assert rc == 0, rc
        self.joint_count = getattr(self, "joint_count", 0) + len(defs)
        return ids

    def get_joint_impulses(self):
        n = getattr(self, "joint_count", 0)
        out = np.zeros((n, 5), np.float32)
        if n:
            self._lib.ora_get_joint_impulses(self._h, 0, n, _ptr(out))
        return out

    def set_mouse_target(self, joint, target):
        assert self._lib.ora_set_mouse_target(self._h, joint, float(target[0]), float(target[1])) == 0

    def set_joint_order(self, order):
        """Ordering hook: islands solve their joints in this order of joint ids."""
        o = np.ascontiguousarray(order, np.uint32)
        self._lib.ora_set_joint_order(self._h, _ptr(o) if len(o) else None, len(o))

    def step(self, dt, vi, pi):
        self._lib.ora_step(self._h, dt, vi, pi)

    def steps(self, dt, vi, pi, n):
        self._lib.ora_steps(self._h, dt, vi, pi, n)

    def get_body_states(self, first=0, count=None):
        if count is None:
            count = self.body_count - first
        out = np.zeros(count, b2g.BODY_STATE)
        self._lib.ora_get_body_states(self._h, first, count, _ptr(out))
        return out

    def set_transform(self, body, position, angle):
        self._lib.ora_set_transform(self._h, body, b2g.Vec2(*position), angle)

    def set_velocity(self, body, v, w):
        self._lib.ora_set_velocity(self._h, body, b2g.Vec2(*v), w)

    def get_counts(self):
        c = b2g.Counts()
        self._lib.ora_get_counts(self._h, ctypes.byref(c))
        return c.as_dict()

    def get_profile(self):
        p = b2g.Profile()
        self._lib.ora_get_profile(self._h, ctypes.byref(p))
        return p.as_dict()

    def _get_list(self, fn, dtype, width=1):
        n = ctypes.c_int(0)
        fn(self._h, None, 0, ctypes.byref(n))
        out = np.zeros(max(n.value, 1) * width, dtype)
        fn(self._h, _ptr(out), n.value, ctypes.byref(n))
        return out[: n.value * width]

    def get_contacts(self):
        return self._get_list(self._lib.ora_get_contacts, b2g.CONTACT_INFO)

    def get_pairs(self):
        """Emitted pairs of the last update_pairs as (min fixture, max fixture), in emission order."""
        return self._get_list(self._lib.ora_get_pairs, np.uint32, 2).reshape(-1, 2)

    def get_solver_order(self):
        return self._get_list(self._lib.ora_get_solver_order, np.uint32, 2).reshape(-1, 2)

    def set_pre_solve(self, fn):
        """fn(contact, old_manifold, edit) as b2g.B2world.set_pre_solve."""
        self._pre_solve_cb = None if fn is None else b2g.pre_solve_callback(fn)
        ptr = None if fn is None else ctypes.cast(self._pre_solve_cb, ctypes.c_void_p)
        self._lib.ora_set_pre_solve(self._h, ptr, None)

    def get_post_solve(self):
        return self._get_list(self._lib.ora_get_post_solve, b2g.CONTACT_IMPULSE)

    def get_events(self):
        return self._get_list(self._lib.ora_get_events, b2g.EVENT)

    def get_proxies(self):
        n = self.fixture_count
        aabbs = np.zeros((n, 4), np.float32)
        moved = np.zeros(n, np.uint8)
        ids = np.full(n, -1, np.int32)
        self._lib.ora_get_proxies(self._h, _ptr(aabbs), _ptr(moved), _ptr(ids), n)
        return aabbs, moved, ids

    def query_aabb(self, boxes):
        """(m, 2) array of (box index, fixture): the reference's tree query per box (fat AABBs)."""
        boxes = np.asarray(boxes, np.float32).reshape(-1, 4)
        out = []
        for i, b in enumerate(boxes):
            buf = np.zeros(max(self.fixture_count, 1), np.int32)
            n = self._lib.ora_query_aabb(self._h, float(b[0]), float(b[1]), float(b[2]), float(b[3]), _ptr(buf),
                                         len(buf))
            out.extend((i, int(f)) for f in buf[:n])
        return np.array(out, np.uint32).reshape(-1, 2)

    def ray_cast_closest(self, rays):
        """The reference's world ray cast with a clipping (closest-hit) callback, per ray."""
        rays = np.asarray(rays, np.float32).reshape(-1, 4)
        out = np.zeros(len(rays), b2g.RAY_HIT)
        buf = np.zeros(6, np.float32)
        for i, r in enumerate(rays):
            self._lib.ora_ray_cast_closest(self._h, float(r[0]), float(r[1]), float(r[2]), float(r[3]), _ptr(buf))
            out[i]["fixture"] = int(buf[0])
            out[i]["point"] = buf[1:3]
            out[i]["normal"] = buf[3:5]
            out[i]["fraction"] = buf[5]
        return out

    def set_solver_order(self, pairs):
        """Ordering hook: each island solves its contacts in this (fixture_a, fixture_b) order."""
        if pairs is None or len(pairs) == 0:
            self._lib.ora_set_solver_order(self._h, None, 0)
            return
        p = np.ascontiguousarray(pairs, np.uint32).reshape(-1, 2)
        self._lib.ora_set_solver_order(self._h, _ptr(p), len(p))

    def hook_misses(self):
        return self._lib.ora_get_hook_misses(self._h)

    def destroy_bodies(self, ids):
        ids = np.ascontiguousarray(ids, np.uint32)
        assert self._lib.ora_destroy_bodies(self._h, _ptr(ids), len(ids)) == 0

    def destroy_fixtures(self, ids):
        ids = np.ascontiguousarray(ids, np.uint32)
        assert self._lib.ora_destroy_fixtures(self._h, _ptr(ids), len(ids)) == 0

    def destroy_joints(self, ids):
        ids = np.ascontiguousarray(ids, np.uint32)
        assert self._lib.ora_destroy_joints(self._h, _ptr(ids), len(ids)) == 0

    def set_filter_data(self, fixture, category_bits, mask_bits, group_index):
        assert self._lib.ora_set_filter_data(self._h, int(fixture), int(category_bits), int(mask_bits),
                                             int(group_index)) == 0

    def set_contact_filter(self, fn):
        """fn(fixture_a, fixture_b) -> bool replaces the default contact filter (None restores it)."""
        if fn is None:
            self._filter_cb = None
            self._lib.ora_set_contact_filter(self._h, None, None)
            return
        self._filter_cb = CONTACT_FILTER_FN(lambda user, a, b: 1 if fn(int(a), int(b)) else 0)
        self._lib.ora_set_contact_filter(self._h, ctypes.cast(self._filter_cb, ctypes.c_void_p), None)

    def import_state(self, bodies, fat_aabbs, contacts, inv_dt0):
        """Continue from another engine's post-step state (see ora_import_state)."""
        b = np.ascontiguousarray(bodies, b2g.BODY_STATE)
        a = np.ascontiguousarray(fat_aabbs, np.float32)
        c = np.ascontiguousarray(contacts, b2g.CONTACT_INFO)
        rc = self._lib.ora_import_state(self._h, _ptr(b), len(b), _ptr(a), len(a), _ptr(c), len(c),
                                        np.float32(inv_dt0))
        if rc != 0:
            raise ValueError(f"ora_import_state failed ({rc})")
