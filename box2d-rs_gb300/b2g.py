"""Python binding of libb2g.so (the GB300 world step) shaped like box2d-rs's `B2world`.

The reference's public API is Rust (`B2world::new`, `create_body`, `create_fixture`,
`step`, `set_contact_listener`, `get_profile`; src/b2_world.rs:22-284). This module
exposes the same calls over the C ABI declared in include/b2g.h. Bodies and
fixtures can be created one at a time (like the reference) or in bulk from numpy
arrays of the C structs (how large scenes are uploaded).

There is no CPU fallback: if libb2g.so is missing or fails to load, importing
`load_library` raises.
"""
from __future__ import annotations

import ctypes
import os
import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libb2g.so")

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
CIRCLE, EDGE, POLYGON = 0, 1, 2
POLYGON_HULL, POLYGON_BOX, POLYGON_BOX_ORIENTED = 0, 1, 2
POLYGON_RADIUS = np.float32(0.01)  # B2_POLYGON_RADIUS = 2 * linear slop

OK = 0
ERR_INVALID_ARG, ERR_OUT_OF_MEMORY, ERR_CAPACITY, ERR_TIMEOUT, ERR_CUDA, ERR_UNSUPPORTED = -1, -2, -3, -4, -5, -6
ERRORS = {
    -1: "invalid argument",
    -2: "out of memory",
    -3: "capacity overflow",
    -4: "device wait timed out",
    -5: "CUDA error",
    -6: "unsupported",
    -7: "world locked",
}


class B2GError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__(f"b2g error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


# ---- struct layouts (must match include/b2g.h) ----
class Vec2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


class WorldDef(ctypes.Structure):
    _fields_ = [
        ("gravity", Vec2),
        ("num_worlds", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("body_capacity", ctypes.c_int32),
        ("fixture_capacity", ctypes.c_int32),
        ("contact_capacity", ctypes.c_int32),
        ("pair_capacity", ctypes.c_int32),
    ]


BODY_DEF = np.dtype(
    [
        ("type", "<i4"),
        ("position", "<f4", (2,)),
        ("angle", "<f4"),
        ("linear_velocity", "<f4", (2,)),
        ("angular_velocity", "<f4"),
        ("linear_damping", "<f4"),
        ("angular_damping", "<f4"),
        ("gravity_scale", "<f4"),
        ("allow_sleep", "u1"),
        ("awake", "u1"),
        ("fixed_rotation", "u1"),
        ("bullet", "u1"),
        ("enabled", "u1"),
        ("pad_", "u1", (3,)),
        ("world_index", "<u4"),
        ("user_data", "<u8"),
    ],
    align=True,
)

FIXTURE_DEF = np.dtype(
    [
        ("body", "<u4"),
        ("shape_type", "<i4"),
        ("polygon_mode", "<i4"),
        ("vertex_count", "<i4"),
        ("vertices", "<f4", (8, 2)),
        ("radius", "<f4"),
        ("box_half_extents", "<f4", (2,)),
        ("box_center", "<f4", (2,)),
        ("box_angle", "<f4"),
        ("one_sided", "<i4"),
        ("friction", "<f4"),
        ("restitution", "<f4"),
        ("restitution_threshold", "<f4"),
        ("density", "<f4"),
        ("is_sensor", "<i4"),
        ("category_bits", "<u2"),
        ("mask_bits", "<u2"),
        ("group_index", "<i2"),
        ("pad_", "<i2"),
        ("user_data", "<u8"),
    ],
    align=True,
)

BODY_STATE = np.dtype(
    [
        ("position", "<f4", (2,)),
        ("angle", "<f4"),
        ("linear_velocity", "<f4", (2,)),
        ("angular_velocity", "<f4"),
        ("world_center", "<f4", (2,)),
    ]
)

CONTACT_INFO = np.dtype(
    [
        ("fixture_a", "<u4"),
        ("fixture_b", "<u4"),
        ("touching", "<i4"),
        ("manifold_type", "<i4"),
        ("point_count", "<i4"),
        ("local_normal", "<f4", (2,)),
        ("local_point", "<f4", (2,)),
        ("point_local", "<f4", (2, 2)),
        ("normal_impulse", "<f4", (2,)),
        ("tangent_impulse", "<f4", (2,)),
        ("point_id", "<u4", (2,)),
        ("friction", "<f4"),
        ("restitution", "<f4"),
        ("restitution_threshold", "<f4"),
    ]
)

EVENT = np.dtype([("kind", "<i4"), ("fixture_a", "<u4"), ("fixture_b", "<u4")])

# B2Sweep (src/b2_math.rs): local centre, centre and angle at the start (c0, a0) and the end (c, a)
SWEEP = np.dtype([("local_center", "<f4", (2,)), ("c0", "<f4", (2,)), ("c", "<f4", (2,)), ("a0", "<f4"),
                  ("a", "<f4"), ("alpha0", "<f4"), ("pad", "<f4")])
JOINT_REVOLUTE = 1
JOINT_DEF = np.dtype(
    [
        ("type", "<i4"),
        ("body_a", "<u4"),
        ("body_b", "<u4"),
        ("collide_connected", "<i4"),
        ("local_anchor_a", "<f4", (2,)),
        ("local_anchor_b", "<f4", (2,)),
        ("reference_angle", "<f4"),
        ("enable_limit", "<i4"),
        ("lower_angle", "<f4"),
        ("upper_angle", "<f4"),
        ("enable_motor", "<i4"),
        ("motor_speed", "<f4"),
        ("max_motor_torque", "<f4"),
        ("length", "<f4"),
        ("min_length", "<f4"),
        ("max_length", "<f4"),
        ("stiffness", "<f4"),
        ("damping", "<f4"),
        ("max_force", "<f4"),
        ("max_torque", "<f4"),
        ("correction_factor", "<f4"),
        ("angular_offset", "<f4"),
        ("linear_offset", "<f4", (2,)),
        ("target", "<f4", (2,)),
        ("local_axis_a", "<f4", (2,)),
        ("lower_translation", "<f4"),
        ("upper_translation", "<f4"),
        ("max_motor_force", "<f4"),
        ("ground_anchor_a", "<f4", (2,)),
        ("ground_anchor_b", "<f4", (2,)),
        ("length_a", "<f4"),
        ("length_b", "<f4"),
        ("ratio", "<f4"),
        ("joint1", "<u4"),
        ("joint2", "<u4"),
    ]
)
JOINT_DISTANCE = 3
JOINT_GEAR = 6
JOINT_WELD = 8
JOINT_FRICTION = 9
JOINT_MOTOR = 11
JOINT_MOUSE = 5
JOINT_PRISMATIC = 2
JOINT_WHEEL = 7
JOINT_PULLEY = 4


def friction_joint(body_a, body_b, anchor_a, anchor_b, max_force, max_torque, collide_connected=False):
    """B2frictionJointDef: top-down friction (linear and angular) between two bodies."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_FRICTION
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["max_force"], d["max_torque"] = max_force, max_torque
    return d


def motor_joint(body_a, body_b, linear_offset=(0.0, 0.0), angular_offset=0.0, max_force=1.0, max_torque=1.0,
                correction_factor=0.3, collide_connected=False):
    """B2motorJointDef: drives body B to body A's position plus linear_offset (in A's frame) and A's
    angle plus angular_offset, with bounded force and torque."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_MOTOR
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["linear_offset"], d["angular_offset"] = linear_offset, angular_offset
    d["max_force"], d["max_torque"], d["correction_factor"] = max_force, max_torque, correction_factor
    return d


def mouse_joint(body_a, body_b, target, max_force, stiffness=0.0, damping=0.0, collide_connected=False):
    """B2mouseJointDef: pulls body B's point under `target` (world) towards the target; body A only ties
    the joint into the world."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_MOUSE
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["target"] = target
    d["max_force"], d["stiffness"], d["damping"] = max_force, stiffness, damping
    return d


def prismatic_joint(body_a, body_b, anchor_a, anchor_b, axis, reference_angle=0.0, limits=None, motor=None,
                    collide_connected=False):
    """B2prismaticJointDef: body B slides along `axis` (body A's frame); limits = (lower, upper)
    translation; motor = (speed, max force)."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_PRISMATIC
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["local_axis_a"], d["reference_angle"] = axis, reference_angle
    if limits is not None:
        d["enable_limit"] = 1
        d["lower_translation"], d["upper_translation"] = limits
    if motor is not None:
        d["enable_motor"] = 1
        d["motor_speed"], d["max_motor_force"] = motor
    return d


def wheel_joint(body_a, body_b, anchor_a, anchor_b, axis, stiffness=0.0, damping=0.0, limits=None, motor=None,
                collide_connected=False):
    """B2wheelJointDef: body B rides a spring along `axis` (body A's frame) and spins freely;
    limits = (lower, upper) translation; motor = (speed, max torque)."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_WHEEL
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["local_axis_a"] = axis
    d["stiffness"], d["damping"] = stiffness, damping
    if limits is not None:
        d["enable_limit"] = 1
        d["lower_translation"], d["upper_translation"] = limits
    if motor is not None:
        d["enable_motor"] = 1
        d["motor_speed"], d["max_motor_torque"] = motor
    return d


def pulley_joint(body_a, body_b, ground_a, ground_b, anchor_a, anchor_b, length_a, length_b, ratio=1.0,
                 collide_connected=True):
    """B2pulleyJointDef: ropes from world ground anchors to local anchors on each body, with
    length_a + ratio * length_b held constant."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_PULLEY
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["ground_anchor_a"], d["ground_anchor_b"] = ground_a, ground_b
    d["length_a"], d["length_b"], d["ratio"] = length_a, length_b, ratio
    return d


def gear_joint(joint1, joint2, body_a, body_b, ratio=1.0, collide_connected=False):
    """B2gearJointDef: couples two revolute or prismatic joints (ids of joints created earlier) so that
    coordinate1 + ratio * coordinate2 stays constant; body_a and body_b are the joints' second bodies."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_GEAR
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["joint1"], d["joint2"], d["ratio"] = joint1, joint2, ratio
    return d


def weld_joint(body_a, body_b, anchor_a, anchor_b, reference_angle=0.0, stiffness=0.0, damping=0.0,
               collide_connected=False):
    """B2weldJointDef with local anchors; stiffness > 0 makes the angular part a spring."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_WELD
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["reference_angle"] = reference_angle
    d["stiffness"], d["damping"] = stiffness, damping
    return d


def distance_joint(body_a, body_b, anchor_a, anchor_b, length, min_length=None, max_length=None, stiffness=0.0,
                   damping=0.0, collide_connected=False):
    """B2distanceJointDef with local anchors; min/max length default to the rest length (rigid)."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_DISTANCE
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["length"] = length
    d["min_length"] = length if min_length is None else min_length
    d["max_length"] = length if max_length is None else max_length
    d["stiffness"], d["damping"] = stiffness, damping
    return d


def revolute_joint(body_a, body_b, anchor_a, anchor_b, reference_angle=0.0, collide_connected=False,
                   limits=None, motor=None):
    """B2revoluteJointDef: local anchors on each body; limits = (lower, upper) radians;
    motor = (speed, max torque)."""
    d = np.zeros(1, JOINT_DEF)
    d["type"] = JOINT_REVOLUTE
    d["body_a"], d["body_b"] = body_a, body_b
    d["collide_connected"] = int(bool(collide_connected))
    d["local_anchor_a"], d["local_anchor_b"] = anchor_a, anchor_b
    d["reference_angle"] = reference_angle
    if limits is not None:
        d["enable_limit"] = 1
        d["lower_angle"], d["upper_angle"] = limits
    if motor is not None:
        d["enable_motor"] = 1
        d["motor_speed"], d["max_motor_torque"] = motor
    return d


TOI_OUTPUT = np.dtype([("state", "<i4"), ("t", "<f4")])
TOI_UNKNOWN, TOI_FAILED, TOI_OVERLAPPED, TOI_TOUCHING, TOI_SEPARATED = range(5)
TOI_SIDE_BY_SIDE, TOI_ONE_AT_A_TIME, TOI_RESTART_ON_ADVANCE = range(3)  # b2g_set_toi_schedule

RAY_HIT = np.dtype([("fixture", "<i4"), ("point", "<f4", (2,)), ("normal", "<f4", (2,)), ("fraction", "<f4")])
assert RAY_HIT.itemsize == 24

# b2g_tape_slot / b2g_tape_step (include/b2g.h)
TAPE_SLOT = np.dtype(
    [
        ("body_a", "<i4"),
        ("body_b", "<i4"),
        ("count_type_flags", "<i4"),
        ("colour", "<i4"),
        ("local_normal", "<f4", (2,)),
        ("local_point", "<f4", (2,)),
        ("points", "<f4", (4,)),
        ("inv_mass", "<f4", (2,)),
        ("inv_inertia", "<f4", (2,)),
        ("local_center_a", "<f4", (2,)),
        ("local_center_b", "<f4", (2,)),
        ("friction", "<f4"),
        ("restitution", "<f4"),
        ("restitution_threshold", "<f4"),
        ("tangent_speed", "<f4"),
        ("radius", "<f4", (2,)),
        ("island", "<i4"),
        ("position_iterations", "<i4"),
        ("impulses", "<f4", (4,)),
        ("carry", "<i4", (2,)),
        ("ids", "<u4", (2,)),
    ]
)
TAPE_STEP = np.dtype(
    [
        ("dt", "<f4"),
        ("dt_ratio", "<f4"),
        ("gravity", "<f4", (2,)),
        ("velocity_iterations", "<i4"),
        ("position_iterations", "<i4"),
        ("warm_starting", "<i4"),
        ("num_slots", "<i4"),
        ("slot_offset", "<i8"),
        ("num_colours", "<i4"),
        ("num_contacts", "<i4"),
    ]
)
assert TAPE_SLOT.itemsize == 144 and TAPE_STEP.itemsize == 48


class LaunchConfig(ctypes.Structure):
    _fields_ = [("coop_blocks_per_sm", ctypes.c_int32), ("collide_block", ctypes.c_int32),
                ("traverse_block", ctypes.c_int32), ("tuning_steps", ctypes.c_int32), ("solver_block", ctypes.c_int32),
                ("collide_group", ctypes.c_int32)]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_ if n != "tuning_steps"}


class TapeInfo(ctypes.Structure):
    _fields_ = [
        ("recording", ctypes.c_int32),
        ("steps", ctypes.c_int32),
        ("slots", ctypes.c_int64),
        ("checkpoint_interval", ctypes.c_int32),
        ("valid", ctypes.c_int32),
        ("device_bytes", ctypes.c_int64),
        ("replay_mismatches", ctypes.c_uint32),
        ("pad", ctypes.c_int32),
    ]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_ if n != "pad"}


class Profile(ctypes.Structure):
    _fields_ = [
        (n, ctypes.c_float)
        for n in ("step", "collide", "solve", "solve_init", "solve_velocity", "solve_position", "broadphase", "solve_toi")
    ]

    def as_dict(self):
        return {n: float(getattr(self, n)) for n, _ in self._fields_}


CONTACT_IMPULSE = np.dtype([("fixture_a", np.uint32), ("fixture_b", np.uint32), ("normal_impulses", np.float32, 2),
                            ("tangent_impulses", np.float32, 2), ("count", np.int32)])


class ContactEdit(ctypes.Structure):
    """b2g_contact_edit: what a pre_solve callback may change (B2contact's setters)."""
    _fields_ = [("enabled", ctypes.c_int32), ("friction", ctypes.c_float), ("restitution", ctypes.c_float),
                ("restitution_threshold", ctypes.c_float), ("tangent_speed", ctypes.c_float)]


CONTACT_FILTER_FN = ctypes.CFUNCTYPE(ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32)
PRE_SOLVE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ContactEdit))


def contact_filter_callback(fn):
    """A C contact filter calling fn(fixture_a, fixture_b) -> bool."""
    return CONTACT_FILTER_FN(lambda user, a, b: 1 if fn(int(a), int(b)) else 0)


def pre_solve_callback(fn):
    """A C pre_solve callback calling fn(contact, old_manifold, edit): the first two are CONTACT_INFO
    records, edit a ContactEdit to change in place."""
    def call(user, c, old, edit):
        info = np.frombuffer(ctypes.string_at(c, CONTACT_INFO.itemsize), CONTACT_INFO)[0]
        prev = np.frombuffer(ctypes.string_at(old, CONTACT_INFO.itemsize), CONTACT_INFO)[0]
        fn(info, prev, edit.contents)
    return PRE_SOLVE_FN(call)


class StepStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("bp_node_visits", "bp_leaf_checks", "new_pairs", "contacts", "constraints",
                                               "interior_slots", "parts", "colours", "contact_capacity",
                                               "pair_capacity", "capacity_grows", "hierarchy_age", "bp_moved_proxies",
                                               "bp_warp_max_visits", "bp_warp_max_checks")]


class Counts(ctypes.Structure):
    _fields_ = [
        (n, ctypes.c_int32)
        for n in ("bodies", "fixtures", "proxies", "contacts", "touching_contacts", "islands_solved", "colours", "pairs")
    ]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


assert BODY_DEF.itemsize == 64, BODY_DEF.itemsize
assert FIXTURE_DEF.itemsize == 144, FIXTURE_DEF.itemsize
assert BODY_STATE.itemsize == 32
assert CONTACT_INFO.itemsize == 88
assert ctypes.sizeof(WorldDef) == 32


# ---- defs (defaults of B2bodyDef, src/b2_body.rs:39-59, and B2fixtureDef, src/b2_fixture.rs:44-56) ----
def body_defs(n):
    d = np.zeros(n, BODY_DEF)
    d["type"] = STATIC
    d["gravity_scale"] = 1.0
    d["allow_sleep"] = 1
    d["awake"] = 1
    d["enabled"] = 1
    return d


def fixture_defs(n):
    d = np.zeros(n, FIXTURE_DEF)
    d["friction"] = 0.2
    d["restitution_threshold"] = 1.0
    d["category_bits"] = 0x0001
    d["mask_bits"] = 0xFFFF
    d["radius"] = POLYGON_RADIUS
    return d


def body_def(type=STATIC, position=(0.0, 0.0), angle=0.0, linear_velocity=(0.0, 0.0), angular_velocity=0.0,
             linear_damping=0.0, angular_damping=0.0, gravity_scale=1.0, allow_sleep=True, awake=True,
             fixed_rotation=False, bullet=False, enabled=True, world_index=0):
    d = body_defs(1)
    d["type"] = type
    d["position"] = position
    d["angle"] = angle
    d["linear_velocity"] = linear_velocity
    d["angular_velocity"] = angular_velocity
    d["linear_damping"] = linear_damping
    d["angular_damping"] = angular_damping
    d["gravity_scale"] = gravity_scale
    d["allow_sleep"] = allow_sleep
    d["awake"] = awake
    d["fixed_rotation"] = fixed_rotation
    d["bullet"] = bullet
    d["enabled"] = enabled
    d["world_index"] = world_index
    return d


def _material(d, density, friction, restitution, restitution_threshold, is_sensor):
    d["density"] = density
    d["friction"] = friction
    d["restitution"] = restitution
    d["restitution_threshold"] = restitution_threshold
    d["is_sensor"] = is_sensor


def circle_fixture(body, radius, center=(0.0, 0.0), density=0.0, friction=0.2, restitution=0.0,
                   restitution_threshold=1.0, is_sensor=False):
    d = fixture_defs(1)
    d["body"] = body
    d["shape_type"] = CIRCLE
    d["radius"] = radius
    d["vertices"][0, 0] = center
    _material(d, density, friction, restitution, restitution_threshold, is_sensor)
    return d


def box_fixture(body, hx, hy, center=None, angle=0.0, density=0.0, friction=0.2, restitution=0.0,
                restitution_threshold=1.0, is_sensor=False):
    d = fixture_defs(1)
    d["body"] = body
    d["shape_type"] = POLYGON
    if center is None:
        d["polygon_mode"] = POLYGON_BOX
    else:
        d["polygon_mode"] = POLYGON_BOX_ORIENTED
        d["box_center"] = center
        d["box_angle"] = angle
    d["box_half_extents"] = (hx, hy)
    _material(d, density, friction, restitution, restitution_threshold, is_sensor)
    return d


def polygon_fixture(body, vertices, density=0.0, friction=0.2, restitution=0.0, restitution_threshold=1.0,
                    is_sensor=False):
    v = np.asarray(vertices, np.float32).reshape(-1, 2)
    d = fixture_defs(1)
    d["body"] = body
    d["shape_type"] = POLYGON
    d["polygon_mode"] = POLYGON_HULL
    d["vertex_count"] = len(v)
    d["vertices"][0, : len(v)] = v
    _material(d, density, friction, restitution, restitution_threshold, is_sensor)
    return d


def edge_fixture(body, v1, v2, v0=None, v3=None, density=0.0, friction=0.2, restitution=0.0,
                 restitution_threshold=1.0, is_sensor=False):
    d = fixture_defs(1)
    d["body"] = body
    d["shape_type"] = EDGE
    one_sided = v0 is not None and v3 is not None
    d["vertices"][0, 0] = v0 if one_sided else (0.0, 0.0)
    d["vertices"][0, 1] = v1
    d["vertices"][0, 2] = v2
    d["vertices"][0, 3] = v3 if one_sided else (0.0, 0.0)
    d["one_sided"] = one_sided
    _material(d, density, friction, restitution, restitution_threshold, is_sensor)
    return d


# ---- library ----
_lib = None


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def load_library(path=LIB_PATH):
    """Load libb2g.so; raises OSError if it is missing (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    vp, i32, u32, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_float
    sig = {
        "b2g_world_create": [ctypes.POINTER(WorldDef), ctypes.POINTER(vp)],
        "b2g_world_destroy": [vp],
        "b2g_create_bodies": [vp, vp, i32, vp],
        "b2g_create_fixtures": [vp, vp, i32, vp],
        "b2g_step": [vp, f32, i32, i32],
        "b2g_synchronize": [vp],
        "b2g_get_body_states": [vp, u32, u32, vp],
        "b2g_get_body_states_async": [vp, u32, u32, vp],
        "b2g_wait_body_states": [vp],
        "b2g_get_mass_data": [vp, u32, u32, vp],
        "b2g_set_transform": [vp, u32, Vec2, f32],
        "b2g_set_linear_velocity": [vp, u32, Vec2],
        "b2g_set_angular_velocity": [vp, u32, f32],
        "b2g_apply_force": [vp, u32, Vec2, Vec2, i32],
        "b2g_apply_linear_impulse": [vp, u32, Vec2, Vec2, i32],
        "b2g_apply_force_to_center": [vp, u32, Vec2, i32],
        "b2g_apply_torque": [vp, u32, f32, i32],
        "b2g_apply_linear_impulse_to_center": [vp, u32, Vec2, i32],
        "b2g_apply_angular_impulse": [vp, u32, f32, i32],
        "b2g_set_awake": [vp, u32, i32],
        "b2g_set_gravity": [vp, Vec2],
        "b2g_set_allow_sleeping": [vp, i32],
        "b2g_set_warm_starting": [vp, i32],
        "b2g_set_part_solve": [vp, i32],
        "b2g_set_continuous_physics": [vp, i32],
        "b2g_set_auto_clear_forces": [vp, i32],
        "b2g_clear_forces": [vp],
        "b2g_get_profile": [vp, ctypes.POINTER(Profile)],
        "b2g_get_counts": [vp, ctypes.POINTER(Counts)],
        "b2g_get_toi_stats": [vp, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                              ctypes.POINTER(ctypes.c_int32)],
        "b2g_set_toi_schedule": [vp, i32],
        "b2g_get_awake": [vp, u32, u32, vp],
        "b2g_create_joints": [vp, vp, i32, vp],
        "b2g_set_mouse_target": [vp, u32, Vec2],
        "b2g_get_joint_impulses": [vp, u32, u32, vp],
        "b2g_get_joint_order": [vp, vp, i32, ctypes.POINTER(ctypes.c_int32)],
        "b2g_state_size": [vp, ctypes.POINTER(ctypes.c_uint64)],
        "b2g_state_save": [vp, vp, ctypes.c_uint64],
        "b2g_state_load": [vp, vp, ctypes.c_uint64],
        "b2g_get_contacts": [vp, vp, i32, ctypes.POINTER(i32)],
        "b2g_get_events": [vp, vp, i32, ctypes.POINTER(i32)],
        "b2g_get_pairs": [vp, vp, i32, ctypes.POINTER(i32)],
        "b2g_get_proxies": [vp, vp, vp, i32],
        "b2g_get_proxy_ids": [vp, vp, i32],
        "b2g_get_post_solve": [vp, vp, i32, ctypes.POINTER(i32)],
        "b2g_set_contact_filter": [vp, vp, vp],
        "b2g_set_pre_solve": [vp, vp, vp],
        "b2g_destroy_bodies": [vp, vp, i32],
        "b2g_destroy_fixtures": [vp, vp, i32],
        "b2g_destroy_joints": [vp, vp, i32],
        "b2g_set_filter_data": [vp, u32, ctypes.c_uint16, ctypes.c_uint16, ctypes.c_int16],
        "b2g_refilter": [vp, u32],
        "b2g_get_solver_order": [vp, vp, i32, ctypes.POINTER(i32)],
        "b2g_set_contact_events": [vp, i32],
        "b2g_set_record_pairs": [vp, i32],
        "b2g_set_graph_capture": [vp, i32],
        "b2g_set_barrier_limit": [vp, ctypes.c_int64],
        "b2g_set_auto_grow": [vp, i32],
        "b2g_set_hierarchy_max_age": [vp, i32],
        "b2g_debug_hold_barriers": [vp, i32],
        "b2g_get_phase_times": [vp, vp, i32],
        "b2g_get_step_stats": [vp, ctypes.POINTER(StepStats)],
        "b2g_ray_cast_closest": [vp, vp, vp, i32, vp],
        "b2g_query_aabb": [vp, vp, vp, i32, vp, i32, ctypes.POINTER(i32)],
        "b2g_get_launch_config": [vp, ctypes.POINTER(LaunchConfig)],
        "b2g_set_launch_config": [vp, ctypes.POINTER(LaunchConfig)],
        "b2g_autotune": [vp, f32, i32, i32, i32, ctypes.POINTER(LaunchConfig)],
        "b2g_tape_begin": [vp, i32, i32, ctypes.c_int64],
        "b2g_tape_end": [vp],
        "b2g_tape_info_get": [vp, ctypes.POINTER(TapeInfo)],
        "b2g_backward": [vp, vp, vp],
        "b2g_tape_get_step": [vp, i32, vp, vp, vp, i32],
        "b2g_tape_get_checkpoint": [vp, i32, vp, u32],
        "b2g_version": [],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.b2g_last_error.argtypes = [vp]
    lib.b2g_last_error.restype = ctypes.c_char_p
    lib.b2g_collide_pairs.argtypes = [vp, vp, vp, vp, i32, vp]
    lib.b2g_collide_pairs.restype = ctypes.c_int
    lib.b2g_time_of_impact.argtypes = [vp, vp, vp, vp, vp, i32, vp]
    lib.b2g_time_of_impact.restype = ctypes.c_int
    lib.b2g_get_launch_count.argtypes = []
    lib.b2g_get_launch_count.restype = ctypes.c_int64
    _lib = lib
    return lib


def collide_pairs(defs_a, xf_a, defs_b, xf_b):
    """GPU manifolds of independent shape pairs (b2_collide_*); xf rows are (x, y, angle)."""
    lib = load_library()
    da = np.ascontiguousarray(defs_a, FIXTURE_DEF)
    db = np.ascontiguousarray(defs_b, FIXTURE_DEF)
    xa = np.ascontiguousarray(xf_a, np.float32)
    xb = np.ascontiguousarray(xf_b, np.float32)
    out = np.zeros(len(da), CONTACT_INFO)
    rc = lib.b2g_collide_pairs(_ptr(da), _ptr(xa), _ptr(db), _ptr(xb), len(da), _ptr(out))
    if rc != OK:
        raise B2GError(rc, "b2g_collide_pairs")
    return out


def time_of_impact(defs_a, sweeps_a, defs_b, sweeps_b, t_max=None):
    """GPU time of impact of independent pairs of moving shapes (b2_time_of_impact): a TOI_OUTPUT
    (state TOI_*, t) per pair; t_max per pair (default 1)."""
    lib = load_library()
    da = np.ascontiguousarray(defs_a, FIXTURE_DEF)
    db = np.ascontiguousarray(defs_b, FIXTURE_DEF)
    sa = np.ascontiguousarray(sweeps_a, SWEEP)
    sb = np.ascontiguousarray(sweeps_b, SWEEP)
    tm = None if t_max is None else np.ascontiguousarray(t_max, np.float32)
    out = np.zeros(len(da), TOI_OUTPUT)
    rc = lib.b2g_time_of_impact(_ptr(da), _ptr(sa), _ptr(db), _ptr(sb), None if tm is None else _ptr(tm), len(da),
                                _ptr(out))
    if rc != OK:
        raise B2GError(rc, "b2g_time_of_impact")
    return out


class B2world:
    """A world (or a batch of independent worlds) stepped on the GPU.

    Mirrors `B2world` of box2d-rs (src/b2_world.rs:22-284). With `num_worlds > 1`
    every body carries `world_index`; worlds share launches but never interact.
    """

    def __init__(self, gravity=(0.0, -10.0), num_worlds=1, device=0, body_capacity=0, fixture_capacity=0,
                 contact_capacity=0, pair_capacity=0):
        self._lib = load_library()
        d = WorldDef(Vec2(*gravity), num_worlds, device, body_capacity, fixture_capacity, contact_capacity,
                     pair_capacity)
        h = ctypes.c_void_p()
        self._check(self._lib.b2g_world_create(ctypes.byref(d), ctypes.byref(h)), None)
        self._h = h
        self._listener = None
        self.body_count = 0
        self.fixture_count = 0

    def _check(self, rc, h="self"):
        if rc != OK:
            msg = ""
            hh = self._h if h == "self" else h
            if hh is not None:
                m = self._lib.b2g_last_error(hh)
                msg = m.decode() if m else ""
            raise B2GError(rc, msg)
        return rc

    def close(self):
        if getattr(self, "_h", None):
            self._lib.b2g_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- creation --
    def create_bodies(self, defs):
        defs = np.ascontiguousarray(defs, BODY_DEF)
        ids = np.zeros(len(defs), np.uint32)
        self._check(self._lib.b2g_create_bodies(self._h, _ptr(defs), len(defs), _ptr(ids)))
        self.body_count += len(defs)
        return ids

    def create_body(self, **kw):
        return int(self.create_bodies(body_def(**kw))[0])

    def create_fixtures(self, defs):
        defs = np.ascontiguousarray(defs, FIXTURE_DEF)
        ids = np.zeros(len(defs), np.uint32)
        self._check(self._lib.b2g_create_fixtures(self._h, _ptr(defs), len(defs), _ptr(ids)))
        self.fixture_count += len(defs)
        return ids

    def create_fixture(self, d):
        return int(self.create_fixtures(d)[0])

    # -- step --
    def step(self, dt, velocity_iterations, position_iterations):
        self._check(self._lib.b2g_step(self._h, dt, velocity_iterations, position_iterations))
        if self._listener is not None:
            for ev in self.get_events():
                if ev["kind"] == 0:
                    self._listener.begin_contact(int(ev["fixture_a"]), int(ev["fixture_b"]))
                else:
                    self._listener.end_contact(int(ev["fixture_a"]), int(ev["fixture_b"]))

    def synchronize(self):
        self._check(self._lib.b2g_synchronize(self._h))

    # -- state --
    def get_body_states(self, first=0, count=None, out=None):
        if count is None:
            count = self.body_count - first
        if out is None:
            out = np.zeros(count, BODY_STATE)
        self._check(self._lib.b2g_get_body_states(self._h, first, count, _ptr(out)))
        return out

    def get_body_states_async(self, out, first=0):
        """Start copying body states [first, first + len(out)) into `out` without waiting; the copy
        overlaps the next steps. `out` must not be read or freed before wait_body_states()."""
        if out.dtype != BODY_STATE or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous BODY_STATE array")
        self._check(self._lib.b2g_get_body_states_async(self._h, first, len(out), _ptr(out)))
        return out

    def wait_body_states(self):
        self._check(self._lib.b2g_wait_body_states(self._h))

    def get_mass_data(self, first=0, count=None):
        """(n, 6) float32: mass, 1/mass, inertia about the centre, its inverse, local centre x, y."""
        if count is None:
            count = self.body_count - first
        out = np.zeros((count, 6), np.float32)
        self._check(self._lib.b2g_get_mass_data(self._h, first, count, _ptr(out)))
        return out

    def set_transform(self, body, position, angle):
        self._check(self._lib.b2g_set_transform(self._h, body, Vec2(*position), angle))

    def set_linear_velocity(self, body, v):
        self._check(self._lib.b2g_set_linear_velocity(self._h, body, Vec2(*v)))

    def set_angular_velocity(self, body, w):
        self._check(self._lib.b2g_set_angular_velocity(self._h, body, w))

    def apply_force(self, body, force, point, wake=True):
        self._check(self._lib.b2g_apply_force(self._h, body, Vec2(*force), Vec2(*point), int(wake)))

    def apply_linear_impulse(self, body, impulse, point, wake=True):
        self._check(self._lib.b2g_apply_linear_impulse(self._h, body, Vec2(*impulse), Vec2(*point), int(wake)))

    def apply_force_to_center(self, body, force, wake=True):
        self._check(self._lib.b2g_apply_force_to_center(self._h, body, Vec2(*force), int(wake)))

    def apply_torque(self, body, torque, wake=True):
        self._check(self._lib.b2g_apply_torque(self._h, body, float(torque), int(wake)))

    def apply_linear_impulse_to_center(self, body, impulse, wake=True):
        self._check(self._lib.b2g_apply_linear_impulse_to_center(self._h, body, Vec2(*impulse), int(wake)))

    def apply_angular_impulse(self, body, impulse, wake=True):
        self._check(self._lib.b2g_apply_angular_impulse(self._h, body, float(impulse), int(wake)))

    def set_awake(self, body, flag):
        self._check(self._lib.b2g_set_awake(self._h, body, int(flag)))

    # -- flags --
    def set_gravity(self, g):
        self._check(self._lib.b2g_set_gravity(self._h, Vec2(*g)))

    def set_allow_sleeping(self, flag):
        self._check(self._lib.b2g_set_allow_sleeping(self._h, int(flag)))

    def set_warm_starting(self, flag):
        self._check(self._lib.b2g_set_warm_starting(self._h, int(flag)))

    def set_part_solve(self, flag):
        """Part-local solve on (default) or off (every constraint in grid-wide colours)."""
        self._check(self._lib.b2g_set_part_solve(self._h, int(flag)))

    def set_continuous_physics(self, flag):
        self._check(self._lib.b2g_set_continuous_physics(self._h, int(flag)))

    def set_auto_clear_forces(self, flag):
        self._check(self._lib.b2g_set_auto_clear_forces(self._h, int(flag)))

    def clear_forces(self):
        self._check(self._lib.b2g_clear_forces(self._h))

    def set_contact_listener(self, listener):
        """`listener` has begin_contact(fa, fb) and end_contact(fa, fb); events are replayed after each step."""
        self._listener = listener
        self.set_contact_events(listener is not None)

    def set_contact_events(self, flag):
        self._check(self._lib.b2g_set_contact_events(self._h, int(flag)))

    def set_record_pairs(self, flag):
        self._check(self._lib.b2g_set_record_pairs(self._h, int(flag)))

    def set_graph_capture(self, flag):
        self._check(self._lib.b2g_set_graph_capture(self._h, int(flag)))

    def set_auto_grow(self, flag):
        """Contact and pair capacities grow on overflow, the pass repeated exactly (b2g_set_auto_grow)."""
        self._check(self._lib.b2g_set_auto_grow(self._h, int(flag)))

    def set_hierarchy_max_age(self, passes):
        """Passes the broadphase keeps its hierarchy before a rebuild (0: rebuild every pass)."""
        self._check(self._lib.b2g_set_hierarchy_max_age(self._h, int(passes)))

    def set_barrier_limit(self, cycles):
        """Grid-barrier wait limit of the world's persistent kernels in clock cycles (0: default)."""
        self._check(self._lib.b2g_set_barrier_limit(self._h, int(cycles)))

    def debug_hold_barriers(self, extra):
        """Test hook: every grid barrier waits for `extra` arrivals that never come (0: off)."""
        self._check(self._lib.b2g_debug_hold_barriers(self._h, int(extra)))

    # -- introspection --
    def get_profile(self):
        p = Profile()
        self._check(self._lib.b2g_get_profile(self._h, ctypes.byref(p)))
        return p.as_dict()

    PHASES = ("initial_broadphase", "collide", "islands", "colouring", "solver", "broadphase_tree", "contact_merge")
    TREE_PHASES = ("bp_sort", "bp_hierarchy", "bp_traverse")

    def get_phase_times(self, tree_split=False):
        """Device milliseconds of the last step's phases (see b2g_get_phase_times); with tree_split
        also the broadphase tree pass in three (keys + sort, hierarchy, traversal)."""
        out = np.zeros(10, np.float32)
        self._check(self._lib.b2g_get_phase_times(self._h, _ptr(out), 10))
        names = self.PHASES + (self.TREE_PHASES if tree_split else ())
        return dict(zip(names, map(float, out)))

    def get_step_stats(self):
        """Work counts of the last step (b2g_get_step_stats)."""
        out = StepStats()
        self._check(self._lib.b2g_get_step_stats(self._h, ctypes.byref(out)))
        return {k: int(getattr(out, k)) for k, _ in StepStats._fields_}

    def get_counts(self):
        c = Counts()
        self._check(self._lib.b2g_get_counts(self._h, ctypes.byref(c)))
        return c.as_dict()

    def get_toi_stats(self):
        """(solid time-of-impact events since creation, iterations of the last step's pass,
        passes restarted one event at a time)."""
        e, it, r = ctypes.c_int32(0), ctypes.c_int32(0), ctypes.c_int32(0)
        self._check(self._lib.b2g_get_toi_stats(self._h, ctypes.byref(e), ctypes.byref(it), ctypes.byref(r)))
        return int(e.value), int(it.value), int(r.value)

    def get_awake(self, first=0, count=None):
        """B2body::is_awake of bodies [first, first + count) as a uint8 array."""
        if count is None:
            count = self.body_count - first
        out = np.zeros(count, np.uint8)
        self._check(self._lib.b2g_get_awake(self._h, int(first), int(count), out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def create_joints(self, defs):
        defs = np.ascontiguousarray(defs, JOINT_DEF)
        ids = np.zeros(len(defs), np.uint32)
        self._check(self._lib.b2g_create_joints(self._h, defs.ctypes.data_as(ctypes.c_void_p), len(defs),
                                                ids.ctypes.data_as(ctypes.c_void_p)))
        self.joint_count = getattr(self, "joint_count", 0) + len(defs)
        return ids

    def get_joint_impulses(self):
        """(joints, 5): accumulated impulse x, y, motor, lower limit, upper limit."""
        n = getattr(self, "joint_count", 0)
        out = np.zeros((n, 5), np.float32)
        if n:
            self._check(self._lib.b2g_get_joint_impulses(self._h, 0, n, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_mouse_target(self, joint, target):
        self._check(self._lib.b2g_set_mouse_target(self._h, joint, Vec2(*target)))

    def get_joint_order(self):
        n = getattr(self, "joint_count", 0)
        out = np.zeros(max(n, 1), np.uint32)
        got = ctypes.c_int32(0)
        self._check(self._lib.b2g_get_joint_order(self._h, out.ctypes.data_as(ctypes.c_void_p), len(out),
                                                  ctypes.byref(got)))
        return out[: got.value]

    def save_state(self):
        """The world's exact state (b2g_state_save) as a uint8 array."""
        n = ctypes.c_uint64(0)
        self._check(self._lib.b2g_state_size(self._h, ctypes.byref(n)))
        out = np.empty(n.value, np.uint8)
        self._check(self._lib.b2g_state_save(self._h, out.ctypes.data_as(ctypes.c_void_p), n.value))
        return out

    def load_state(self, state):
        """Continue from a state of save_state (this world, or one built the same way)."""
        state = np.ascontiguousarray(state, np.uint8)
        self._check(self._lib.b2g_state_load(self._h, state.ctypes.data_as(ctypes.c_void_p), len(state)))

    def set_toi_schedule(self, schedule):
        """TOI_SIDE_BY_SIDE (default), TOI_ONE_AT_A_TIME or TOI_RESTART_ON_ADVANCE."""
        self._check(self._lib.b2g_set_toi_schedule(self._h, int(schedule)))

    def _get_list(self, fn, dtype, cap_hint, width=1):
        n = ctypes.c_int32(0)
        cap = max(cap_hint, 1)
        while True:
            out = np.zeros(cap * width, dtype)
            self._check(fn(self._h, _ptr(out), cap, ctypes.byref(n)))
            if n.value <= cap:
                return out[: n.value * width]
            cap = n.value

    def get_contacts(self):
        return self._get_list(self._lib.b2g_get_contacts, CONTACT_INFO, 4096)

    def get_events(self):
        return self._get_list(self._lib.b2g_get_events, EVENT, 1024)

    def get_pairs(self):
        return self._get_list(self._lib.b2g_get_pairs, np.uint32, 65536, 2).reshape(-1, 2)

    def get_solver_order(self):
        return self._get_list(self._lib.b2g_get_solver_order, np.uint32, 65536, 2).reshape(-1, 2)

    # ---- world queries (B2world::ray_cast / query_aabb) ----
    def ray_cast_closest(self, rays, world_index=None):
        """Closest hit per ray; rays (n, 4) = p1.x, p1.y, p2.x, p2.y. Returns a RAY_HIT array."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 4)
        wi = None if world_index is None else np.ascontiguousarray(world_index, np.uint32)
        out = np.zeros(len(rays), RAY_HIT)
        self._check(self._lib.b2g_ray_cast_closest(self._h, _ptr(rays), None if wi is None else _ptr(wi), len(rays),
                                                   _ptr(out)))
        return out

    def query_aabb(self, boxes, world_index=None):
        """(m, 2) array of (box index, fixture) for every fat AABB overlapping each box."""
        boxes = np.ascontiguousarray(boxes, np.float32).reshape(-1, 4)
        wi = None if world_index is None else np.ascontiguousarray(world_index, np.uint32)
        n = ctypes.c_int32(0)
        cap = max(64, 16 * len(boxes))
        while True:
            out = np.zeros((cap, 2), np.uint32)
            rc = self._lib.b2g_query_aabb(self._h, _ptr(boxes), None if wi is None else _ptr(wi), len(boxes),
                                          _ptr(out), cap, ctypes.byref(n))
            if rc == -3 and n.value > cap:
                cap = n.value
                continue
            self._check(rc)
            return out[: n.value]

    # ---- launch configuration ----
    def get_launch_config(self):
        c = LaunchConfig()
        self._check(self._lib.b2g_get_launch_config(self._h, ctypes.byref(c)))
        return c.as_dict()

    def set_launch_config(self, coop_blocks_per_sm=1, collide_block=128, traverse_block=256, solver_block=256,
                          collide_group=0):
        c = LaunchConfig(coop_blocks_per_sm, collide_block, traverse_block, 0, solver_block, collide_group)
        self._check(self._lib.b2g_set_launch_config(self._h, ctypes.byref(c)))

    def autotune(self, dt, velocity_iterations, position_iterations, steps_per_candidate=4):
        """Pick the fastest launch configuration on the world's next steps (they are real steps)."""
        c = LaunchConfig()
        self._check(self._lib.b2g_autotune(self._h, dt, velocity_iterations, position_iterations,
                                           steps_per_candidate, ctypes.byref(c)))
        return c.as_dict()

    def tuning_steps(self):
        """Steps the last autotune() ran on this world."""
        c = LaunchConfig()
        self._check(self._lib.b2g_get_launch_config(self._h, ctypes.byref(c)))
        return int(c.tuning_steps)

    # ---- differentiable step ----
    def tape_begin(self, max_steps, checkpoint_interval=16, max_slots=0):
        """Record the next steps for backward() (sleeping must be off)."""
        self._check(self._lib.b2g_tape_begin(self._h, int(max_steps), int(checkpoint_interval), int(max_slots)))

    def tape_end(self):
        self._check(self._lib.b2g_tape_end(self._h))

    def tape_info(self):
        t = TapeInfo()
        self._check(self._lib.b2g_tape_info_get(self._h, ctypes.byref(t)))
        return t.as_dict()

    def backward(self, d_final):
        """dL/d(initial state) from dL/d(final state), both BODY_STATE arrays over all bodies."""
        d_final = np.ascontiguousarray(d_final, dtype=BODY_STATE)
        if d_final.shape != (self.body_count,):
            raise ValueError("d_final must hold one BODY_STATE per body")
        out = np.zeros(self.body_count, BODY_STATE)
        self._check(self._lib.b2g_backward(self._h, _ptr(d_final), _ptr(out)))
        return out

    def tape_step(self, step):
        """(step parameters, colour offsets, slots) of one taped step."""
        info = np.zeros(1, TAPE_STEP)
        self._check(self._lib.b2g_tape_get_step(self._h, int(step), _ptr(info), None, None, 0))
        ns, nc = int(info["num_slots"][0]), int(info["num_colours"][0])
        col = np.zeros(nc + 1, np.int32)
        slots = np.zeros(max(ns, 1), TAPE_SLOT)
        self._check(self._lib.b2g_tape_get_step(self._h, int(step), _ptr(info), _ptr(col), _ptr(slots), ns))
        return info[0], col, slots[:ns]

    def tape_checkpoint(self, index):
        """(n, 8) float32: centre x, y, angle, -, vx, vy, w, - per body; index -1 is the final state."""
        out = np.zeros((self.body_count, 8), np.float32)
        self._check(self._lib.b2g_tape_get_checkpoint(self._h, int(index), _ptr(out), self.body_count))
        return out

    def set_contact_filter(self, fn):
        """fn(fixture_a, fixture_b) -> bool replaces the default contact filter (None restores it)."""
        self._filter_cb = None if fn is None else contact_filter_callback(fn)
        ptr = None if fn is None else ctypes.cast(self._filter_cb, ctypes.c_void_p)
        self._check(self._lib.b2g_set_contact_filter(self._h, ptr, None))

    def set_pre_solve(self, fn):
        """fn(contact, old_manifold, edit) is called after collide for every updated touching contact."""
        self._pre_solve_cb = None if fn is None else pre_solve_callback(fn)
        ptr = None if fn is None else ctypes.cast(self._pre_solve_cb, ctypes.c_void_p)
        self._check(self._lib.b2g_set_pre_solve(self._h, ptr, None))

    def get_post_solve(self):
        """The last step's post_solve reports (b2g_get_post_solve), as a CONTACT_IMPULSE array."""
        n = ctypes.c_int32(0)
        self._check(self._lib.b2g_get_post_solve(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(max(n.value, 1), CONTACT_IMPULSE)
        self._check(self._lib.b2g_get_post_solve(self._h, _ptr(out), n.value, ctypes.byref(n)))
        return out[: n.value]

    def get_proxy_ids(self):
        """Each fixture's proxy id (the reference's dynamic-tree leaf id), -1 without a proxy."""
        out = np.zeros(max(self.fixture_count, 1), np.int32)
        self._check(self._lib.b2g_get_proxy_ids(self._h, _ptr(out), self.fixture_count))
        return out[: self.fixture_count]

    # -- destruction and filtering (B2world::destroy_body / destroy_joint, B2body::destroy_fixture,
    #    B2fixture::set_filter_data / refilter) --
    def destroy_bodies(self, ids):
        ids = np.ascontiguousarray(np.atleast_1d(ids), np.uint32)
        self._check(self._lib.b2g_destroy_bodies(self._h, _ptr(ids), len(ids)))

    def destroy_fixtures(self, ids):
        ids = np.ascontiguousarray(np.atleast_1d(ids), np.uint32)
        self._check(self._lib.b2g_destroy_fixtures(self._h, _ptr(ids), len(ids)))

    def destroy_joints(self, ids):
        ids = np.ascontiguousarray(np.atleast_1d(ids), np.uint32)
        self._check(self._lib.b2g_destroy_joints(self._h, _ptr(ids), len(ids)))

    def set_filter_data(self, fixture, category_bits, mask_bits, group_index):
        self._check(self._lib.b2g_set_filter_data(self._h, int(fixture), int(category_bits), int(mask_bits),
                                                  int(group_index)))

    def refilter(self, fixture):
        self._check(self._lib.b2g_refilter(self._h, int(fixture)))

    def get_proxies(self):
        n = self.fixture_count
        aabbs = np.zeros((n, 4), np.float32)
        moved = np.zeros(n, np.uint8)
        self._check(self._lib.b2g_get_proxies(self._h, _ptr(aabbs), _ptr(moved), n))
        return aabbs, moved
