/*
 * b2g.h — C ABI of the GB300-native Box2D world step (libb2g.so).
 *
 * This header is the drop-in boundary for box2d-rs 0.0.4's `B2world` step path.
 * The reference has no FFI of its own; its seam is the public Rust `B2world`
 * API, and each entry point below names the reference function it replaces
 * (paths are inside the box2d-rs source tree).
 *
 * Conventions
 *   - Every function returns an int status: B2G_OK (0) or a negative B2G_ERR_*.
 *     The reference panics on misuse (src/private/dynamics/b2_world.rs:84-87);
 *     here misuse returns B2G_ERR_INVALID_ARG / B2G_ERR_LOCKED and
 *     b2g_last_error() holds a one-line reason.
 *   - The library owns all device memory. The caller owns every host buffer
 *     passed in or out. Ids are dense uint32 in creation order.
 *   - One world (or batch of worlds) per host thread; the library starts no
 *     threads. Each world has its own CUDA stream; b2g_step is asynchronous
 *     and b2g_synchronize / any b2g_get_* call waits for it.
 *   - Listener callbacks are never called from device code: begin/end contact
 *     events are buffered on the device and read with b2g_get_events after a
 *     step (the reference fires them inside `step`,
 *     src/private/dynamics/b2_contact.rs:201-217).
 *   - Arithmetic is IEEE f32 with no fused multiply-add, like the reference.
 */
#ifndef B2G_H
#define B2G_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define B2G_OK 0
#define B2G_ERR_INVALID_ARG (-1)
#define B2G_ERR_OUT_OF_MEMORY (-2)
#define B2G_ERR_CAPACITY (-3)     /* a device buffer overflowed; results of that step are void */
#define B2G_ERR_TIMEOUT (-4)      /* a bounded device wait gave up (grid barrier)               */
#define B2G_ERR_CUDA (-5)         /* a CUDA runtime call failed                                  */
#define B2G_ERR_UNSUPPORTED (-6)  /* feature outside the GPU path (see b2g_last_error)           */
#define B2G_ERR_LOCKED (-7)       /* world is inside a step                                      */

#define B2G_MAX_POLYGON_VERTICES 8

/* B2bodyType, src/b2_body.rs:20-30 */
enum { B2G_STATIC_BODY = 0, B2G_KINEMATIC_BODY = 1, B2G_DYNAMIC_BODY = 2 };
/* B2ShapeType order, src/b2_shape.rs:25-31 (chain shapes are not supported) */
enum { B2G_SHAPE_CIRCLE = 0, B2G_SHAPE_EDGE = 1, B2G_SHAPE_POLYGON = 2 };
/* How a polygon is built: B2polygonShape::set (hull, private/collision/b2_polygon_shape.rs:96-211),
 * set_as_box (:12-23) or set_as_box_angle (:25-50). */
enum { B2G_POLYGON_HULL = 0, B2G_POLYGON_BOX = 1, B2G_POLYGON_BOX_ORIENTED = 2 };

typedef struct b2g_vec2 { float x, y; } b2g_vec2;

typedef struct b2g_world_def {
    b2g_vec2 gravity;          /* B2world::new(gravity), src/b2_world.rs:25-27 */
    int32_t num_worlds;        /* >= 1. Bodies carry world_index; worlds never interact. */
    int32_t device;            /* CUDA device ordinal */
    int32_t body_capacity;     /* 0 = grow on demand at creation time */
    int32_t fixture_capacity;
    int32_t contact_capacity;  /* 0 = 8 x fixtures */
    int32_t pair_capacity;     /* 0 = 16 x fixtures */
} b2g_world_def;

/* B2bodyDef, src/b2_body.rs:91-147 (defaults :39-59) */
typedef struct b2g_body_def {
    int32_t type;
    b2g_vec2 position;
    float angle;
    b2g_vec2 linear_velocity;
    float angular_velocity;
    float linear_damping;
    float angular_damping;
    float gravity_scale;
    uint8_t allow_sleep;
    uint8_t awake;
    uint8_t fixed_rotation;
    uint8_t bullet;
    uint8_t enabled;
    uint8_t pad_[3];
    uint32_t world_index;      /* which world of a batch (0 for a single world) */
    uint64_t user_data;
} b2g_body_def;

/* B2fixtureDef (src/b2_fixture.rs:44-56) with its shape inlined.
 *   circle : vertices[0] = centre (m_p), radius
 *   edge   : vertices[0..3] = vertex0..vertex3, one_sided selects set_one_sided/set_two_sided
 *   polygon: polygon_mode HULL uses vertices[0..vertex_count); BOX/BOX_ORIENTED use box_* fields
 *   radius for polygons and edges is the skin radius (B2_POLYGON_RADIUS = 0.01 by default) */
typedef struct b2g_fixture_def {
    uint32_t body;
    int32_t shape_type;
    int32_t polygon_mode;
    int32_t vertex_count;
    b2g_vec2 vertices[B2G_MAX_POLYGON_VERTICES];
    float radius;
    b2g_vec2 box_half_extents;
    b2g_vec2 box_center;
    float box_angle;
    int32_t one_sided;
    float friction;
    float restitution;
    float restitution_threshold;
    float density;
    int32_t is_sensor;
    uint16_t category_bits;
    uint16_t mask_bits;
    int16_t group_index;
    int16_t pad_;
    uint64_t user_data;
} b2g_fixture_def;

/* A joint definition: the B2jointDef base (bodies, collide_connected) and the fields of its type.
 * Anchors are in the bodies' local frames.
 *   B2G_JOINT_REVOLUTE: B2revoluteJointDef (src/joints/b2_revolute_joint.rs:10-72): reference angle,
 *     limit (enable_limit, lower/upper angle), motor (enable_motor, speed, max torque)
 *   B2G_JOINT_DISTANCE: B2distanceJointDef (src/joints/b2_distance_joint.rs): rest length, min and
 *     max length, stiffness and damping (a spring when stiffness > 0 and min < max)
 *   B2G_JOINT_WELD: B2weldJointDef (src/joints/b2_weld_joint.rs): reference angle, stiffness and
 *     damping (an angular spring when stiffness > 0)
 *   B2G_JOINT_FRICTION: B2frictionJointDef (src/joints/b2_friction_joint.rs): max force, max torque
 *   B2G_JOINT_MOTOR: B2motorJointDef (src/joints/b2_motor_joint.rs): linear offset (in body A's frame),
 *     angular offset, max force, max torque, correction factor (the anchors are not used)
 *   B2G_JOINT_MOUSE: B2mouseJointDef (src/joints/b2_mouse_joint.rs): a world target that body B's point
 *     under it at creation is pulled to by a soft constraint (max force, stiffness, damping); body A only
 *     ties the joint into the world (usually a static body)
 *   B2G_JOINT_PRISMATIC: B2prismaticJointDef (src/joints/b2_prismatic_joint.rs): local axis in body A
 *     (normalized at creation), reference angle, limit (enable_limit, lower/upper translation), motor
 *     (enable_motor, motor_speed, max_motor_force)
 *   B2G_JOINT_WHEEL: B2wheelJointDef (src/joints/b2_wheel_joint.rs): local axis in body A (used as given),
 *     suspension spring (stiffness, damping), limit (lower/upper translation), motor (speed, max torque)
 *   B2G_JOINT_PULLEY: B2pulleyJointDef (src/joints/b2_pulley_joint.rs): ground anchors (world), rope
 *     lengths at rest, ratio (length_a + ratio * length_b stays constant)
 * The type numbers follow Box2D's C++ b2JointType. */
#define B2G_JOINT_REVOLUTE 1
#define B2G_JOINT_DISTANCE 3
#define B2G_JOINT_WELD 8
#define B2G_JOINT_FRICTION 9
#define B2G_JOINT_PRISMATIC 2
#define B2G_JOINT_PULLEY 4
#define B2G_JOINT_MOUSE 5
#define B2G_JOINT_WHEEL 7
#define B2G_JOINT_MOTOR 11
#define B2G_JOINT_GEAR 6
typedef struct b2g_joint_def {
    int32_t type;              /* B2G_JOINT_* */
    uint32_t body_a, body_b;
    int32_t collide_connected;
    b2g_vec2 local_anchor_a, local_anchor_b;
    float reference_angle;
    int32_t enable_limit;
    float lower_angle, upper_angle;
    int32_t enable_motor;
    float motor_speed, max_motor_torque;
    float length, min_length, max_length, stiffness, damping;
    float max_force, max_torque;
    float correction_factor, angular_offset;
    b2g_vec2 linear_offset;
    b2g_vec2 target;
    b2g_vec2 local_axis_a;
    float lower_translation, upper_translation, max_motor_force;
    b2g_vec2 ground_anchor_a, ground_anchor_b;
    float length_a, length_b, ratio;
    /* gear joint (B2gearJointDef, src/joints/b2_gear_joint.rs): the revolute or prismatic joints it
     * couples (ids of joints created earlier); body_a and body_b must be their second bodies; ratio */
    uint32_t joint1, joint2;
} b2g_joint_def;

/* Body state read back after a step (B2body getters, src/b2_body.rs:650-680). */
typedef struct b2g_body_state {
    b2g_vec2 position;         /* m_xf.p  (get_position)        */
    float angle;               /* m_sweep.a (get_angle)         */
    b2g_vec2 linear_velocity;
    float angular_velocity;
    b2g_vec2 world_center;     /* m_sweep.c (get_world_center)  */
} b2g_body_state;

/* B2Profile, src/b2_time_step.rs:5-14; milliseconds measured with CUDA events. */
typedef struct b2g_profile {
    float step, collide, solve, solve_init, solve_velocity, solve_position, broadphase, solve_toi;
} b2g_profile;

typedef struct b2g_counts {
    int32_t bodies, fixtures, proxies, contacts, touching_contacts, islands_solved, colours, pairs;
} b2g_counts;

/* One contact with its manifold (B2manifold, src/b2_collision.rs:104-114). */
typedef struct b2g_contact_info {
    uint32_t fixture_a, fixture_b;  /* after the primary-type ordering of b2_contact_registers.rs */
    int32_t touching;
    int32_t manifold_type;          /* 0 circles, 1 faceA, 2 faceB */
    int32_t point_count;
    b2g_vec2 local_normal;
    b2g_vec2 local_point;
    b2g_vec2 point_local[2];
    float normal_impulse[2];
    float tangent_impulse[2];
    uint32_t point_id[2];           /* B2contactFeature packed: index_a | index_b<<8 | type_a<<16 | type_b<<24 */
    float friction, restitution, restitution_threshold;
} b2g_contact_info;

enum { B2G_EVENT_BEGIN = 0, B2G_EVENT_END = 1 };
typedef struct b2g_contact_event {
    int32_t kind;
    uint32_t fixture_a, fixture_b;
} b2g_contact_event;

/* ---- lifecycle (B2world::new / drop) ---- */
int b2g_world_create(const b2g_world_def* def, void** out_world);
int b2g_world_destroy(void* world);
const char* b2g_last_error(const void* world);
int b2g_version(void);
/* Number of CUDA kernels this library has launched so far (all worlds of the process). */
int64_t b2g_get_launch_count(void);

/* ---- creation: B2world::create_body (src/b2_world.rs:60-62),
 *                B2body::create_fixture (src/b2_body.rs:233) ---- */
int b2g_create_bodies(void* world, const b2g_body_def* defs, int32_t n, uint32_t* out_ids);
int b2g_create_fixtures(void* world, const b2g_fixture_def* defs, int32_t n, uint32_t* out_ids);
/* B2world::create_joint (private/dynamics/b2_world.rs:156-276): every joint type of b2g_joint_def (the ten
 * of B2JointType). A joint that does not let its bodies collide flags their contacts for the next
 * collide, which destroys them. A world with joints runs the grid-wide colour schedule (no
 * part-local solve) and cannot be taped. */
int b2g_create_joints(void* world, const b2g_joint_def* defs, int32_t n, uint32_t* out_ids);

/* ---- destruction and filtering ----
 * Ids stay valid after a destruction: a destroyed body keeps its slot as a static, disabled body
 * without fixtures (its last state stays readable), a destroyed fixture keeps its slot without a
 * proxy, a destroyed joint leaves the solver; none is reused, and any further call that names one
 * returns B2G_ERR_INVALID_ARG. Destroyed proxies return their ids to the dynamic tree's free list
 * exactly as the reference's node pool does (private/collision/b2_dynamic_tree.rs:28-99), so proxy
 * ids, which fixture of a same-type pair is A, and the contact order stay the reference's.
 * End events of contacts a destruction removes are added to the event list of the last step
 * (b2g_get_events); the next step clears the list. Not between b2g_tape_begin and b2g_tape_end. */
/* B2world::destroy_body (src/b2_world.rs:72-74, private/dynamics/b2_world.rs:100-158), for each body
 * in order: its joints (waking their bodies), its contacts (end events, wakes), its fixtures'
 * proxies in fixture-list order. */
int b2g_destroy_bodies(void* world, const uint32_t* ids, int32_t n);
/* B2body::destroy_fixture (src/b2_body.rs:259-261, private/dynamics/b2_body.rs:214-289), for each
 * fixture in order: its contacts, its proxy, then the body's mass data is reset. */
int b2g_destroy_fixtures(void* world, const uint32_t* ids, int32_t n);
/* B2world::destroy_joint (src/b2_world.rs:89-91, private/dynamics/b2_world.rs:278-340): both
 * bodies woken; without collide_connected the contacts between them are flagged for filtering. */
int b2g_destroy_joints(void* world, const uint32_t* ids, int32_t n);
/* B2fixture::set_filter_data (src/b2_fixture.rs:179-181, private/dynamics/b2_fixture.rs:175-211):
 * new filter data, then refilter: the fixture's contacts are flagged for filtering at the next
 * collide and its proxy is touched so the next broadphase queries it. */
int b2g_set_filter_data(void* world, uint32_t fixture, uint16_t category_bits, uint16_t mask_bits,
                        int16_t group_index);
/* B2fixture::refilter (src/b2_fixture.rs:183-189) with the fixture's current filter data. */
int b2g_refilter(void* world, uint32_t fixture);
/* Accumulated joint impulses (for warm starting), 5 per joint: revolute x, y, motor, lower, upper;
 * prismatic x, y, motor, lower, upper; wheel impulse, spring, motor, lower, upper; pulley impulse, 0, 0, 0, 0; distance impulse, lower, upper, 0, 0; weld, friction and motor x, y,
 * angular, 0, 0; mouse x, y, 0, 0, 0 */
int b2g_get_joint_impulses(void* world, uint32_t first, uint32_t count, float* out);
/* B2mouseJoint::set_target (src/joints/b2_mouse_joint.rs:114-119): a new target wakes body B */
int b2g_set_mouse_target(void* world, uint32_t joint, b2g_vec2 target);
/* The order the GPU solves joints in (ids, colour by colour): the oracle's joint ordering hook */
int b2g_get_joint_order(void* world, uint32_t* out, int32_t cap, int32_t* n);

/* ---- the step: B2world::step(dt, velocity_iterations, position_iterations),
 *      src/b2_world.rs:98-100 -> src/private/dynamics/b2_world.rs:903-959 ---- */
int b2g_step(void* world, float dt, int32_t velocity_iterations, int32_t position_iterations);
int b2g_synchronize(void* world);

/* ---- state I/O (src/b2_body.rs getters/setters) ---- */
int b2g_get_body_states(void* world, uint32_t first, uint32_t count, b2g_body_state* out);
/* The same states without waiting (not in the reference: pipelined read-back). A snapshot is
 * taken on the world's stream after the last issued step and copied into `out` on a second
 * stream while the next steps run; at most two requests are in flight (a third waits, on the
 * device, for the first copy). `out` must stay valid and untouched until b2g_wait_body_states
 * returns; it must be host memory the device can write asynchronously: page-locked memory, or
 * any memory on systems with coherent access to pageable memory (Grace). */
int b2g_get_body_states_async(void* world, uint32_t first, uint32_t count, b2g_body_state* out);
/* Wait for the asynchronous copies and the world's stream; reports device-side errors. */
int b2g_wait_body_states(void* world);
/* B2body::get_mass_data / get_local_center: 6 floats per body: mass, 1/mass, rotational inertia
 * about the centre of mass (get_inertia adds mass * |local centre|^2), its inverse, local centre. */
int b2g_get_mass_data(void* world, uint32_t first, uint32_t count, float* out);
/* B2body::set_transform, private/dynamics/b2_body.rs:418-447 */
int b2g_set_transform(void* world, uint32_t body, b2g_vec2 position, float angle);
int b2g_set_linear_velocity(void* world, uint32_t body, b2g_vec2 v);
int b2g_set_angular_velocity(void* world, uint32_t body, float w);
/* B2body::apply_force / apply_linear_impulse (src/b2_body.rs:870-940) */
int b2g_apply_force(void* world, uint32_t body, b2g_vec2 force, b2g_vec2 point, int32_t wake);
int b2g_apply_linear_impulse(void* world, uint32_t body, b2g_vec2 impulse, b2g_vec2 point, int32_t wake);
/* B2body::apply_force_to_center, apply_torque, apply_linear_impulse_to_center, apply_angular_impulse
 * (src/b2_body.rs:890-980) and set_awake (:783-801) */
int b2g_apply_force_to_center(void* world, uint32_t body, b2g_vec2 force, int32_t wake);
int b2g_apply_torque(void* world, uint32_t body, float torque, int32_t wake);
int b2g_apply_linear_impulse_to_center(void* world, uint32_t body, b2g_vec2 impulse, int32_t wake);
int b2g_apply_angular_impulse(void* world, uint32_t body, float impulse, int32_t wake);
int b2g_set_awake(void* world, uint32_t body, int32_t flag);
/* B2body::is_awake (src/b2_body.rs:803-805) of bodies [first, first + count): 1 awake, 0 asleep */
int b2g_get_awake(void* world, uint32_t first, uint32_t count, uint8_t* out);

/* ---- world flags, src/b2_world.rs:163-193, :232-253 ---- */
int b2g_set_gravity(void* world, b2g_vec2 gravity);
int b2g_set_allow_sleeping(void* world, int32_t flag);
int b2g_set_warm_starting(void* world, int32_t flag);
/* Continuous physics (B2world::solve_toi, private/dynamics/b2_world.rs:534-901): after the
 * discrete solve, time-of-impact events against static, kinematic and bullet bodies are solved
 * in order of time. Off by default in this ABI (the reference's B2world starts with it on: a
 * wrapper mirroring B2world::new sets it); not recorded by the tape (b2g_step fails while a tape
 * records with it on). */
int b2g_set_continuous_physics(void* world, int32_t flag);
/* How the continuous pass orders its time-of-impact events (not in the reference: a schedule).
 * Side by side (default): the earliest events of bodies that touch only static bodies are solved
 * together, the others one at a time; a pass whose side-by-side events would advance one body's
 * sweep to two different times restarts one event at a time. One at a time: every event alone, in
 * the reference's order. Restart on advance: side by side, but the first sweep advance restarts the
 * pass (exercises the restart). Bodies and manifolds are the same under all three. */
#define B2G_TOI_SCHEDULE_SIDE_BY_SIDE 0
#define B2G_TOI_SCHEDULE_ONE_AT_A_TIME 1
#define B2G_TOI_SCHEDULE_RESTART_ON_ADVANCE 2
int b2g_set_toi_schedule(void* world, int32_t schedule);
int b2g_set_auto_clear_forces(void* world, int32_t flag);
int b2g_clear_forces(void* world);
/* Part-local solve (default on; not in the reference: a solver schedule). Each solver block owns a
 * part of the constraint bodies (equal-work ranges in Morton order) and solves the constraints
 * inside it from shared memory; the constraints between parts follow in grid-wide colours. It
 * applies to worlds of up to 2048 proxies per SM. The solve order, and so the bits of the
 * results, then depend on the GPU's SM count; with the flag off every constraint is solved in
 * grid-wide colours, whose order does not. Both orders are exported by b2g_get_solver_order. */
int b2g_set_part_solve(void* world, int32_t flag);

/* ---- introspection ---- */
int b2g_get_profile(void* world, b2g_profile* out);       /* B2world::get_profile, src/b2_world.rs:268-270 */
int b2g_get_counts(void* world, b2g_counts* out);         /* get_body_count / get_contact_count / get_proxy_count */
/* Work counts of the last step, for traffic models of its kernels (not in the reference, whose
 * B2Profile holds times only): hierarchy nodes the broadphase traversal fetched and leaves it
 * checked, new contacts it found, the contact table's size, constraint slots solved (of them
 * part-locally), the parts and colours of the colouring; the contact and pair capacities and how
 * often they grew (b2g_set_auto_grow); the broadphase hierarchy's age (0: the last pass rebuilt it; else
 * the passes since, which kept it and updated the moved proxies' leaves in place), the proxies the
 * step's solver moved (the traversal's queries), and the most node fetches and leaf checks one warp
 * of the traversal made (its load balance). */
typedef struct b2g_step_stats {
    int32_t bp_node_visits, bp_leaf_checks, new_pairs, contacts;
    int32_t constraints, interior_slots, parts, colours;
    int32_t contact_capacity, pair_capacity, capacity_grows, hierarchy_age;
    int32_t bp_moved_proxies, bp_warp_max_visits, bp_warp_max_checks;
} b2g_step_stats;
int b2g_get_step_stats(void* world, b2g_step_stats* out);
/* Exact checkpoint and resume (not in the reference's API, which serialises a world through serde,
 * src/serialize/): the world's device buffers (bodies, fixtures, the contact table with its
 * manifolds and impulses, the colouring and partition the next steps reuse) and its stepping state,
 * written to caller memory of b2g_state_size bytes. A world loaded from it continues bit for bit
 * like the saved one: load into the same world, or one built with the same world definition, bodies
 * and fixtures (B2G_ERR_INVALID_ARG otherwise). Not while a tape records. */
int b2g_state_size(void* world, uint64_t* bytes);
int b2g_state_save(void* world, void* out, uint64_t bytes);
int b2g_state_load(void* world, const void* in, uint64_t bytes);

/* Continuous physics: solid time-of-impact events solved since the world was made, the
 * iterations of the last step's pass, and the passes restarted one event at a time. */
int b2g_get_toi_stats(void* world, int32_t* events, int32_t* last_iterations, int32_t* restarts);
/* Device times (ms, CUDA events) of the last step's phases, n >= 7: initial broadphase (only
 * after fixtures were added), collide, islands + constraint list, colouring, solver kernel,
 * broadphase tree pass (keys, sort, hierarchy, traversal), contact merge (with the continuous
 * pass when it runs); with n >= 10 also the tree pass in three: keys + sort, hierarchy (build,
 * refit, four-way records, contact rows), traversal. */
int b2g_get_phase_times(void* world, float* out, int32_t n);
int b2g_get_contacts(void* world, b2g_contact_info* out, int32_t capacity, int32_t* out_count);
/* begin/end events produced since the previous call (B2contactListener, src/b2_world_callbacks.rs:68-104) */
int b2g_get_events(void* world, b2g_contact_event* out, int32_t capacity, int32_t* out_count);
/* B2contactImpulse (src/b2_world_callbacks.rs:52-58) of one contact, as B2contactListener::post_solve
 * receives it. */
typedef struct b2g_contact_impulse {
    uint32_t fixture_a, fixture_b;
    float normal_impulses[2];
    float tangent_impulses[2];
    int32_t count;                  /* points as solved: a 2-point manifold solved as 1 reports 1 */
} b2g_contact_impulse;
/* The post_solve reports of the last step (B2island::report, private/dynamics/b2_island_private.rs:
 * 460-487): one per contact of the islands the discrete solve solved, in solve order, with the
 * impulses after the velocity iterations. The reference calls post_solve only when a listener is
 * set; here the records are always kept on the device and read on demand. The time-of-impact
 * sub-steps of continuous physics are not reported. */
int b2g_get_post_solve(void* world, b2g_contact_impulse* out, int32_t capacity, int32_t* out_count);

/* ---- host callbacks (a slow path: the world's steps run without graphs and synchronise at each
 * callback point; not with continuous physics, whose pass runs on the device alone) ----
 * B2world::set_contact_filter (src/b2_world.rs:38-40) with a B2contactFilter::should_collide
 * (src/b2_world_callbacks.rs:33-45) written on the host: it replaces the default filter. It is asked
 * about every new pair the broadphase finds (with the fixtures of the smaller and the larger proxy
 * id, after add_pair's body and joint checks), and about every contact flagged for filtering (a
 * destroyed joint, new filter data) whose bodies still may collide, before collide; nonzero keeps the
 * pair. fn = NULL restores the default filter. */
typedef int32_t (*b2g_contact_filter_fn)(void* user, uint32_t fixture_a, uint32_t fixture_b);
int b2g_set_contact_filter(void* world, b2g_contact_filter_fn fn, void* user);
/* B2contactListener::pre_solve (src/b2_world_callbacks.rs:68-104; called from
 * private/dynamics/b2_contact.rs:201-217): after collide, once for every contact the step updated that
 * touches, in the contact table's key order, with the new manifold and the manifold before the update.
 * The callback may edit the contact for this step's solve as B2contact's setters do: set_enabled,
 * set_friction, set_restitution, set_restitution_threshold, set_tangent_speed (friction and
 * restitution persist, as in the reference; enabled is set again by the next update). */
typedef struct b2g_contact_edit {
    int32_t enabled;
    float friction, restitution, restitution_threshold, tangent_speed;
} b2g_contact_edit;
typedef void (*b2g_pre_solve_fn)(void* user, const b2g_contact_info* contact, const b2g_contact_info* old_manifold,
                                 b2g_contact_edit* edit);
int b2g_set_pre_solve(void* world, b2g_pre_solve_fn fn, void* user);

/* Buffer begin/end contact events during steps (off by default: the reference only
 * calls a listener once one is installed, src/b2_world.rs:44-46). */
int b2g_set_contact_events(void* world, int32_t flag);

/* Manifolds of n independent shape pairs evaluated on the GPU, like the reference's public
 * b2_collide_circles / polygon_and_circle / polygons / edge_and_circle / edge_and_polygon
 * (src/b2_collision.rs:259-315). Shape A must be the routine's first type (circle-circle,
 * polygon-circle, polygon-polygon, edge-circle, edge-polygon); xf_a/xf_b hold (x, y, angle)
 * per pair. Fills fixture_a = fixture_b = pair index and the manifold fields of out[i]. */
int b2g_collide_pairs(const b2g_fixture_def* shape_a, const float* xf_a, const b2g_fixture_def* shape_b,
                      const float* xf_b, int32_t n, b2g_contact_info* out);

/* Time of impact of n independent pairs of moving shapes on the GPU (the routine the step's
 * continuous pass runs per contact), like the reference's public b2_time_of_impact
 * (src/b2_time_of_impact.rs:48-50, private/collision/b2_time_of_impact.rs:191-463) with its GJK
 * distance (private/collision/b2_distance.rs:331-440). A sweep is a body's motion over the
 * interval (B2Sweep, src/b2_math.rs): local centre of mass, centre and angle at the start
 * (c0, a0) and at the end (c, a); alpha0 is carried for the caller and not read. t_max: per pair
 * (NULL: 1). Shapes are circles, polygons or edges. out[i] is the state (B2G_TOI_*) and the time
 * in [0, t_max]. */
enum { B2G_TOI_UNKNOWN = 0, B2G_TOI_FAILED = 1, B2G_TOI_OVERLAPPED = 2, B2G_TOI_TOUCHING = 3, B2G_TOI_SEPARATED = 4 };
typedef struct b2g_sweep {
    b2g_vec2 local_center;
    b2g_vec2 c0, c;
    float a0, a;
    float alpha0;
    float pad;
} b2g_sweep;
typedef struct b2g_toi_output {
    int32_t state;
    float t;
} b2g_toi_output;
int b2g_time_of_impact(const b2g_fixture_def* shape_a, const b2g_sweep* sweep_a, const b2g_fixture_def* shape_b,
                       const b2g_sweep* sweep_b, const float* t_max, int32_t n, b2g_toi_output* out);

/* Run steady-state steps as captured CUDA graphs (on by default). A step is captured once
 * per contact-buffer parity and replayed while dt, iterations, flags, gravity and the body
 * and fixture counts stay the same; any change re-captures. */
int b2g_set_graph_capture(void* world, int32_t flag);

/* Grid-barrier wait limit of the world's persistent kernels, in SM clock cycles (0 restores
 * the default of 2e9 cycles, about 1 s at 2 GHz; the value is rounded down to a multiple of
 * 1024). A wait that runs out sets the device status: the step's results are void, the next
 * status check returns B2G_ERR_TIMEOUT and clears it, and the world can be restored with
 * b2g_state_load. The reference has no device waits (it panics or loops on the host). */
int b2g_set_barrier_limit(void* world, int64_t cycles);
/* Automatic growth of the contact and pair capacities (off by default; not with continuous physics or
 * a host contact filter). When a step's broadphase finds more new pairs, or merges more contacts, than
 * the capacities hold, b2g_step drains the world's stream, doubles the capacity (keeping every device
 * buffer's contents) and repeats that pass with every proxy queried, which yields the same contacts;
 * the world then continues bit for bit as one created with the larger capacities. The reference grows
 * its containers on the host as needed; here each step with it on waits for the device once. */
int b2g_set_auto_grow(void* world, int32_t flag);
/* The broadphase keeps its hierarchy between passes and updates only the moved proxies' leaves (their
 * ancestors' boxes grow to cover them); it rebuilds when proxies were created, destroyed or edited on
 * the host, when many proxies moved, or when the hierarchy is `passes` passes old (default 16; 0
 * rebuilds every pass). The pairs found never depend on it (the reference's dynamic tree is likewise
 * updated per moved proxy, b2_dynamic_tree.rs:109-168); with the part-local solve the solve order
 * follows the hierarchy's Morton order, so the result bits do (b2g_get_solver_order exports it). */
int b2g_set_hierarchy_max_age(void* world, int32_t passes);
/* Test hook for the timeout path: every grid barrier of the world's kernels also waits for
 * `extra` arrivals that never come, so each wait runs out its limit (0 turns it off). */
int b2g_debug_hold_barriers(void* world, int32_t extra);

/* The same stand-alone manifolds as b2g_collide_pairs, for callers that must not allocate
 * memory: a frame loop with a fixed time budget (freeing device memory can wait for the whole
 * device) or a host program whose device memory is owned by its own pool allocator. It calls
 * no cudaMalloc/cudaFree and no host heap allocation; its staging buffers are fixed arrays
 * inside the library, sized for at most B2G_NOALLOC_MAX_PAIRS pairs (about 6 MB of device
 * memory that every GPU using the library keeps until the process exits).
 *   - n > B2G_NOALLOC_MAX_PAIRS returns B2G_ERR_CAPACITY and does nothing.
 *   - The first call on a device looks up the device address of the scratch array; make
 *     that first call before any stream capture.
 *   - All calls share the one scratch array. The function holds a process-wide lock and
 *     returns only after its results are copied back, because two calls running on the GPU
 *     at the same time would overwrite each other's data.
 *   - It copies and launches on the legacy default stream of the current device. On entry it
 *     clears a CUDA error left pending on the calling thread by an earlier call; after a failed
 *     call it looks the scratch address up again (for example after a device reset).
 * It has no counterpart in the reference. */
#define B2G_NOALLOC_MAX_PAIRS 16384
int b2g_collide_pairs_noalloc(const b2g_fixture_def* shape_a, const float* xf_a, const b2g_fixture_def* shape_b,
                              const float* xf_b, int32_t n, b2g_contact_info* out);

/* ---- differentiable step: a recorded tape and its hand-written adjoint ----
 * The model differentiated is the solver of every taped step (B2island::solve,
 * private/dynamics/b2_island_private.rs:129-328, with B2contactSolver,
 * private/dynamics/b2_contact_solver_private.rs) with its discrete decisions frozen from the
 * forward pass: the contact set and each manifold in local coordinates, the colour order,
 * restitution triggers, friction-cone and normal clamp states, the 2-point block-solver case,
 * translation/rotation clamps, position-correction clamps and each island's position-iteration
 * count. Velocity integration, constraint initialisation (world manifold from the poses),
 * warm starting with impulses carried between steps, velocity iterations, position
 * integration and position iterations are differentiated exactly. It has no counterpart in
 * the reference. */
typedef struct b2g_tape_slot {           /* one solver constraint of one taped step (144 bytes) */
    int32_t body_a, body_b;
    int32_t count_type_flags;            /* point count | manifold type << 8 | dynamic A/B << 16 */
    int32_t colour;                      /* its boundary colour (0 for a part's interior slot); the
                                            solve order is the slot order */
    float local_normal[2], local_point[2];
    float points[4];                     /* manifold points (local) */
    float inv_mass_a, inv_mass_b, inv_inertia_a, inv_inertia_b;
    float local_center_a[2], local_center_b[2];
    float friction, restitution, restitution_threshold, tangent_speed;
    float radius_a, radius_b;
    int32_t island;                      /* island root body */
    int32_t position_iterations;         /* position iterations this slot's island ran */
    float impulses[4];                   /* normal 0, tangent 0, normal 1, tangent 1 as carried in */
    int32_t carry[2];                    /* previous step's slot * 2 + point each impulse came from, or -1 */
    uint32_t ids[2];                     /* contact feature ids */
} b2g_tape_slot;

typedef struct b2g_tape_step {           /* 48 bytes */
    float dt, dt_ratio, gravity_x, gravity_y;
    int32_t velocity_iterations, position_iterations, warm_starting, num_slots;
    int64_t slot_offset;
    int32_t num_colours, num_contacts;
} b2g_tape_step;

typedef struct b2g_tape_info {
    int32_t recording;                   /* 1 between b2g_tape_begin and b2g_tape_end */
    int32_t steps;                       /* taped steps (steps with dt > 0) */
    int64_t slots;                       /* constraint slots over all taped steps */
    int32_t checkpoint_interval;
    int32_t valid;                       /* 0 once an edit between steps or an overflow broke it */
    int64_t device_bytes;                /* tape plus backward work buffers */
    uint32_t replay_mismatches;          /* bodies whose replayed state differed from the recorded one
                                            in the last b2g_backward (0 expected) */
    int32_t pad;
} b2g_tape_info;

/* Start recording the next steps (up to max_steps; max_slots constraint slots in total, <= 0
 * picks max_steps x (4 x fixtures + 1024)); body state is checkpointed every
 * checkpoint_interval steps (<= 0: 16). Needs sleeping off. Editing bodies between taped steps
 * (transforms, velocities, forces, impulses, new bodies or fixtures) invalidates the tape and
 * b2g_backward then fails; gravity, iterations, dt and warm starting may change per step. */
int b2g_tape_begin(void* world, int32_t max_steps, int32_t checkpoint_interval, int64_t max_slots);
/* Stop recording and checkpoint the final state. */
int b2g_tape_end(void* world);
int b2g_tape_info_get(void* world, b2g_tape_info* out);
/* Reverse pass over the whole tape. d_final: dL/d(state after the last taped step) per body,
 * in b2g_body_state layout (position, angle, linear and angular velocity, world centre; the
 * position and world-centre terms add up). d_initial receives dL/d(state before the first
 * taped step) in the same layout: position = dL/d(body origin) with the angle held,
 * angle = dL/d(angle) with the origin held, world_center = dL/d(centre of mass) with the angle
 * held. Either pointer covers all bodies. */
int b2g_backward(void* world, const b2g_body_state* d_final, b2g_body_state* d_initial);
/* Copy one taped step out: its parameters, colour offsets (num_colours + 1 ints) and slots. The
 * offsets list the step's solve order as groups of independent slots, in order: with the
 * part-local solve, every part's interior colours, then the boundary colours. Call it first with
 * out_colour_offsets = NULL to learn num_colours. */
int b2g_tape_get_step(void* world, int32_t step, b2g_tape_step* out_step, int32_t* out_colour_offsets,
                      b2g_tape_slot* out_slots, int32_t slot_capacity);
/* Body solver state (centre x, y, angle, -, vx, vy, w, - per body) of checkpoint `index`
 * (state before step index x interval), or after the last taped step for index = -1. */
int b2g_tape_get_checkpoint(void* world, int32_t index, float* out, uint32_t count);

/* ---- world queries: B2world::query_aabb / ray_cast (private/dynamics/b2_world.rs:969-1056),
 *      many per call, on the hierarchy of the last step's broadphase (fat AABBs as of that step;
 *      the world must have stepped once) ---- */
typedef struct b2g_ray_hit {
    int32_t fixture;            /* -1: no hit */
    b2g_vec2 point;             /* (1 - fraction) * p1 + fraction * p2 */
    b2g_vec2 normal;
    float fraction;
} b2g_ray_hit;
/* Closest hit of each ray p1 -> p2 (rays: n x (p1.x, p1.y, p2.x, p2.y)), i.e. the result of the
 * reference's ray cast with a callback that returns the reported fraction (clipping the ray).
 * world_index: per ray, which world of a batch (NULL: world 0). Among hits at exactly the same
 * fraction the GPU reports the first its hierarchy meets, which can differ from the reference. */
int b2g_ray_cast_closest(void* world, const float* rays, const uint32_t* world_index, int32_t n, b2g_ray_hit* out);
/* Fixtures whose fat AABB overlaps each box (boxes: n x (lower.x, lower.y, upper.x, upper.y)), as
 * (box index, fixture) pairs sorted by box then fixture (the reference reports the same set per
 * box through its query callback, in tree order). *out_count = total pairs; at most capacity are
 * written (B2G_ERR_CAPACITY if more exist). */
int b2g_query_aabb(void* world, const float* boxes, const uint32_t* world_index, int32_t n, uint32_t* out_pairs,
                   int32_t capacity, int32_t* out_count);

/* ---- launch configuration and autotuner (no counterpart in the reference) ----
 * How the step's kernels are launched; results are bit-identical for every configuration. */
typedef struct b2g_launch_config {
    int32_t coop_blocks_per_sm;   /* persistent colouring/solver kernels: 1 or 2 blocks per SM */
    int32_t collide_block;        /* narrowphase threads per block: 32..256, power of two */
    int32_t traverse_block;       /* broadphase traversal threads per block: 32..256, power of two */
    int32_t tuning_steps;         /* out: steps the world's last b2g_autotune ran (ignored on set) */
    int32_t solver_block;         /* solver threads per block: 256, or 512 with one block per SM (more
                                     loads in flight on large worlds and batches); 0 on set: 256 */
    int32_t collide_group;        /* narrowphase pairs per warp: a warp's batch of 32 contacts with at
                                     most this many polygon pairs evaluates each of them on 8 lanes (4
                                     pairs at a time); more, one lane per pair. 0..32, default 0 */
} b2g_launch_config;
int b2g_get_launch_config(void* world, b2g_launch_config* out);
int b2g_set_launch_config(void* world, const b2g_launch_config* config);
/* Time the world's next steps under candidate configurations (one knob at a time: blocks per SM,
 * narrowphase block, traversal block, solver block, narrowphase pairs per warp (collide_group 0, 8 or
 * 32); each candidate 2 untimed steps and its share of steps_per_candidate timed steps),
 * keep the fastest for this world and for later worlds of the same size bucket (log2 bodies per
 * world, single or batch) created in this process. The tuning steps are ordinary steps of the
 * world with the given dt and iterations. */
int b2g_autotune(void* world, float dt, int32_t velocity_iterations, int32_t position_iterations,
                 int32_t steps_per_candidate, b2g_launch_config* out);

/* ---- parity hooks ---- */
/* Record every pair the broadphase emits (off by default; needed by b2g_get_pairs). */
int b2g_set_record_pairs(void* world, int32_t flag);
/* Pairs emitted by the last broadphase pass (update_pairs, src/b2_broad_phase.rs:200-249),
 * as fixture-id pairs (a < b), sorted. 2 uint32 per pair. */
int b2g_get_pairs(void* world, uint32_t* out_pairs, int32_t capacity, int32_t* out_count);
/* Fat AABBs (lower.x, lower.y, upper.x, upper.y per fixture) and moved flags
 * (B2dynamicTree::move_proxy, private/collision/b2_dynamic_tree.rs:109-168). */
int b2g_get_proxies(void* world, float* out_aabbs, uint8_t* out_moved, int32_t capacity);
/* Each fixture's proxy id (the reference's node index of its leaf in the dynamic tree,
 * B2fixtureProxy::proxy_id, src/b2_fixture.rs:93-99), -1 for a fixture without a proxy. */
int b2g_get_proxy_ids(void* world, int32_t* out_ids, int32_t capacity);
/* The constraint order the GPU solved in during the last step: one (fixture_a, fixture_b)
 * pair per island contact, grouped by colour. Feeding it to the host reference solver as its
 * island contact order reproduces the GPU's Gauss-Seidel sweep
 * (B2island::solve, private/dynamics/b2_island_private.rs:129-328). */
int b2g_get_solver_order(void* world, uint32_t* out_pairs, int32_t capacity, int32_t* out_count);

#ifdef __cplusplus
}
#endif
#endif /* B2G_H */
