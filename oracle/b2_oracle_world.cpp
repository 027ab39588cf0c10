/*
 * Oracle world step — TEST INFRASTRUCTURE ONLY.
 *
 * This is the CPU restatement of box2d-rs 0.0.4's `B2world::step` path that the
 * tests (and bench.py's cpu_baseline leg) use as the checker for the GPU path.
 * It is never linked into, loaded by or called from the product library.
 *
 * Restated reference code (paths inside the box2d-rs tree):
 *   B2world::step / solve / clear_forces     src/private/dynamics/b2_world.rs:356-531, 903-967
 *   B2world::create_body                     src/private/dynamics/b2_world.rs:83-98
 *   B2body (new, create_fixture, reset_mass_data, should_collide, synchronize_fixtures,
 *           set_transform, set_awake)        src/private/dynamics/b2_body.rs:15-78, 155-200,
 *                                            292-350, 391-475; src/b2_body.rs:783-801, 974-977
 *   B2fixture create_proxies / synchronize   src/private/dynamics/b2_fixture.rs:114-173
 *   B2contactManager collide / add_pair / destroy
 *                                            src/private/dynamics/b2_contact_manager.rs:24-302
 *   B2contact create / update / mixing       src/private/dynamics/b2_contact.rs:11-218,
 *                                            src/b2_contact.rs:29-46, b2_contact_registers.rs:67-103
 *   default contact filter                   src/private/dynamics/b2_world_callbacks.rs:6-18
 *   B2island::solve                          src/private/dynamics/b2_island_private.rs:129-328
 *   B2contactSolver (new, initialize_velocity_constraints, warm_start,
 *     solve_velocity_constraints, store_impulses, solve_position_constraints)
 *                                            src/private/dynamics/b2_contact_solver_private.rs:20-730
 * Linked lists keep the reference's newest-first order (src/b2rs_double_linked_list.rs:200-222).
 *
 * Added for parity (not in the reference): an ordering hook that replaces each
 * island's contact order with a caller-given order (the GPU's colour order), a
 * switch between libm and the project's sin/cos, and state export functions.
 * Not restated: continuous collision (solve_toi), joints, sensors' shape
 * overlap test, chain shapes, re-filtering. ora_set_flags rejects continuous=1.
 */
#include <algorithm>
#include <chrono>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../include/b2g.h"
#include "b2_oracle_collide.h"
#include "b2_oracle_tree.h"

namespace ora {

enum { STATIC = 0, KINEMATIC = 1, DYNAMIC = 2 };

struct Body {
    bool alive = true;  /* false once destroyed (its slot keeps its last state) */
    int type = STATIC;
    Xf xf{};
    Sweep sweep{};
    Vec2 v{0, 0};
    float w = 0.0f;
    Vec2 force{0, 0};
    float torque = 0.0f;
    float mass = 0, inv_mass = 0, I = 0, inv_I = 0;
    float lin_damp = 0, ang_damp = 0, grav_scale = 1;
    float sleep_time = 0;
    bool awake = false, enabled = true, auto_sleep = true, fixed_rotation = false, bullet = false;
    bool island_flag = false;
    int island_index = -1;
    int prev = -1, next = -1;
    int fixture_head = -1;
    int edge_head = -1;
    int jedge_head = -1;  /* joint edges, newest first */
};

struct Fixture {
    bool alive = true;
    int body = -1;
    Shape shape;
    float density = 0, friction = 0.2f, restitution = 0, threshold = 1.0f;
    bool sensor = false;
    uint16_t category = 1, mask = 0xffff;
    int16_t group = 0;
    int proxy = -1;
    int next = -1;
};

struct Edge {
    int contact = -1;
    int other = -1;
    int prev = -1, next = -1;
};

struct Contact {
    int fa = -1, fb = -1;
    Manifold m;
    bool touching = false, enabled = true, island_flag = false;
    bool filter_flag = false;  /* E_FILTER_FLAG: re-check should_collide at the next collide */
    bool toi_flag = false;   /* solve_toi: toi holds a valid time of impact */
    int toi_count = 0;
    float toi = 1.0f;
    float friction = 0, restitution = 0, threshold = 0, tangent_speed = 0;
    int prev = -1, next = -1;
    bool alive = false;
};

/* B2revoluteJoint (src/joints/b2_revolute_joint.rs:97-140) with the B2joint base */
struct Joint {
    int type = B2G_JOINT_REVOLUTE;
    int body_a = -1, body_b = -1;
    /* B2distanceJoint (private/dynamics/joints/b2_distance_joint.rs:42-76) */
    float length = 0, min_length = 0, max_length = 0, stiffness = 0, damping = 0;
    float dist_impulse = 0, gamma = 0, bias = 0, current_length = 0, mass = 0, soft_mass = 0;
    Vec2 u{0, 0};
    /* B2weldJoint (private/dynamics/joints/b2_weld_joint.rs): impulse (x, y, angular), mass matrix */
    float weld_impulse[3] = {0, 0, 0};
    /* B2frictionJoint (private/dynamics/joints/b2_friction_joint.rs) */
    float max_force = 0, max_torque = 0, angular_impulse = 0, angular_mass = 0;
    Vec2 linear_impulse{0, 0};
    Mat22 linear_mass{};
    /* B2motorJoint (private/dynamics/joints/b2_motor_joint.rs): shares max_force, max_torque, the
     * linear and angular impulses and masses with the friction joint */
    Vec2 linear_offset{0, 0}, linear_error{0, 0};
    float angular_offset = 0, correction_factor = 0, angular_error = 0;
    /* B2mouseJoint (private/dynamics/joints/b2_mouse_joint.rs): shares the linear impulse and mass, gamma,
     * max_force, stiffness and damping */
    Vec2 target{0, 0}, mouse_c{0, 0};
    float beta = 0;
    /* B2prismaticJoint (private/dynamics/joints/b2_prismatic_joint.rs): shares the point impulse, motor and
     * limit impulses, axial mass and K with the revolute joint */
    Vec2 local_xaxis_a{1, 0}, local_yaxis_a{0, 1}, axis{0, 0}, perp{0, 0};
    float a1 = 0, a2 = 0, s1 = 0, s2 = 0, translation = 0;
    float lower_translation = 0, upper_translation = 0, max_motor_force = 0;
    /* B2wheelJoint (private/dynamics/joints/b2_wheel_joint.rs): ax, ay in axis, perp; s_ax, s_bx in a1, a2;
     * s_ay, s_by in s1, s2; shares the motor and limit impulses, axial mass, bias and gamma */
    float wheel_impulse = 0, spring_impulse = 0, wheel_mass = 0, spring_mass = 0, motor_mass = 0;
    /* B2pulleyJoint (private/dynamics/joints/b2_pulley_joint.rs) */
    Vec2 ground_a{0, 0}, ground_b{0, 0}, u_a{0, 0}, u_b{0, 0};
    float pulley_constant = 0, ratio = 1, pulley_impulse = 0, pulley_mass = 0;
    float weld_mass[9] = {0};  /* ex, ey, ez columns */
    /* B2gearJoint (private/dynamics/joints/b2_gear_joint.rs): bodies C and D, the four local anchors, the
     * prismatic sides' axes and the sides' reference angles fixed at creation; the step's Jacobian */
    int body_c = -1, body_d = -1, index_c = 0, index_d = 0;
    bool gear_prismatic_a = false, gear_prismatic_b = false;
    Vec2 gear_anchor_a{0, 0}, gear_anchor_b{0, 0}, gear_anchor_c{0, 0}, gear_anchor_d{0, 0};
    Vec2 gear_axis_c{0, 0}, gear_axis_d{0, 0}, jv_ac{0, 0}, jv_bd{0, 0}, lc_c{0, 0}, lc_d{0, 0};
    float gear_ref_a = 0, gear_ref_b = 0, gear_constant = 0, gear_impulse = 0, gear_mass = 0;
    float jw_a = 0, jw_b = 0, jw_c = 0, jw_d = 0, inv_mass_c = 0, inv_mass_d = 0, inv_ic = 0, inv_id = 0;
    bool collide_connected = false, island_flag = false, alive = true;
    Vec2 local_anchor_a{0, 0}, local_anchor_b{0, 0};
    float reference_angle = 0;
    bool enable_limit = false, enable_motor = false;
    float lower_angle = 0, upper_angle = 0, motor_speed = 0, max_motor_torque = 0;
    Vec2 impulse{0, 0};
    float motor_impulse = 0, lower_impulse = 0, upper_impulse = 0;
    /* solver temporaries */
    int index_a = 0, index_b = 0;
    Vec2 r_a{0, 0}, r_b{0, 0}, lc_a{0, 0}, lc_b{0, 0};
    float inv_mass_a = 0, inv_mass_b = 0, inv_ia = 0, inv_ib = 0, axial_mass = 0, angle = 0;
    Mat22 k{};
    int prev = -1, next = -1;
};

struct JointEdge {
    int joint = -1;
    int other = -1;
    int next = -1;
};

struct Position {
    Vec2 c;
    float a;
};
struct Velocity {
    Vec2 v;
    float w;
};
struct VCPoint {
    Vec2 rA, rB;
    float ni, ti, nm, tm, bias;
};
struct VelocityConstraint {
    VCPoint p[2];
    Vec2 normal;
    Mat22 normal_mass, K;
    int ia, ib;
    float ma, mb, Ia, Ib;
    float friction, restitution, threshold, tangent_speed;
    int count;
    int contact;
};
struct PositionConstraint {
    Vec2 lp[2];
    Vec2 ln, lpt, lcA, lcB;
    int ia, ib;
    float ma, mb, IA, IB, rA, rB;
    int type, count;
};

struct Step {
    float dt, inv_dt, dt_ratio;
    int vi, pi;
    bool warm;
};

typedef int (*ContactFilterFn)(void* user, uint32_t fixture_a, uint32_t fixture_b);
typedef void (*PreSolveFn)(void* user, const b2g_contact_info* contact, const b2g_contact_info* old_manifold,
                           b2g_contact_edit* edit);

struct World {
    Vec2 gravity{0, -10};
    ContactFilterFn filter_fn = nullptr;  /* the user's contact filter (nullptr: the default filter) */
    std::vector<b2g_contact_impulse> post_solve;  /* the last step's island reports, in solve order */
    PreSolveFn pre_solve_fn = nullptr;            /* the listener's pre_solve (nullptr: none) */
    void* pre_solve_user = nullptr;
    void* filter_user = nullptr;
    std::vector<Body> bodies;
    std::vector<Fixture> fixtures;
    std::vector<Contact> contacts;
    std::vector<int> free_contacts;
    std::vector<Edge> edges;  /* 2 per contact slot: [2c] = node A, [2c+1] = node B */
    std::vector<Joint> joints;
    std::vector<JointEdge> jedges;  /* 2 per joint: [2j] = body A's, [2j+1] = body B's */
    int joint_head = -1;
    std::vector<int> joint_rank;    /* joint ordering hook: rank of each joint, -1 none */
    std::vector<int> isl_joints;
    int body_head = -1;
    int contact_head = -1;
    int contact_count = 0;
    BroadPhase bp;
    bool warm_starting = true, continuous = false, allow_sleep = true, auto_clear = true;
    bool new_contacts = false, locked = false;
    float inv_dt0 = 0.0f;
    b2g_profile profile{};
    /* parity / export */
    bool record_events = false;
    std::vector<b2g_contact_event> events;
    std::vector<Pair> last_pairs;   /* proxy-id pairs of the last update_pairs */
    std::vector<uint8_t> last_moved; /* per fixture: was in the move buffer at the last update_pairs */
    std::vector<int> proxy_to_fixture;
    bool hook = false;
    std::unordered_map<uint64_t, int> hook_rank;
    int hook_misses = 0;
    std::vector<uint64_t> last_order;  /* island contact order solved last step */
    int islands_solved = 0;
    int toi_events = 0;                /* solid time-of-impact events solved so far */
    bool key_order = false;            /* collide and solve_toi take contacts in key order */
    /* island scratch */
    std::vector<int> isl_bodies, isl_contacts, stack;
    std::vector<Position> pos;
    std::vector<Velocity> vel;
    std::vector<VelocityConstraint> vcs;
    std::vector<PositionConstraint> pcs;
    std::vector<Pair> pairs;
};

static inline uint64_t pair_key(int fa, int fb) { return ((uint64_t)(uint32_t)fa << 32) | (uint32_t)fb; }

/* ---- bodies ---- */

/* b2_body, private/dynamics/b2_body.rs:15-78 */
static int create_body(World& w, const b2g_body_def& d) {
    Body b;
    b.type = d.type;
    b.auto_sleep = d.allow_sleep != 0;
    b.fixed_rotation = d.fixed_rotation != 0;
    b.bullet = d.bullet != 0;
    b.awake = d.awake != 0 && d.type != STATIC;
    b.enabled = d.enabled != 0;
    b.xf.p = v2(d.position.x, d.position.y);
    b.xf.q = rot(d.angle);
    b.sweep.local_center = v2(0, 0);
    b.sweep.c0 = b.xf.p;
    b.sweep.c = b.xf.p;
    b.sweep.a0 = d.angle;
    b.sweep.a = d.angle;
    b.sweep.alpha0 = 0.0f;
    b.v = v2(d.linear_velocity.x, d.linear_velocity.y);
    b.w = d.angular_velocity;
    b.lin_damp = d.linear_damping;
    b.ang_damp = d.angular_damping;
    b.grav_scale = d.gravity_scale;
    int id = (int)w.bodies.size();
    /* push_front onto the world body list (private/dynamics/b2_world.rs:83-98) */
    b.next = w.body_head;
    if (w.body_head >= 0) w.bodies[w.body_head].prev = id;
    w.body_head = id;
    w.bodies.push_back(b);
    return id;
}

static void set_awake(Body& b, bool flag) {
    if (b.type == STATIC) return;
    b.awake = flag;
    b.sleep_time = 0.0f;
    if (!flag) {
        b.v = v2(0, 0);
        b.w = 0.0f;
        b.force = v2(0, 0);
        b.torque = 0.0f;
    }
}

/* reset_mass_data, private/dynamics/b2_body.rs:292-350 */
static void reset_mass_data(World& w, Body& b) {
    b.mass = 0.0f;
    b.inv_mass = 0.0f;
    b.I = 0.0f;
    b.inv_I = 0.0f;
    b.sweep.local_center = v2(0, 0);
    if (b.type == STATIC || b.type == KINEMATIC) {
        b.sweep.c0 = b.xf.p;
        b.sweep.c = b.xf.p;
        b.sweep.a0 = b.sweep.a;
        return;
    }
    Vec2 lc{0, 0};
    for (int f = b.fixture_head; f >= 0; f = w.fixtures[f].next) {
        const Fixture& fx = w.fixtures[f];
        if (fx.density == 0.0f) continue;
        MassData md;
        compute_mass(fx.shape, fx.density, md);
        b.mass += md.mass;
        lc += md.mass * md.center;
        b.I += md.I;
    }
    if (b.mass > 0.0f) {
        b.inv_mass = 1.0f / b.mass;
        lc *= b.inv_mass;
    }
    if (b.I > 0.0f && !b.fixed_rotation) {
        b.I -= b.mass * dot(lc, lc);
        b.inv_I = 1.0f / b.I;
    } else {
        b.I = 0.0f;
        b.inv_I = 0.0f;
    }
    Vec2 oldCenter = b.sweep.c;
    b.sweep.local_center = lc;
    b.sweep.c0 = mul(b.xf, b.sweep.local_center);
    b.sweep.c = b.sweep.c0;
    b.v += cross_sv(b.w, b.sweep.c - oldCenter);
}

static void build_shape(const b2g_fixture_def& d, Shape& s) {
    s.type = d.shape_type;
    s.radius = d.radius;
    if (d.shape_type == SHAPE_CIRCLE) {
        s.p = v2(d.vertices[0].x, d.vertices[0].y);
    } else if (d.shape_type == SHAPE_EDGE) {
        s.v0 = v2(d.vertices[0].x, d.vertices[0].y);
        s.v1 = v2(d.vertices[1].x, d.vertices[1].y);
        s.v2 = v2(d.vertices[2].x, d.vertices[2].y);
        s.v3 = v2(d.vertices[3].x, d.vertices[3].y);
        s.one_sided = d.one_sided != 0;
    } else {
        if (d.polygon_mode == B2G_POLYGON_BOX) {
            polygon_set_as_box(s, d.box_half_extents.x, d.box_half_extents.y);
        } else if (d.polygon_mode == B2G_POLYGON_BOX_ORIENTED) {
            polygon_set_as_box_oriented(s, d.box_half_extents.x, d.box_half_extents.y,
                                        v2(d.box_center.x, d.box_center.y), d.box_angle);
        } else {
            Vec2 pts[kMaxPolygonVertices];
            int n = d.vertex_count < kMaxPolygonVertices ? d.vertex_count : kMaxPolygonVertices;
            for (int i = 0; i < n; ++i) pts[i] = v2(d.vertices[i].x, d.vertices[i].y);
            polygon_set_hull(s, pts, n);
        }
        s.radius = d.radius;
    }
}

/* the fixture definition's shape, for the stand-alone routines (time of impact) */
void shape_from_def(const b2g_fixture_def& d, Shape& s) { build_shape(d, s); }

/* create_fixture, private/dynamics/b2_body.rs:155-200; create_proxies, private/dynamics/b2_fixture.rs:114-133 */
static int create_fixture(World& w, const b2g_fixture_def& d) {
    Fixture f;
    f.body = (int)d.body;
    build_shape(d, f.shape);
    f.density = d.density;
    f.friction = d.friction;
    f.restitution = d.restitution;
    f.threshold = d.restitution_threshold;
    f.sensor = d.is_sensor != 0;
    f.category = d.category_bits;
    f.mask = d.mask_bits;
    f.group = d.group_index;
    int id = (int)w.fixtures.size();
    Body& b = w.bodies[f.body];
    if (b.enabled) {
        AABB aabb;
        compute_aabb(f.shape, b.xf, aabb);
        f.proxy = w.bp.create_proxy(aabb, id);
        if ((int)w.proxy_to_fixture.size() <= f.proxy) w.proxy_to_fixture.resize((size_t)f.proxy + 1, -1);
        w.proxy_to_fixture[f.proxy] = id;
    }
    f.next = b.fixture_head;
    b.fixture_head = id;
    w.fixtures.push_back(f);
    w.last_moved.push_back(0);
    if (f.density > 0.0f) reset_mass_data(w, w.bodies[f.body]);
    w.new_contacts = true;
    return id;
}

/* b2_fixture_synchronize, private/dynamics/b2_fixture.rs:147-173 */
static void synchronize_fixture(World& w, Fixture& f, const Xf& xf1, const Xf& xf2) {
    if (f.proxy < 0) return;
    AABB a1, a2;
    compute_aabb(f.shape, xf1, a1);
    compute_aabb(f.shape, xf2, a2);
    AABB swept = combine(a1, a2);
    Vec2 disp = center(a2) - center(a1);
    w.bp.move_proxy(f.proxy, swept, disp);
}

/* synchronize_fixtures_internal, private/dynamics/b2_body.rs:455-475 */
static void synchronize_fixtures(World& w, Body& b) {
    if (b.awake) {
        Xf xf1;
        xf1.q = rot(b.sweep.a0);
        xf1.p = b.sweep.c0 - mul(xf1.q, b.sweep.local_center);
        for (int f = b.fixture_head; f >= 0; f = w.fixtures[f].next) synchronize_fixture(w, w.fixtures[f], xf1, b.xf);
    } else {
        for (int f = b.fixture_head; f >= 0; f = w.fixtures[f].next) synchronize_fixture(w, w.fixtures[f], b.xf, b.xf);
    }
}

static void synchronize_transform(Body& b) {
    b.xf.q = rot(b.sweep.a);
    b.xf.p = b.sweep.c - mul(b.xf.q, b.sweep.local_center);
}

/* ---- contacts ---- */

static void list_unlink_edge(World& w, int bodyId, int e) {
    Edge& E = w.edges[e];
    if (E.prev >= 0) w.edges[E.prev].next = E.next;
    else w.bodies[bodyId].edge_head = E.next;
    if (E.next >= 0) w.edges[E.next].prev = E.prev;
    E.prev = E.next = -1;
}

static void list_push_edge(World& w, int bodyId, int e) {
    Edge& E = w.edges[e];
    E.prev = -1;
    E.next = w.bodies[bodyId].edge_head;
    if (E.next >= 0) w.edges[E.next].prev = e;
    w.bodies[bodyId].edge_head = e;
}

/* default filter, private/dynamics/b2_world_callbacks.rs:6-18 */
static bool filter_should_collide(const Fixture& a, const Fixture& b) {
    if (a.group == b.group && a.group != 0) return a.group > 0;
    return (a.mask & b.category) != 0 && (a.category & b.mask) != 0;
}

/* the world's contact filter: the user's (B2world::set_contact_filter, src/b2_world.rs:38-40, replacing
 * the default) or the default one; called with the fixtures of the pair's smaller and larger proxy id
 * in add_pair, with the contact's fixtures A and B for a flagged contact in collide */
static bool contact_filter(const World& w, int fa, int fb) {
    if (w.filter_fn) return w.filter_fn(w.filter_user, (uint32_t)fa, (uint32_t)fb) != 0;
    return filter_should_collide(w.fixtures[fa], w.fixtures[fb]);
}

/* b2_contact_registers.rs:67-103: which (typeA, typeB) has a manifold routine with A first */
static int register_kind(int t1, int t2) {
    /* +1 primary, -1 swap, 0 none */
    static const int table[3][3] = {
        /* circle  edge  polygon */
        {+1, -1, -1}, /* circle */
        {+1, 0, +1},  /* edge   */
        {+1, -1, +1}, /* polygon*/
    };
    return table[t1][t2];
}

/* B2body::should_collide, private/dynamics/b2_body.rs:391-416: one body dynamic, and no joint
 * between them that keeps them from colliding */
static bool should_collide(const World& w, int self, int other) {
    if (w.bodies[self].type != DYNAMIC && w.bodies[other].type != DYNAMIC) return false;
    for (int e = w.bodies[self].jedge_head; e >= 0; e = w.jedges[e].next)
        if (w.jedges[e].other == other && !w.joints[w.jedges[e].joint].collide_connected) return false;
    return true;
}

/* b2_contact_manager_add_pair, private/dynamics/b2_contact_manager.rs:178-302 */
static void add_pair(World& w, int fixA, int fixB) {
    int bodyA = w.fixtures[fixA].body;
    int bodyB = w.fixtures[fixB].body;
    if (bodyA == bodyB) return;
    for (int e = w.bodies[bodyB].edge_head; e >= 0; e = w.edges[e].next) {
        if (w.edges[e].other == bodyA) {
            const Contact& c = w.contacts[w.edges[e].contact];
            if (c.fa == fixA && c.fb == fixB) return;
            if (c.fa == fixB && c.fb == fixA) return;
        }
    }
    if (!should_collide(w, bodyB, bodyA)) return;
    if (!contact_filter(w, fixA, fixB)) return;
    int kind = register_kind(w.fixtures[fixA].shape.type, w.fixtures[fixB].shape.type);
    if (kind == 0) return;
    if (kind < 0) std::swap(fixA, fixB);
    int id;
    if (!w.free_contacts.empty()) {
        id = w.free_contacts.back();
        w.free_contacts.pop_back();
    } else {
        id = (int)w.contacts.size();
        w.contacts.emplace_back();
        w.edges.emplace_back();
        w.edges.emplace_back();
    }
    Contact& c = w.contacts[id];
    c = Contact{};
    c.alive = true;
    c.fa = fixA;
    c.fb = fixB;
    const Fixture& FA = w.fixtures[fixA];
    const Fixture& FB = w.fixtures[fixB];
    c.friction = std::sqrt(FA.friction * FB.friction);
    c.restitution = FA.restitution > FB.restitution ? FA.restitution : FB.restitution;
    c.threshold = FA.threshold < FB.threshold ? FA.threshold : FB.threshold;
    c.tangent_speed = 0.0f;
    c.enabled = true;
    c.m.point_count = 0;
    /* push_front onto the world contact list */
    c.prev = -1;
    c.next = w.contact_head;
    if (w.contact_head >= 0) w.contacts[w.contact_head].prev = id;
    w.contact_head = id;
    int bA = FA.body, bB = FB.body;
    w.edges[2 * id].contact = id;
    w.edges[2 * id].other = bB;
    list_push_edge(w, bA, 2 * id);
    w.edges[2 * id + 1].contact = id;
    w.edges[2 * id + 1].other = bA;
    list_push_edge(w, bB, 2 * id + 1);
    ++w.contact_count;
}

/* b2_contact_manager_destroy, private/dynamics/b2_contact_manager.rs:24-78 */
static void destroy_contact(World& w, int id) {
    Contact& c = w.contacts[id];
    if (w.record_events && c.touching)
        w.events.push_back(b2g_contact_event{B2G_EVENT_END, (uint32_t)c.fa, (uint32_t)c.fb});
    if (c.prev >= 0) w.contacts[c.prev].next = c.next;
    else w.contact_head = c.next;
    if (c.next >= 0) w.contacts[c.next].prev = c.prev;
    int bA = w.fixtures[c.fa].body, bB = w.fixtures[c.fb].body;
    list_unlink_edge(w, bA, 2 * id);
    list_unlink_edge(w, bB, 2 * id + 1);
    /* B2contact::destroy wakes both bodies of a touching, non-sensor contact */
    if (c.m.point_count > 0 && !w.fixtures[c.fa].sensor && !w.fixtures[c.fb].sensor) {
        set_awake(w.bodies[bA], true);
        set_awake(w.bodies[bB], true);
    }
    c.alive = false;
    w.free_contacts.push_back(id);
    --w.contact_count;
}

static void evaluate(const Contact& c, const World& w, Manifold& m, const Xf& xfA, const Xf& xfB) {
    const Shape& sa = w.fixtures[c.fa].shape;
    const Shape& sb = w.fixtures[c.fb].shape;
    if (sa.type == SHAPE_CIRCLE) collide_circles(m, sa, xfA, sb, xfB);
    else if (sa.type == SHAPE_POLYGON && sb.type == SHAPE_CIRCLE) collide_polygon_circle(m, sa, xfA, sb, xfB);
    else if (sa.type == SHAPE_POLYGON) collide_polygons(m, sa, xfA, sb, xfB);
    else if (sb.type == SHAPE_CIRCLE) collide_edge_circle(m, sa, xfA, sb, xfB);
    else collide_edge_polygon(m, sa, xfA, sb, xfB);
}

/* a contact (fixtures, touching flag, material) with manifold m, as the C ABI reports it */
static void contact_info(const Contact& c, const Manifold& m, b2g_contact_info& o) {
    memset(&o, 0, sizeof(o));
    o.fixture_a = (uint32_t)c.fa;
    o.fixture_b = (uint32_t)c.fb;
    o.touching = c.touching ? 1 : 0;
    o.manifold_type = m.type;
    o.point_count = m.point_count;
    o.local_normal = b2g_vec2{m.local_normal.x, m.local_normal.y};
    o.local_point = b2g_vec2{m.local_point.x, m.local_point.y};
    for (int j = 0; j < 2; ++j) {
        o.point_local[j] = b2g_vec2{m.points[j].local_point.x, m.points[j].local_point.y};
        o.normal_impulse[j] = m.points[j].normal_impulse;
        o.tangent_impulse[j] = m.points[j].tangent_impulse;
        o.point_id[j] = m.points[j].id;
    }
    o.friction = c.friction;
    o.restitution = c.restitution;
    o.restitution_threshold = c.threshold;
}

/* b2_contact_update, private/dynamics/b2_contact.rs:103-218 */
static void update_contact(World& w, int id) {
    Contact& c = w.contacts[id];
    c.enabled = true;
    Manifold old = c.m;
    bool wasTouching = c.touching;
    bool sensor = w.fixtures[c.fa].sensor || w.fixtures[c.fb].sensor;
    Body& bA = w.bodies[w.fixtures[c.fa].body];
    Body& bB = w.bodies[w.fixtures[c.fb].body];
    bool touching;
    if (sensor) {
        /* shape overlap for sensors is not restated (GJK is outside this path) */
        touching = false;
        c.m.point_count = 0;
    } else {
        Manifold nm;
        evaluate(c, w, nm, bA.xf, bB.xf);
        c.m = nm;
        touching = c.m.point_count > 0;
        for (int i = 0; i < c.m.point_count; ++i) {
            ManifoldPoint& mp2 = c.m.points[i];
            mp2.normal_impulse = 0.0f;
            mp2.tangent_impulse = 0.0f;
            for (int j = 0; j < old.point_count; ++j) {
                if (old.points[j].id == mp2.id) {
                    mp2.normal_impulse = old.points[j].normal_impulse;
                    mp2.tangent_impulse = old.points[j].tangent_impulse;
                    break;
                }
            }
        }
        if (touching != wasTouching) {
            set_awake(bA, true);
            set_awake(bB, true);
        }
    }
    c.touching = touching;
    if (w.record_events) {
        if (!wasTouching && touching) w.events.push_back(b2g_contact_event{B2G_EVENT_BEGIN, (uint32_t)c.fa, (uint32_t)c.fb});
        if (wasTouching && !touching) w.events.push_back(b2g_contact_event{B2G_EVENT_END, (uint32_t)c.fa, (uint32_t)c.fb});
    }
    /* listener.pre_solve(contact, old_manifold) for a touching non-sensor contact (:215); the
     * listener may disable the contact or change its material for this step */
    if (!sensor && touching && w.pre_solve_fn) {
        b2g_contact_info now, prev;
        contact_info(c, c.m, now);
        contact_info(c, old, prev);
        prev.touching = wasTouching ? 1 : 0;
        b2g_contact_edit e{c.enabled ? 1 : 0, c.friction, c.restitution, c.threshold, c.tangent_speed};
        w.pre_solve_fn(w.pre_solve_user, &now, &prev, &e);
        c.enabled = e.enabled != 0;
        c.friction = e.friction;
        c.restitution = e.restitution;
        c.threshold = e.restitution_threshold;
        c.tangent_speed = e.tangent_speed;
    }
}

static uint64_t contact_proxy_key(const World& w, const Contact& c);

/* b2_contact_manager_collide, private/dynamics/b2_contact_manager.rs:83-171. The loop sees, at
 * each contact, the bodies woken by the updates before it; with key_order set it goes through the
 * contacts in key order (the GPU's table order) instead of the list order. */
static void collide(World& w) {
    std::vector<int> to_destroy;
    std::vector<int> order;
    for (int id = w.contact_head; id >= 0; id = w.contacts[id].next) order.push_back(id);
    if (w.key_order)
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            return contact_proxy_key(w, w.contacts[x]) < contact_proxy_key(w, w.contacts[y]);
        });
    for (int id : order) {
        Contact& c = w.contacts[id];
        const Fixture& FA = w.fixtures[c.fa];
        const Fixture& FB = w.fixtures[c.fb];
        if (c.filter_flag) {
            /* should these bodies collide, and does the contact filter still allow the fixtures? */
            if (!should_collide(w, FB.body, FA.body) || !contact_filter(w, c.fa, c.fb)) {
                to_destroy.push_back(id);
                continue;
            }
            c.filter_flag = false;
        }
        const Body& bA = w.bodies[FA.body];
        const Body& bB = w.bodies[FB.body];
        bool activeA = bA.awake && bA.type != STATIC;
        bool activeB = bB.awake && bB.type != STATIC;
        if (!activeA && !activeB) continue;
        if (!w.bp.test_overlap(FA.proxy, FB.proxy)) {
            to_destroy.push_back(id);
            continue;
        }
        update_contact(w, id);
    }
    for (int id : to_destroy) destroy_contact(w, id);
}

/* find_new_contacts -> update_pairs -> add_pair */
static void find_new_contacts(World& w) {
    std::fill(w.last_moved.begin(), w.last_moved.end(), 0);
    for (int q : w.bp.move_buffer())
        if (q != kNullNode) w.last_moved[w.bp.tree.user(q)] = 1;
    w.bp.update_pairs(w.pairs);
    w.last_pairs = w.pairs;
    for (const Pair& p : w.pairs) add_pair(w, w.bp.tree.user(p.a), w.bp.tree.user(p.b));
}

/* ---- island solver ---- */

/* B2contactSolver::new + initialize_velocity_constraints, b2_contact_solver_private.rs:20-226 */
static void init_constraints(World& w, const Step& step) {
    int n = (int)w.isl_contacts.size();
    w.vcs.resize(n);
    w.pcs.resize(n);
    for (int i = 0; i < n; ++i) {
        const Contact& c = w.contacts[w.isl_contacts[i]];
        const Fixture& FA = w.fixtures[c.fa];
        const Fixture& FB = w.fixtures[c.fb];
        const Body& bA = w.bodies[FA.body];
        const Body& bB = w.bodies[FB.body];
        const Manifold& m = c.m;
        VelocityConstraint& vc = w.vcs[i];
        vc.friction = c.friction;
        vc.restitution = c.restitution;
        vc.threshold = c.threshold;
        vc.tangent_speed = c.tangent_speed;
        vc.ia = bA.island_index;
        vc.ib = bB.island_index;
        vc.ma = bA.inv_mass;
        vc.mb = bB.inv_mass;
        vc.Ia = bA.inv_I;
        vc.Ib = bB.inv_I;
        vc.contact = i;
        vc.count = m.point_count;
        vc.K = Mat22{v2(0, 0), v2(0, 0)};
        vc.normal_mass = Mat22{v2(0, 0), v2(0, 0)};
        PositionConstraint& pc = w.pcs[i];
        pc.ia = bA.island_index;
        pc.ib = bB.island_index;
        pc.ma = bA.inv_mass;
        pc.mb = bB.inv_mass;
        pc.lcA = bA.sweep.local_center;
        pc.lcB = bB.sweep.local_center;
        pc.IA = bA.inv_I;
        pc.IB = bB.inv_I;
        pc.ln = m.local_normal;
        pc.lpt = m.local_point;
        pc.count = m.point_count;
        pc.rA = FA.shape.radius;
        pc.rB = FB.shape.radius;
        pc.type = m.type;
        for (int j = 0; j < m.point_count; ++j) {
            VCPoint& p = vc.p[j];
            if (step.warm) {
                p.ni = step.dt_ratio * m.points[j].normal_impulse;
                p.ti = step.dt_ratio * m.points[j].tangent_impulse;
            } else {
                p.ni = 0.0f;
                p.ti = 0.0f;
            }
            p.rA = v2(0, 0);
            p.rB = v2(0, 0);
            p.nm = 0.0f;
            p.tm = 0.0f;
            p.bias = 0.0f;
            pc.lp[j] = m.points[j].local_point;
        }
    }
    for (int i = 0; i < n; ++i) {
        VelocityConstraint& vc = w.vcs[i];
        PositionConstraint& pc = w.pcs[i];
        const Manifold& m = w.contacts[w.isl_contacts[vc.contact]].m;
        float mA = vc.ma, mB = vc.mb, iA = vc.Ia, iB = vc.Ib;
        Vec2 cA = w.pos[vc.ia].c;
        float aA = w.pos[vc.ia].a;
        Vec2 vA = w.vel[vc.ia].v;
        float wA = w.vel[vc.ia].w;
        Vec2 cB = w.pos[vc.ib].c;
        float aB = w.pos[vc.ib].a;
        Vec2 vB = w.vel[vc.ib].v;
        float wB = w.vel[vc.ib].w;
        Xf xfA, xfB;
        xfA.q = rot(aA);
        xfB.q = rot(aB);
        xfA.p = cA - mul(xfA.q, pc.lcA);
        xfB.p = cB - mul(xfB.q, pc.lcB);
        WorldManifold wm;
        world_manifold(wm, m, xfA, pc.rA, xfB, pc.rB);
        vc.normal = wm.normal;
        for (int j = 0; j < vc.count; ++j) {
            VCPoint& p = vc.p[j];
            p.rA = wm.points[j] - cA;
            p.rB = wm.points[j] - cB;
            float rnA = cross(p.rA, vc.normal);
            float rnB = cross(p.rB, vc.normal);
            float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
            p.nm = kNormal > 0.0f ? 1.0f / kNormal : 0.0f;
            Vec2 tangent = cross_vs(vc.normal, 1.0f);
            float rtA = cross(p.rA, tangent);
            float rtB = cross(p.rB, tangent);
            float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
            p.tm = kTangent > 0.0f ? 1.0f / kTangent : 0.0f;
            p.bias = 0.0f;
            float vRel = dot(vc.normal, vB + cross_sv(wB, p.rB) - vA - cross_sv(wA, p.rA));
            if (vRel < -vc.threshold) p.bias = -vc.restitution * vRel;
        }
        if (vc.count == 2) {
            const VCPoint& p1 = vc.p[0];
            const VCPoint& p2 = vc.p[1];
            float rn1A = cross(p1.rA, vc.normal);
            float rn1B = cross(p1.rB, vc.normal);
            float rn2A = cross(p2.rA, vc.normal);
            float rn2B = cross(p2.rB, vc.normal);
            float k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
            float k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
            float k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
            const float kMaxConditionNumber = 1000.0f;
            if (k11 * k11 < kMaxConditionNumber * (k11 * k22 - k12 * k12)) {
                vc.K.ex = v2(k11, k12);
                vc.K.ey = v2(k12, k22);
                vc.normal_mass = inverse(vc.K);
            } else {
                vc.count = 1;
            }
        }
    }
}

/* warm_start, :228-266 */
static void warm_start(World& w) {
    for (VelocityConstraint& vc : w.vcs) {
        float mA = vc.ma, iA = vc.Ia, mB = vc.mb, iB = vc.Ib;
        Vec2 vA = w.vel[vc.ia].v;
        float wA = w.vel[vc.ia].w;
        Vec2 vB = w.vel[vc.ib].v;
        float wB = w.vel[vc.ib].w;
        Vec2 normal = vc.normal;
        Vec2 tangent = cross_vs(normal, 1.0f);
        for (int j = 0; j < vc.count; ++j) {
            const VCPoint& p = vc.p[j];
            Vec2 P = p.ni * normal + p.ti * tangent;
            wA -= iA * cross(p.rA, P);
            vA -= mA * P;
            wB += iB * cross(p.rB, P);
            vB += mB * P;
        }
        w.vel[vc.ia].v = vA;
        w.vel[vc.ia].w = wA;
        w.vel[vc.ib].v = vB;
        w.vel[vc.ib].w = wB;
    }
}

/* solve_velocity_constraints, :268-583 (friction, then normal: 1-point or 2-point block LCP) */
static void solve_velocity(World& w) {
    for (VelocityConstraint& vc : w.vcs) {
        float mA = vc.ma, iA = vc.Ia, mB = vc.mb, iB = vc.Ib;
        Vec2 vA = w.vel[vc.ia].v;
        float wA = w.vel[vc.ia].w;
        Vec2 vB = w.vel[vc.ib].v;
        float wB = w.vel[vc.ib].w;
        Vec2 normal = vc.normal;
        Vec2 tangent = cross_vs(normal, 1.0f);
        float friction = vc.friction;
        for (int j = 0; j < vc.count; ++j) {
            VCPoint& p = vc.p[j];
            Vec2 dv = vB + cross_sv(wB, p.rB) - vA - cross_sv(wA, p.rA);
            float vt = dot(dv, tangent) - vc.tangent_speed;
            float lambda = p.tm * (-vt);
            float maxFriction = friction * p.ni;
            float newImpulse = bclamp(p.ti + lambda, -maxFriction, maxFriction);
            lambda = newImpulse - p.ti;
            p.ti = newImpulse;
            Vec2 P = lambda * tangent;
            vA -= mA * P;
            wA -= iA * cross(p.rA, P);
            vB += mB * P;
            wB += iB * cross(p.rB, P);
        }
        if (vc.count == 1) {
            VCPoint& p = vc.p[0];
            Vec2 dv = vB + cross_sv(wB, p.rB) - vA - cross_sv(wA, p.rA);
            float vn = dot(dv, normal);
            float lambda = -p.nm * (vn - p.bias);
            float newImpulse = bmax(p.ni + lambda, 0.0f);
            lambda = newImpulse - p.ni;
            p.ni = newImpulse;
            Vec2 P = lambda * normal;
            vA -= mA * P;
            wA -= iA * cross(p.rA, P);
            vB += mB * P;
            wB += iB * cross(p.rB, P);
        } else {
            VCPoint& cp1 = vc.p[0];
            VCPoint& cp2 = vc.p[1];
            Vec2 a{cp1.ni, cp2.ni};
            Vec2 dv1 = vB + cross_sv(wB, cp1.rB) - vA - cross_sv(wA, cp1.rA);
            Vec2 dv2 = vB + cross_sv(wB, cp2.rB) - vA - cross_sv(wA, cp2.rA);
            float vn1 = dot(dv1, normal);
            float vn2 = dot(dv2, normal);
            Vec2 b{vn1 - cp1.bias, vn2 - cp2.bias};
            b -= mul(vc.K, a);
            for (;;) {
                Vec2 x = -mul(vc.normal_mass, b);
                if (x.x >= 0.0f && x.y >= 0.0f) goto apply;
                x.x = -cp1.nm * b.x;
                x.y = 0.0f;
                vn2 = vc.K.ex.y * x.x + b.y;
                if (x.x >= 0.0f && vn2 >= 0.0f) goto apply;
                x.x = 0.0f;
                x.y = -cp2.nm * b.y;
                vn1 = vc.K.ey.x * x.y + b.x;
                if (x.y >= 0.0f && vn1 >= 0.0f) goto apply;
                x.x = 0.0f;
                x.y = 0.0f;
                vn1 = b.x;
                vn2 = b.y;
                if (vn1 >= 0.0f && vn2 >= 0.0f) goto apply;
                break;
            apply : {
                Vec2 d = x - a;
                Vec2 P1 = d.x * normal;
                Vec2 P2 = d.y * normal;
                vA -= mA * (P1 + P2);
                wA -= iA * (cross(cp1.rA, P1) + cross(cp2.rA, P2));
                vB += mB * (P1 + P2);
                wB += iB * (cross(cp1.rB, P1) + cross(cp2.rB, P2));
                cp1.ni = x.x;
                cp2.ni = x.y;
                break;
            }
            }
        }
        w.vel[vc.ia].v = vA;
        w.vel[vc.ia].w = wA;
        w.vel[vc.ib].v = vB;
        w.vel[vc.ib].w = wB;
    }
}

/* store_impulses, :585-598 */
static void store_impulses(World& w) {
    for (const VelocityConstraint& vc : w.vcs) {
        Manifold& m = w.contacts[w.isl_contacts[vc.contact]].m;
        for (int j = 0; j < vc.count; ++j) {
            m.points[j].normal_impulse = vc.p[j].ni;
            m.points[j].tangent_impulse = vc.p[j].ti;
        }
    }
}

/* B2positionSolverManifold::initialize, :600-642 */
static void position_manifold(const PositionConstraint& pc, const Xf& xfA, const Xf& xfB, int index, Vec2& normal,
                              Vec2& point, float& separation) {
    if (pc.type == MANIFOLD_CIRCLES) {
        Vec2 pA = mul(xfA, pc.lpt);
        Vec2 pB = mul(xfB, pc.lp[0]);
        normal = pB - pA;
        normalize(normal);
        point = 0.5f * (pA + pB);
        separation = dot(pB - pA, normal) - pc.rA - pc.rB;
    } else if (pc.type == MANIFOLD_FACE_A) {
        normal = mul(xfA.q, pc.ln);
        Vec2 plane = mul(xfA, pc.lpt);
        Vec2 clip = mul(xfB, pc.lp[index]);
        separation = dot(clip - plane, normal) - pc.rA - pc.rB;
        point = clip;
    } else {
        normal = mul(xfB.q, pc.ln);
        Vec2 plane = mul(xfB, pc.lpt);
        Vec2 clip = mul(xfA, pc.lp[index]);
        separation = dot(clip - plane, normal) - pc.rA - pc.rB;
        point = clip;
        normal = -normal;
    }
}

/* solve_position_constraints, :653-730 */
static bool solve_position(World& w) {
    float minSeparation = 0.0f;
    for (const PositionConstraint& pc : w.pcs) {
        Vec2 lcA = pc.lcA, lcB = pc.lcB;
        float mA = pc.ma, iA = pc.IA, mB = pc.mb, iB = pc.IB;
        Vec2 cA = w.pos[pc.ia].c;
        float aA = w.pos[pc.ia].a;
        Vec2 cB = w.pos[pc.ib].c;
        float aB = w.pos[pc.ib].a;
        for (int j = 0; j < pc.count; ++j) {
            Xf xfA, xfB;
            xfA.q = rot(aA);
            xfB.q = rot(aB);
            xfA.p = cA - mul(xfA.q, lcA);
            xfB.p = cB - mul(xfB.q, lcB);
            Vec2 normal, point;
            float separation;
            position_manifold(pc, xfA, xfB, j, normal, point, separation);
            Vec2 rA = point - cA;
            Vec2 rB = point - cB;
            minSeparation = bmin(minSeparation, separation);
            float C = bclamp(kBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
            float rnA = cross(rA, normal);
            float rnB = cross(rB, normal);
            float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
            float impulse = K > 0.0f ? -C / K : 0.0f;
            Vec2 P = impulse * normal;
            cA -= mA * P;
            aA -= iA * cross(rA, P);
            cB += mB * P;
            aB += iB * cross(rB, P);
        }
        w.pos[pc.ia].c = cA;
        w.pos[pc.ia].a = aA;
        w.pos[pc.ib].c = cB;
        w.pos[pc.ib].a = aB;
    }
    return minSeparation >= -3.0f * kLinearSlop;
}

/* ---- revolute joint, private/dynamics/joints/b2_revolute_joint.rs ---- */

/* ---- distance joint, private/dynamics/joints/b2_distance_joint.rs ---- */

/* init_velocity_constraints (:78-181) */
static void distance_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const Vec2 cA = w.pos[j.index_a].c;
    const float aA = w.pos[j.index_a].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    const Vec2 cB = w.pos[j.index_b].c;
    const float aB = w.pos[j.index_b].a;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    j.r_a = mul(qA, j.local_anchor_a - j.lc_a);
    j.r_b = mul(qB, j.local_anchor_b - j.lc_b);
    j.u = cB + j.r_b - cA - j.r_a;
    j.current_length = length(j.u);
    if (j.current_length > kLinearSlop) {
        j.u *= 1.0f / j.current_length;
    } else {
        j.u = v2(0.0f, 0.0f);
        j.mass = 0.0f;
        j.dist_impulse = 0.0f;
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    const float crAu = cross(j.r_a, j.u);
    const float crBu = cross(j.r_b, j.u);
    float inv_mass = j.inv_mass_a + j.inv_ia * crAu * crAu + j.inv_mass_b + j.inv_ib * crBu * crBu;
    j.mass = inv_mass != 0.0f ? 1.0f / inv_mass : 0.0f;
    if (j.stiffness > 0.0f && j.min_length < j.max_length) {
        const float C = j.current_length - j.length;
        const float d = j.damping;
        const float k = j.stiffness;
        const float h = step.dt;
        j.gamma = h * (d + h * k);
        j.gamma = j.gamma != 0.0f ? 1.0f / j.gamma : 0.0f;
        j.bias = C * h * k * j.gamma;
        inv_mass += j.gamma;
        j.soft_mass = inv_mass != 0.0f ? 1.0f / inv_mass : 0.0f;
    } else {
        j.gamma = 0.0f;
        j.bias = 0.0f;
        j.soft_mass = j.mass;
    }
    if (step.warm) {
        j.dist_impulse *= step.dt_ratio;
        j.lower_impulse *= step.dt_ratio;
        j.upper_impulse *= step.dt_ratio;
        const Vec2 P = (j.dist_impulse + j.lower_impulse - j.upper_impulse) * j.u;
        vA -= j.inv_mass_a * P;
        wA -= j.inv_ia * cross(j.r_a, P);
        vB += j.inv_mass_b * P;
        wB += j.inv_ib * cross(j.r_b, P);
    } else {
        j.dist_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* solve_velocity_constraints (:183-274) */
static void distance_solve_velocity(World& w, Joint& j, const Step& step) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    auto apply = [&](Vec2 P) {
        vA -= j.inv_mass_a * P;
        wA -= j.inv_ia * cross(j.r_a, P);
        vB += j.inv_mass_b * P;
        wB += j.inv_ib * cross(j.r_b, P);
    };
    if (j.min_length < j.max_length) {
        if (j.stiffness > 0.0f) {
            const Vec2 vpA = vA + cross_sv(wA, j.r_a);
            const Vec2 vpB = vB + cross_sv(wB, j.r_b);
            const float cdot = dot(j.u, vpB - vpA);
            const float impulse = -j.soft_mass * (cdot + j.bias + j.gamma * j.dist_impulse);
            j.dist_impulse += impulse;
            apply(impulse * j.u);
        }
        {
            const float C = j.current_length - j.min_length;
            const float bias = bmax(0.0f, C) * step.inv_dt;
            const Vec2 vpA = vA + cross_sv(wA, j.r_a);
            const Vec2 vpB = vB + cross_sv(wB, j.r_b);
            const float cdot = dot(j.u, vpB - vpA);
            float impulse = -j.mass * (cdot + bias);
            const float old_impulse = j.lower_impulse;
            j.lower_impulse = bmax(0.0f, j.lower_impulse + impulse);
            impulse = j.lower_impulse - old_impulse;
            apply(impulse * j.u);
        }
        {
            const float C = j.max_length - j.current_length;
            const float bias = bmax(0.0f, C) * step.inv_dt;
            const Vec2 vpA = vA + cross_sv(wA, j.r_a);
            const Vec2 vpB = vB + cross_sv(wB, j.r_b);
            const float cdot = dot(j.u, vpA - vpB);
            float impulse = -j.mass * (cdot + bias);
            const float old_impulse = j.upper_impulse;
            j.upper_impulse = bmax(0.0f, j.upper_impulse + impulse);
            impulse = j.upper_impulse - old_impulse;
            apply(-impulse * j.u);
        }
    } else {
        const Vec2 vpA = vA + cross_sv(wA, j.r_a);
        const Vec2 vpB = vB + cross_sv(wB, j.r_b);
        const float cdot = dot(j.u, vpB - vpA);
        const float impulse = -j.mass * cdot;
        j.dist_impulse += impulse;
        apply(impulse * j.u);
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* solve_position_constraints (:276-319) */
static bool distance_solve_position(World& w, Joint& j) {
    Vec2 cA = w.pos[j.index_a].c;
    float aA = w.pos[j.index_a].a;
    Vec2 cB = w.pos[j.index_b].c;
    float aB = w.pos[j.index_b].a;
    const Rot qA = rot(aA), qB = rot(aB);
    const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
    const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
    Vec2 u = cB + rB - cA - rA;
    const float len = normalize(u);
    float C;
    if (j.min_length == j.max_length) C = len - j.min_length;
    else if (len < j.min_length) C = len - j.min_length;
    else if (j.max_length < len) C = len - j.max_length;
    else return true;
    const float impulse = -j.mass * C;
    const Vec2 P = impulse * u;
    cA -= j.inv_mass_a * P;
    aA -= j.inv_ia * cross(rA, P);
    cB += j.inv_mass_b * P;
    aB += j.inv_ib * cross(rB, P);
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    return std::fabs(C) < kLinearSlop;
}

/* ---- weld joint, private/dynamics/joints/b2_weld_joint.rs (with B2Mat33, src/b2_math.rs and
 * private/common/b2_math.rs:5-71) ---- */

struct V3 {
    float x, y, z;
};
static V3 v3add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static V3 v3scale(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
static float v3dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static V3 v3cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
struct M33 {
    V3 ex, ey, ez;
};
/* K of the weld joint (b2_weld_joint.rs init and position solve share its expressions) */
static M33 weld_k(float mA, float mB, float iA, float iB, Vec2 rA, Vec2 rB) {
    M33 k;
    k.ex.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;
    k.ey.x = -rA.y * rA.x * iA - rB.y * rB.x * iB;
    k.ez.x = -rA.y * iA - rB.y * iB;
    k.ex.y = k.ey.x;
    k.ey.y = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;
    k.ez.y = rA.x * iA + rB.x * iB;
    k.ex.z = k.ez.x;
    k.ey.z = k.ez.y;
    k.ez.z = iA + iB;
    return k;
}
static void m33_inverse22(const M33& a, M33& m) {
    const float A = a.ex.x, B = a.ey.x, C = a.ex.y, D = a.ey.y;
    float det = A * D - B * C;
    if (det != 0.0f) det = 1.0f / det;
    m.ex.x = det * D;
    m.ey.x = -det * B;
    m.ex.z = 0.0f;
    m.ex.y = -det * C;
    m.ey.y = det * A;
    m.ey.z = 0.0f;
    m.ez.x = 0.0f;
    m.ez.y = 0.0f;
    m.ez.z = 0.0f;
}
static void m33_sym_inverse33(const M33& a, M33& m) {
    float det = v3dot(a.ex, v3cross(a.ey, a.ez));
    if (det != 0.0f) det = 1.0f / det;
    const float a11 = a.ex.x, a12 = a.ey.x, a13 = a.ez.x, a22 = a.ey.y, a23 = a.ez.y, a33 = a.ez.z;
    m.ex.x = det * (a22 * a33 - a23 * a23);
    m.ex.y = det * (a13 * a23 - a12 * a33);
    m.ex.z = det * (a12 * a23 - a13 * a22);
    m.ey.x = m.ex.y;
    m.ey.y = det * (a11 * a33 - a13 * a13);
    m.ey.z = det * (a13 * a12 - a11 * a23);
    m.ez.x = m.ex.z;
    m.ez.y = m.ey.z;
    m.ez.z = det * (a11 * a22 - a12 * a12);
}
static V3 m33_solve33(const M33& a, V3 b) {
    float det = v3dot(a.ex, v3cross(a.ey, a.ez));
    if (det != 0.0f) det = 1.0f / det;
    return V3{det * v3dot(b, v3cross(a.ey, a.ez)), det * v3dot(a.ex, v3cross(b, a.ez)), det * v3dot(a.ex, v3cross(a.ey, b))};
}
static Vec2 m33_solve22(const M33& a, Vec2 b) {
    const float a11 = a.ex.x, a12 = a.ey.x, a21 = a.ex.y, a22 = a.ey.y;
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = 1.0f / det;
    return v2(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}
static M33 weld_mass_of(const Joint& j) {
    M33 m;
    m.ex = V3{j.weld_mass[0], j.weld_mass[1], j.weld_mass[2]};
    m.ey = V3{j.weld_mass[3], j.weld_mass[4], j.weld_mass[5]};
    m.ez = V3{j.weld_mass[6], j.weld_mass[7], j.weld_mass[8]};
    return m;
}

/* init_velocity_constraints */
static void weld_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    j.r_a = mul(qA, j.local_anchor_a - j.lc_a);
    j.r_b = mul(qB, j.local_anchor_b - j.lc_b);
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const M33 k = weld_k(mA, mB, iA, iB, j.r_a, j.r_b);
    M33 mass{};
    if (j.stiffness > 0.0f) {
        m33_inverse22(k, mass);
        float inv_m = iA + iB;
        const float C = aB - aA - j.reference_angle;
        const float d = j.damping;
        const float kk = j.stiffness;
        const float h = step.dt;
        j.gamma = h * (d + h * kk);
        j.gamma = j.gamma != 0.0f ? 1.0f / j.gamma : 0.0f;
        j.bias = C * h * kk * j.gamma;
        inv_m += j.gamma;
        mass.ez.z = inv_m != 0.0f ? 1.0f / inv_m : 0.0f;
    } else if (k.ez.z == 0.0f) {
        m33_inverse22(k, mass);
        j.gamma = 0.0f;
        j.bias = 0.0f;
    } else {
        m33_sym_inverse33(k, mass);
        j.gamma = 0.0f;
        j.bias = 0.0f;
    }
    const float mm[9] = {mass.ex.x, mass.ex.y, mass.ex.z, mass.ey.x, mass.ey.y, mass.ey.z, mass.ez.x, mass.ez.y, mass.ez.z};
    for (int q = 0; q < 9; ++q) j.weld_mass[q] = mm[q];
    if (step.warm) {
        for (float& x : j.weld_impulse) x *= step.dt_ratio;
        const Vec2 P = v2(j.weld_impulse[0], j.weld_impulse[1]);
        vA -= mA * P;
        wA -= iA * (cross(j.r_a, P) + j.weld_impulse[2]);
        vB += mB * P;
        wB += iB * (cross(j.r_b, P) + j.weld_impulse[2]);
    } else {
        j.weld_impulse[0] = j.weld_impulse[1] = j.weld_impulse[2] = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* solve_velocity_constraints */
static void weld_solve_velocity(World& w, Joint& j) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const M33 mass = weld_mass_of(j);
    if (j.stiffness > 0.0f) {
        const float cdot2 = wB - wA;
        const float impulse2 = -mass.ez.z * (cdot2 + j.bias + j.gamma * j.weld_impulse[2]);
        j.weld_impulse[2] += impulse2;
        wA -= iA * impulse2;
        wB += iB * impulse2;
        const Vec2 cdot1 = vB + cross_sv(wB, j.r_b) - vA - cross_sv(wA, j.r_a);
        const Vec2 impulse1 = -v2(mass.ex.x * cdot1.x + mass.ey.x * cdot1.y, mass.ex.y * cdot1.x + mass.ey.y * cdot1.y);
        j.weld_impulse[0] += impulse1.x;
        j.weld_impulse[1] += impulse1.y;
        const Vec2 P = impulse1;
        vA -= mA * P;
        wA -= iA * cross(j.r_a, P);
        vB += mB * P;
        wB += iB * cross(j.r_b, P);
    } else {
        const Vec2 cdot1 = vB + cross_sv(wB, j.r_b) - vA - cross_sv(wA, j.r_a);
        const float cdot2 = wB - wA;
        const V3 cdot{cdot1.x, cdot1.y, cdot2};
        const V3 mc = v3add(v3add(v3scale(cdot.x, mass.ex), v3scale(cdot.y, mass.ey)), v3scale(cdot.z, mass.ez));
        const V3 impulse{-mc.x, -mc.y, -mc.z};
        j.weld_impulse[0] += impulse.x;
        j.weld_impulse[1] += impulse.y;
        j.weld_impulse[2] += impulse.z;
        const Vec2 P = v2(impulse.x, impulse.y);
        vA -= mA * P;
        wA -= iA * (cross(j.r_a, P) + impulse.z);
        vB += mB * P;
        wB += iB * (cross(j.r_b, P) + impulse.z);
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* solve_position_constraints (:230-287) */
static bool weld_solve_position(World& w, Joint& j) {
    Vec2 cA = w.pos[j.index_a].c;
    float aA = w.pos[j.index_a].a;
    Vec2 cB = w.pos[j.index_b].c;
    float aB = w.pos[j.index_b].a;
    const Rot qA = rot(aA), qB = rot(aB);
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
    const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
    float position_error, angular_error;
    const M33 K = weld_k(mA, mB, iA, iB, rA, rB);
    if (j.stiffness > 0.0f) {
        const Vec2 C1 = cB + rB - cA - rA;
        position_error = length(C1);
        angular_error = 0.0f;
        const Vec2 P = -m33_solve22(K, C1);
        cA -= mA * P;
        aA -= iA * cross(rA, P);
        cB += mB * P;
        aB += iB * cross(rB, P);
    } else {
        const Vec2 C1 = cB + rB - cA - rA;
        const float C2 = aB - aA - j.reference_angle;
        position_error = length(C1);
        angular_error = std::fabs(C2);
        const V3 C{C1.x, C1.y, C2};
        V3 impulse;
        if (K.ez.z > 0.0f) {
            const V3 x = m33_solve33(K, C);
            impulse = V3{-x.x, -x.y, -x.z};
        } else {
            const Vec2 i2 = -m33_solve22(K, C1);
            impulse = V3{i2.x, i2.y, 0.0f};
        }
        const Vec2 P = v2(impulse.x, impulse.y);
        cA -= mA * P;
        aA -= iA * (cross(rA, P) + impulse.z);
        cB += mB * P;
        aB += iB * (cross(rB, P) + impulse.z);
    }
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    return position_error <= kLinearSlop && angular_error <= kAngularSlop;
}

/* ---- friction joint, private/dynamics/joints/b2_friction_joint.rs ---- */

static void friction_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    j.r_a = mul(qA, j.local_anchor_a - j.lc_a);
    j.r_b = mul(qB, j.local_anchor_b - j.lc_b);
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    Mat22 K;
    K.ex.x = mA + mB + iA * j.r_a.y * j.r_a.y + iB * j.r_b.y * j.r_b.y;
    K.ex.y = -iA * j.r_a.x * j.r_a.y - iB * j.r_b.x * j.r_b.y;
    K.ey.x = K.ex.y;
    K.ey.y = mA + mB + iA * j.r_a.x * j.r_a.x + iB * j.r_b.x * j.r_b.x;
    j.linear_mass = inverse(K);
    j.angular_mass = iA + iB;
    if (j.angular_mass > 0.0f) j.angular_mass = 1.0f / j.angular_mass;
    if (step.warm) {
        j.linear_impulse *= step.dt_ratio;
        j.angular_impulse *= step.dt_ratio;
        const Vec2 P = v2(j.linear_impulse.x, j.linear_impulse.y);
        vA -= mA * P;
        wA -= iA * (cross(j.r_a, P) + j.angular_impulse);
        vB += mB * P;
        wB += iB * (cross(j.r_b, P) + j.angular_impulse);
    } else {
        j.linear_impulse = v2(0, 0);
        j.angular_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static void friction_solve_velocity(World& w, Joint& j, const Step& step) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const float h = step.dt;
    {
        const float cdot = wB - wA;
        float impulse = -j.angular_mass * cdot;
        const float old_impulse = j.angular_impulse;
        const float max_impulse = h * j.max_torque;
        j.angular_impulse = bclamp(j.angular_impulse + impulse, -max_impulse, max_impulse);
        impulse = j.angular_impulse - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        const Vec2 cdot = vB + cross_sv(wB, j.r_b) - vA - cross_sv(wA, j.r_a);
        Vec2 impulse = -mul(j.linear_mass, cdot);
        const Vec2 old_impulse = j.linear_impulse;
        j.linear_impulse += impulse;
        const float max_impulse = h * j.max_force;
        if (dot(j.linear_impulse, j.linear_impulse) > max_impulse * max_impulse) {
            normalize(j.linear_impulse);
            j.linear_impulse *= max_impulse;
        }
        impulse = j.linear_impulse - old_impulse;
        vA -= mA * impulse;
        wA -= iA * cross(j.r_a, impulse);
        vB += mB * impulse;
        wB += iB * cross(j.r_b, impulse);
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* ---- motor joint, private/dynamics/joints/b2_motor_joint.rs ---- */

static void motor_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const Vec2 cA = w.pos[j.index_a].c, cB = w.pos[j.index_b].c;
    const float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    j.r_a = mul(qA, j.linear_offset - j.lc_a);
    j.r_b = mul(qB, -j.lc_b);
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    Mat22 K;
    K.ex.x = mA + mB + iA * j.r_a.y * j.r_a.y + iB * j.r_b.y * j.r_b.y;
    K.ex.y = -iA * j.r_a.x * j.r_a.y - iB * j.r_b.x * j.r_b.y;
    K.ey.x = K.ex.y;
    K.ey.y = mA + mB + iA * j.r_a.x * j.r_a.x + iB * j.r_b.x * j.r_b.x;
    j.linear_mass = inverse(K);
    j.angular_mass = iA + iB;
    if (j.angular_mass > 0.0f) j.angular_mass = 1.0f / j.angular_mass;
    j.linear_error = cB + j.r_b - cA - j.r_a;
    j.angular_error = aB - aA - j.angular_offset;
    if (step.warm) {
        j.linear_impulse *= step.dt_ratio;
        j.angular_impulse *= step.dt_ratio;
        const Vec2 P = v2(j.linear_impulse.x, j.linear_impulse.y);
        vA -= mA * P;
        wA -= iA * (cross(j.r_a, P) + j.angular_impulse);
        vB += mB * P;
        wB += iB * (cross(j.r_b, P) + j.angular_impulse);
    } else {
        j.linear_impulse = v2(0, 0);
        j.angular_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static void motor_solve_velocity(World& w, Joint& j, const Step& step) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const float h = step.dt, inv_h = step.inv_dt;
    {
        const float cdot = wB - wA + inv_h * j.correction_factor * j.angular_error;
        float impulse = -j.angular_mass * cdot;
        const float old_impulse = j.angular_impulse;
        const float max_impulse = h * j.max_torque;
        j.angular_impulse = bclamp(j.angular_impulse + impulse, -max_impulse, max_impulse);
        impulse = j.angular_impulse - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        const Vec2 cdot = vB + cross_sv(wB, j.r_b) - vA - cross_sv(wA, j.r_a) +
                          (inv_h * j.correction_factor) * j.linear_error;
        Vec2 impulse = -mul(j.linear_mass, cdot);
        const Vec2 old_impulse = j.linear_impulse;
        j.linear_impulse += impulse;
        const float max_impulse = h * j.max_force;
        if (dot(j.linear_impulse, j.linear_impulse) > max_impulse * max_impulse) {
            normalize(j.linear_impulse);
            j.linear_impulse *= max_impulse;
        }
        impulse = j.linear_impulse - old_impulse;
        vA -= mA * impulse;
        wA -= iA * cross(j.r_a, impulse);
        vB += mB * impulse;
        wB += iB * cross(j.r_b, impulse);
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* ---- mouse joint, private/dynamics/joints/b2_mouse_joint.rs ---- */

static void mouse_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& B = w.bodies[j.body_b];
    j.index_b = B.island_index;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_b = B.inv_mass;
    j.inv_ib = B.inv_I;
    const Vec2 cB = w.pos[j.index_b].c;
    const float aB = w.pos[j.index_b].a;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qB = rot(aB);
    const float d = j.damping, k = j.stiffness, h = step.dt;
    j.gamma = h * (d + h * k);
    if (j.gamma != 0.0f) j.gamma = 1.0f / j.gamma;
    j.beta = h * k * j.gamma;
    j.r_b = mul(qB, j.local_anchor_b - j.lc_b);
    Mat22 K;
    K.ex.x = j.inv_mass_b + j.inv_ib * j.r_b.y * j.r_b.y + j.gamma;
    K.ex.y = -j.inv_ib * j.r_b.x * j.r_b.y;
    K.ey.x = K.ex.y;
    K.ey.y = j.inv_mass_b + j.inv_ib * j.r_b.x * j.r_b.x + j.gamma;
    j.linear_mass = inverse(K);
    j.mouse_c = cB + j.r_b - j.target;
    j.mouse_c *= j.beta;
    wB *= 0.98f;
    if (step.warm) {
        j.linear_impulse *= step.dt_ratio;
        vB += j.inv_mass_b * j.linear_impulse;
        wB += j.inv_ib * cross(j.r_b, j.linear_impulse);
    } else {
        j.linear_impulse = v2(0, 0);
    }
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static void mouse_solve_velocity(World& w, Joint& j, const Step& step) {
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Vec2 cdot = vB + cross_sv(wB, j.r_b);
    Vec2 impulse = mul(j.linear_mass, -(cdot + j.mouse_c + j.gamma * j.linear_impulse));
    const Vec2 old_impulse = j.linear_impulse;
    j.linear_impulse += impulse;
    const float max_impulse = step.dt * j.max_force;
    if (dot(j.linear_impulse, j.linear_impulse) > max_impulse * max_impulse)
        j.linear_impulse *= max_impulse / length(j.linear_impulse);
    impulse = j.linear_impulse - old_impulse;
    vB += j.inv_mass_b * impulse;
    wB += j.inv_ib * cross(j.r_b, impulse);
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* ---- prismatic joint, private/dynamics/joints/b2_prismatic_joint.rs:120-460 ---- */

static void prismatic_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const Vec2 cA = w.pos[j.index_a].c, cB = w.pos[j.index_b].c;
    const float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
    const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
    const Vec2 d = (cB - cA) + rB - rA;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    j.axis = mul(qA, j.local_xaxis_a);
    j.a1 = cross(d + rA, j.axis);
    j.a2 = cross(rB, j.axis);
    j.axial_mass = mA + mB + iA * j.a1 * j.a1 + iB * j.a2 * j.a2;
    if (j.axial_mass > 0.0f) j.axial_mass = 1.0f / j.axial_mass;
    j.perp = mul(qA, j.local_yaxis_a);
    j.s1 = cross(d + rA, j.perp);
    j.s2 = cross(rB, j.perp);
    const float k11 = mA + mB + iA * j.s1 * j.s1 + iB * j.s2 * j.s2;
    const float k12 = iA * j.s1 + iB * j.s2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    j.k.ex = v2(k11, k12);
    j.k.ey = v2(k12, k22);
    if (j.enable_limit) {
        j.translation = dot(j.axis, d);
    } else {
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    if (!j.enable_motor) j.motor_impulse = 0.0f;
    if (step.warm) {
        j.impulse *= step.dt_ratio;
        j.motor_impulse *= step.dt_ratio;
        j.lower_impulse *= step.dt_ratio;
        j.upper_impulse *= step.dt_ratio;
        const float axial = j.motor_impulse + j.lower_impulse - j.upper_impulse;
        const Vec2 P = j.impulse.x * j.perp + axial * j.axis;
        const float LA = j.impulse.x * j.s1 + j.impulse.y + axial * j.a1;
        const float LB = j.impulse.x * j.s2 + j.impulse.y + axial * j.a2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    } else {
        j.impulse = v2(0, 0);
        j.motor_impulse = 0.0f;
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static void prismatic_solve_velocity(World& w, Joint& j, const Step& step) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    if (j.enable_motor) {
        const float cdot = dot(j.axis, vB - vA) + j.a2 * wB - j.a1 * wA;
        float impulse = j.axial_mass * (j.motor_speed - cdot);
        const float old_impulse = j.motor_impulse;
        const float max_impulse = step.dt * j.max_motor_force;
        j.motor_impulse = bclamp(j.motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = j.motor_impulse - old_impulse;
        const Vec2 P = impulse * j.axis;
        const float LA = impulse * j.a1, LB = impulse * j.a2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    if (j.enable_limit) {
        {
            const float C = j.translation - j.lower_translation;
            const float cdot = dot(j.axis, vB - vA) + j.a2 * wB - j.a1 * wA;
            float impulse = -j.axial_mass * (cdot + bmax(C, 0.0f) * step.inv_dt);
            const float old_impulse = j.lower_impulse;
            j.lower_impulse = bmax(j.lower_impulse + impulse, 0.0f);
            impulse = j.lower_impulse - old_impulse;
            const Vec2 P = impulse * j.axis;
            const float LA = impulse * j.a1, LB = impulse * j.a2;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        }
        {
            const float C = j.upper_translation - j.translation;
            const float cdot = dot(j.axis, vA - vB) + j.a1 * wA - j.a2 * wB;
            float impulse = -j.axial_mass * (cdot + bmax(C, 0.0f) * step.inv_dt);
            const float old_impulse = j.upper_impulse;
            j.upper_impulse = bmax(j.upper_impulse + impulse, 0.0f);
            impulse = j.upper_impulse - old_impulse;
            const Vec2 P = impulse * j.axis;
            const float LA = impulse * j.a1, LB = impulse * j.a2;
            vA += mA * P;
            wA += iA * LA;
            vB -= mB * P;
            wB -= iB * LB;
        }
    }
    {
        const Vec2 cdot = v2(dot(j.perp, vB - vA) + j.s2 * wB - j.s1 * wA, wB - wA);
        const Vec2 df = solve(j.k, -cdot);
        j.impulse += df;
        const Vec2 P = df.x * j.perp;
        const float LA = df.x * j.s1 + df.y, LB = df.x * j.s2 + df.y;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static bool prismatic_solve_position(World& w, Joint& j) {
    Vec2 cA = w.pos[j.index_a].c;
    float aA = w.pos[j.index_a].a;
    Vec2 cB = w.pos[j.index_b].c;
    float aB = w.pos[j.index_b].a;
    const Rot qA = rot(aA), qB = rot(aB);
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
    const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
    const Vec2 d = cB + rB - cA - rA;
    const Vec2 axis = mul(qA, j.local_xaxis_a);
    const float a1 = cross(d + rA, axis), a2 = cross(rB, axis);
    const Vec2 perp = mul(qA, j.local_yaxis_a);
    const float s1 = cross(d + rA, perp), s2 = cross(rB, perp);
    const Vec2 C1 = v2(dot(perp, d), aB - aA - j.reference_angle);
    float linear_error = std::fabs(C1.x);
    const float angular_error = std::fabs(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (j.enable_limit) {
        const float translation = dot(axis, d);
        if (std::fabs(j.upper_translation - j.lower_translation) < 2.0f * kLinearSlop) {
            C2 = translation;
            linear_error = bmax(linear_error, std::fabs(translation));
            active = true;
        } else if (translation <= j.lower_translation) {
            C2 = bmin(translation - j.lower_translation, 0.0f);
            linear_error = bmax(linear_error, j.lower_translation - translation);
            active = true;
        } else if (translation >= j.upper_translation) {
            C2 = bmax(translation - j.upper_translation, 0.0f);
            linear_error = bmax(linear_error, translation - j.upper_translation);
            active = true;
        }
    }
    V3 impulse;
    if (active) {
        const float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
        const float k12 = iA * s1 + iB * s2;
        const float k13 = iA * s1 * a1 + iB * s2 * a2;
        float k22 = iA + iB;
        if (k22 == 0.0f) k22 = 1.0f;
        const float k23 = iA * a1 + iB * a2;
        const float k33 = mA + mB + iA * a1 * a1 + iB * a2 * a2;
        M33 K;
        K.ex = V3{k11, k12, k13};
        K.ey = V3{k12, k22, k23};
        K.ez = V3{k13, k23, k33};
        impulse = m33_solve33(K, V3{-C1.x, -C1.y, -C2});
    } else {
        const float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
        const float k12 = iA * s1 + iB * s2;
        float k22 = iA + iB;
        if (k22 == 0.0f) k22 = 1.0f;
        Mat22 K;
        K.ex = v2(k11, k12);
        K.ey = v2(k12, k22);
        const Vec2 i1 = solve(K, -C1);
        impulse = V3{i1.x, i1.y, 0.0f};
    }
    const Vec2 P = impulse.x * perp + impulse.z * axis;
    const float LA = impulse.x * s1 + impulse.y + impulse.z * a1;
    const float LB = impulse.x * s2 + impulse.y + impulse.z * a2;
    cA -= mA * P;
    aA -= iA * LA;
    cB += mB * P;
    aB += iB * LB;
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    return linear_error <= kLinearSlop && angular_error <= kAngularSlop;
}

/* ---- wheel joint, private/dynamics/joints/b2_wheel_joint.rs:24-398 ---- */

static void wheel_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const Vec2 cA = w.pos[j.index_a].c, cB = w.pos[j.index_b].c;
    const float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
    const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
    const Vec2 d = cB + rB - cA - rA;
    j.perp = mul(qA, j.local_yaxis_a);
    j.s1 = cross(d + rA, j.perp);
    j.s2 = cross(rB, j.perp);
    j.wheel_mass = mA + mB + iA * j.s1 * j.s1 + iB * j.s2 * j.s2;
    if (j.wheel_mass > 0.0f) j.wheel_mass = 1.0f / j.wheel_mass;
    j.axis = mul(qA, j.local_xaxis_a);
    j.a1 = cross(d + rA, j.axis);
    j.a2 = cross(rB, j.axis);
    const float inv_mass = mA + mB + iA * j.a1 * j.a1 + iB * j.a2 * j.a2;
    j.axial_mass = inv_mass > 0.0f ? 1.0f / inv_mass : 0.0f;
    j.spring_mass = 0.0f;
    j.bias = 0.0f;
    j.gamma = 0.0f;
    if (j.stiffness > 0.0f && inv_mass > 0.0f) {
        j.spring_mass = 1.0f / inv_mass;
        const float C = dot(d, j.axis);
        const float h = step.dt;
        j.gamma = h * (j.damping + h * j.stiffness);
        if (j.gamma > 0.0f) j.gamma = 1.0f / j.gamma;
        j.bias = C * h * j.stiffness * j.gamma;
        j.spring_mass = inv_mass + j.gamma;
        if (j.spring_mass > 0.0f) j.spring_mass = 1.0f / j.spring_mass;
    } else {
        j.spring_impulse = 0.0f;
    }
    if (j.enable_limit) {
        j.translation = dot(j.axis, d);
    } else {
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    if (j.enable_motor) {
        j.motor_mass = iA + iB;
        if (j.motor_mass > 0.0f) j.motor_mass = 1.0f / j.motor_mass;
    } else {
        j.motor_mass = 0.0f;
        j.motor_impulse = 0.0f;
    }
    if (step.warm) {
        j.wheel_impulse *= step.dt_ratio;
        j.spring_impulse *= step.dt_ratio;
        j.motor_impulse *= step.dt_ratio;
        const float axial = j.spring_impulse + j.lower_impulse - j.upper_impulse;
        const Vec2 P = j.wheel_impulse * j.perp + axial * j.axis;
        const float LA = j.wheel_impulse * j.s1 + axial * j.a1 + j.motor_impulse;
        const float LB = j.wheel_impulse * j.s2 + axial * j.a2 + j.motor_impulse;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    } else {
        j.wheel_impulse = 0.0f;
        j.spring_impulse = 0.0f;
        j.motor_impulse = 0.0f;
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static void wheel_solve_velocity(World& w, Joint& j, const Step& step) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    {
        const float cdot = dot(j.axis, vB - vA) + j.a2 * wB - j.a1 * wA;
        const float impulse = -j.spring_mass * (cdot + j.bias + j.gamma * j.spring_impulse);
        j.spring_impulse += impulse;
        const Vec2 P = impulse * j.axis;
        const float LA = impulse * j.a1, LB = impulse * j.a2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    {
        const float cdot = wB - wA - j.motor_speed;
        float impulse = -j.motor_mass * cdot;
        const float old_impulse = j.motor_impulse;
        const float max_impulse = step.dt * j.max_motor_torque;
        j.motor_impulse = bclamp(j.motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = j.motor_impulse - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    if (j.enable_limit) {
        {
            const float C = j.translation - j.lower_translation;
            const float cdot = dot(j.axis, vB - vA) + j.a2 * wB - j.a1 * wA;
            float impulse = -j.axial_mass * (cdot + bmax(C, 0.0f) * step.inv_dt);
            const float old_impulse = j.lower_impulse;
            j.lower_impulse = bmax(j.lower_impulse + impulse, 0.0f);
            impulse = j.lower_impulse - old_impulse;
            const Vec2 P = impulse * j.axis;
            const float LA = impulse * j.a1, LB = impulse * j.a2;
            vA -= mA * P;
            wA -= iA * LA;
            vB += mB * P;
            wB += iB * LB;
        }
        {
            const float C = j.upper_translation - j.translation;
            const float cdot = dot(j.axis, vA - vB) + j.a1 * wA - j.a2 * wB;
            float impulse = -j.axial_mass * (cdot + bmax(C, 0.0f) * step.inv_dt);
            const float old_impulse = j.upper_impulse;
            j.upper_impulse = bmax(j.upper_impulse + impulse, 0.0f);
            impulse = j.upper_impulse - old_impulse;
            const Vec2 P = impulse * j.axis;
            const float LA = impulse * j.a1, LB = impulse * j.a2;
            vA += mA * P;
            wA += iA * LA;
            vB -= mB * P;
            wB -= iB * LB;
        }
    }
    {
        const float cdot = dot(j.perp, vB - vA) + j.s2 * wB - j.s1 * wA;
        const float impulse = -j.wheel_mass * cdot;
        j.wheel_impulse += impulse;
        const Vec2 P = impulse * j.perp;
        const float LA = impulse * j.s1, LB = impulse * j.s2;
        vA -= mA * P;
        wA -= iA * LA;
        vB += mB * P;
        wB += iB * LB;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static bool wheel_solve_position(World& w, Joint& j) {
    Vec2 cA = w.pos[j.index_a].c;
    float aA = w.pos[j.index_a].a;
    Vec2 cB = w.pos[j.index_b].c;
    float aB = w.pos[j.index_b].a;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    float linear_error = 0.0f;
    if (j.enable_limit) {
        const Rot qA = rot(aA), qB = rot(aB);
        const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
        const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
        const Vec2 d = (cB - cA) + rB - rA;
        const Vec2 ax = mul(qA, j.local_xaxis_a);
        const float s_ax = cross(d + rA, j.axis), s_bx = cross(rB, j.axis);
        float C = 0.0f;
        const float translation = dot(ax, d);
        if (std::fabs(j.upper_translation - j.lower_translation) < 2.0f * kLinearSlop) C = translation;
        else if (translation <= j.lower_translation) C = bmin(translation - j.lower_translation, 0.0f);
        else if (translation >= j.upper_translation) C = bmax(translation - j.upper_translation, 0.0f);
        if (C != 0.0f) {
            const float inv_mass = mA + mB + iA * s_ax * s_ax + iB * s_bx * s_bx;
            float impulse = 0.0f;
            if (inv_mass != 0.0f) impulse = -C / inv_mass;
            const Vec2 P = impulse * ax;
            const float LA = impulse * s_ax, LB = impulse * s_bx;
            cA -= mA * P;
            aA -= iA * LA;
            cB += mB * P;
            aB += iB * LB;
            linear_error = std::fabs(C);
        }
    }
    {
        const Rot qA = rot(aA), qB = rot(aB);
        const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
        const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
        const Vec2 d = (cB - cA) + rB - rA;
        const Vec2 ay = mul(qA, j.local_yaxis_a);
        const float s_ay = cross(d + rA, ay), s_by = cross(rB, ay);
        const float C = dot(d, ay);
        const float inv_mass = mA + mB + iA * j.s1 * j.s1 + iB * j.s2 * j.s2;
        float impulse = 0.0f;
        if (inv_mass != 0.0f) impulse = -C / inv_mass;
        const Vec2 P = impulse * ay;
        const float LA = impulse * s_ay, LB = impulse * s_by;
        cA -= mA * P;
        aA -= iA * LA;
        cB += mB * P;
        aB += iB * LB;
        linear_error = bmax(linear_error, std::fabs(C));
    }
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    return linear_error <= kLinearSlop;
}

/* ---- pulley joint, private/dynamics/joints/b2_pulley_joint.rs ---- */

static float pulley_dir(Vec2& u) {
    const float len = length(u);
    if (len > 10.0f * kLinearSlop) u *= 1.0f / len;
    else u = v2(0, 0);
    return len;
}

static void pulley_init_velocity(World& w, Joint& j, const Step& step) {
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const Vec2 cA = w.pos[j.index_a].c, cB = w.pos[j.index_b].c;
    const float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    j.r_a = mul(qA, j.local_anchor_a - j.lc_a);
    j.r_b = mul(qB, j.local_anchor_b - j.lc_b);
    j.u_a = cA + j.r_a - j.ground_a;
    j.u_b = cB + j.r_b - j.ground_b;
    pulley_dir(j.u_a);
    pulley_dir(j.u_b);
    const float ruA = cross(j.r_a, j.u_a), ruB = cross(j.r_b, j.u_b);
    const float mA = j.inv_mass_a + j.inv_ia * ruA * ruA;
    const float mB = j.inv_mass_b + j.inv_ib * ruB * ruB;
    j.pulley_mass = mA + j.ratio * j.ratio * mB;
    if (j.pulley_mass > 0.0f) j.pulley_mass = 1.0f / j.pulley_mass;
    if (step.warm) {
        j.pulley_impulse *= step.dt_ratio;
        const Vec2 PA = (-j.pulley_impulse) * j.u_a;
        const Vec2 PB = (-j.ratio * j.pulley_impulse) * j.u_b;
        vA += j.inv_mass_a * PA;
        wA += j.inv_ia * cross(j.r_a, PA);
        vB += j.inv_mass_b * PB;
        wB += j.inv_ib * cross(j.r_b, PB);
    } else {
        j.pulley_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static void pulley_solve_velocity(World& w, Joint& j) {
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Vec2 vpA = vA + cross_sv(wA, j.r_a);
    const Vec2 vpB = vB + cross_sv(wB, j.r_b);
    const float cdot = -dot(j.u_a, vpA) - j.ratio * dot(j.u_b, vpB);
    const float impulse = -j.pulley_mass * cdot;
    j.pulley_impulse += impulse;
    const Vec2 PA = -impulse * j.u_a;
    const Vec2 PB = -j.ratio * impulse * j.u_b;
    vA += j.inv_mass_a * PA;
    wA += j.inv_ia * cross(j.r_a, PA);
    vB += j.inv_mass_b * PB;
    wB += j.inv_ib * cross(j.r_b, PB);
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

static bool pulley_solve_position(World& w, Joint& j) {
    Vec2 cA = w.pos[j.index_a].c;
    float aA = w.pos[j.index_a].a;
    Vec2 cB = w.pos[j.index_b].c;
    float aB = w.pos[j.index_b].a;
    const Rot qA = rot(aA), qB = rot(aB);
    const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
    const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
    Vec2 uA = cA + rA - j.ground_a;
    Vec2 uB = cB + rB - j.ground_b;
    const float lenA = pulley_dir(uA), lenB = pulley_dir(uB);
    const float ruA = cross(rA, uA), ruB = cross(rB, uB);
    const float mA = j.inv_mass_a + j.inv_ia * ruA * ruA;
    const float mB = j.inv_mass_b + j.inv_ib * ruB * ruB;
    float mass = mA + j.ratio * j.ratio * mB;
    if (mass > 0.0f) mass = 1.0f / mass;
    const float C = j.pulley_constant - lenA - j.ratio * lenB;
    const float linear_error = std::fabs(C);
    const float impulse = -mass * C;
    const Vec2 PA = -impulse * uA;
    const Vec2 PB = -j.ratio * impulse * uB;
    cA += j.inv_mass_a * PA;
    aA += j.inv_ia * cross(rA, PA);
    cB += j.inv_mass_b * PB;
    aB += j.inv_ib * cross(rB, PB);
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    return linear_error < kLinearSlop;
}

/* init_velocity_constraints (:21-116): anchors, effective masses, warm start */
/* ---- gear joint, private/dynamics/joints/b2_gear_joint.rs ---- */

/* the Jacobian rows and the (not yet inverted) mass of :209-241 and :326-359 */
static float gear_jacobian(Joint& j, const Rot& qA, const Rot& qB, const Rot& qC, const Rot& qD, Vec2& jv_ac,
                           Vec2& jv_bd, float& jw_a, float& jw_b, float& jw_c, float& jw_d) {
    float mass = 0.0f;
    if (!j.gear_prismatic_a) {
        jv_ac = v2(0, 0);
        jw_a = 1.0f;
        jw_c = 1.0f;
        mass += j.inv_ia + j.inv_ic;
    } else {
        const Vec2 u = mul(qC, j.gear_axis_c);
        const Vec2 rC = mul(qC, j.gear_anchor_c - j.lc_c);
        const Vec2 rA = mul(qA, j.gear_anchor_a - j.lc_a);
        jv_ac = u;
        jw_c = cross(rC, u);
        jw_a = cross(rA, u);
        mass += j.inv_mass_c + j.inv_mass_a + j.inv_ic * jw_c * jw_c + j.inv_ia * jw_a * jw_a;
    }
    if (!j.gear_prismatic_b) {
        jv_bd = v2(0, 0);
        jw_b = j.ratio;
        jw_d = j.ratio;
        mass += j.ratio * j.ratio * (j.inv_ib + j.inv_id);
    } else {
        const Vec2 u = mul(qD, j.gear_axis_d);
        const Vec2 rD = mul(qD, j.gear_anchor_d - j.lc_d);
        const Vec2 rB = mul(qB, j.gear_anchor_b - j.lc_b);
        jv_bd = j.ratio * u;
        jw_d = j.ratio * cross(rD, u);
        jw_b = j.ratio * cross(rB, u);
        mass += j.ratio * j.ratio * (j.inv_mass_d + j.inv_mass_b) + j.inv_id * jw_d * jw_d + j.inv_ib * jw_b * jw_b;
    }
    return mass;
}

/* the four island velocities changed by impulse (:264-273, :300-307): read all, write A, B, C, D */
static void gear_apply_velocity(World& w, const Joint& j, float impulse) {
    Vec2 vA = w.vel[j.index_a].v, vB = w.vel[j.index_b].v, vC = w.vel[j.index_c].v, vD = w.vel[j.index_d].v;
    float wA = w.vel[j.index_a].w, wB = w.vel[j.index_b].w, wC = w.vel[j.index_c].w, wD = w.vel[j.index_d].w;
    vA += (j.inv_mass_a * impulse) * j.jv_ac;
    wA += j.inv_ia * impulse * j.jw_a;
    vB += (j.inv_mass_b * impulse) * j.jv_bd;
    wB += j.inv_ib * impulse * j.jw_b;
    vC -= (j.inv_mass_c * impulse) * j.jv_ac;
    wC -= j.inv_ic * impulse * j.jw_c;
    vD -= (j.inv_mass_d * impulse) * j.jv_bd;
    wD -= j.inv_id * impulse * j.jw_d;
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
    w.vel[j.index_c].v = vC;
    w.vel[j.index_c].w = wC;
    w.vel[j.index_d].v = vD;
    w.vel[j.index_d].w = wD;
}

/* init_velocity_constraints, :190-289 */
static void gear_init_velocity(World& w, Joint& j, const Step& step) {
    const Body* bs[4] = {&w.bodies[j.body_a], &w.bodies[j.body_b], &w.bodies[j.body_c], &w.bodies[j.body_d]};
    j.index_a = bs[0]->island_index;
    j.index_b = bs[1]->island_index;
    j.index_c = bs[2]->island_index;
    j.index_d = bs[3]->island_index;
    j.lc_a = bs[0]->sweep.local_center;
    j.lc_b = bs[1]->sweep.local_center;
    j.lc_c = bs[2]->sweep.local_center;
    j.lc_d = bs[3]->sweep.local_center;
    j.inv_mass_a = bs[0]->inv_mass;
    j.inv_mass_b = bs[1]->inv_mass;
    j.inv_mass_c = bs[2]->inv_mass;
    j.inv_mass_d = bs[3]->inv_mass;
    j.inv_ia = bs[0]->inv_I;
    j.inv_ib = bs[1]->inv_I;
    j.inv_ic = bs[2]->inv_I;
    j.inv_id = bs[3]->inv_I;
    const Rot qA = rot(w.pos[j.index_a].a), qB = rot(w.pos[j.index_b].a), qC = rot(w.pos[j.index_c].a),
              qD = rot(w.pos[j.index_d].a);
    j.gear_mass = gear_jacobian(j, qA, qB, qC, qD, j.jv_ac, j.jv_bd, j.jw_a, j.jw_b, j.jw_c, j.jw_d);
    j.gear_mass = j.gear_mass > 0.0f ? 1.0f / j.gear_mass : 0.0f;
    if (step.warm) gear_apply_velocity(w, j, j.gear_impulse);
    else j.gear_impulse = 0.0f;
}

/* solve_velocity_constraints, :291-319 */
static void gear_solve_velocity(World& w, Joint& j) {
    const Velocity A = w.vel[j.index_a], B = w.vel[j.index_b], C = w.vel[j.index_c], D = w.vel[j.index_d];
    float cdot = dot(j.jv_ac, A.v - C.v) + dot(j.jv_bd, B.v - D.v);
    cdot += (j.jw_a * A.w - j.jw_c * C.w) + (j.jw_b * B.w - j.jw_d * D.w);
    const float impulse = -j.gear_mass * cdot;
    j.gear_impulse += impulse;
    gear_apply_velocity(w, j, impulse);
}

/* solve_position_constraints, :321-393 */
static bool gear_solve_position(World& w, Joint& j) {
    Vec2 cA = w.pos[j.index_a].c, cB = w.pos[j.index_b].c, cC = w.pos[j.index_c].c, cD = w.pos[j.index_d].c;
    float aA = w.pos[j.index_a].a, aB = w.pos[j.index_b].a, aC = w.pos[j.index_c].a, aD = w.pos[j.index_d].a;
    const Rot qA = rot(aA), qB = rot(aB), qC = rot(aC), qD = rot(aD);
    Vec2 jv_ac, jv_bd;
    float jw_a, jw_b, jw_c, jw_d;
    const float mass = gear_jacobian(j, qA, qB, qC, qD, jv_ac, jv_bd, jw_a, jw_b, jw_c, jw_d);
    float coordinate_a, coordinate_b;
    if (!j.gear_prismatic_a) {
        coordinate_a = aA - aC - j.gear_ref_a;
    } else {
        const Vec2 rA = mul(qA, j.gear_anchor_a - j.lc_a);
        const Vec2 p_c = j.gear_anchor_c - j.lc_c;
        const Vec2 p_a = mul_t(qC, rA + (cA - cC));
        coordinate_a = dot(p_a - p_c, j.gear_axis_c);
    }
    if (!j.gear_prismatic_b) {
        coordinate_b = aB - aD - j.gear_ref_b;
    } else {
        const Vec2 rB = mul(qB, j.gear_anchor_b - j.lc_b);
        const Vec2 p_d = j.gear_anchor_d - j.lc_d;
        const Vec2 p_b = mul_t(qD, rB + (cB - cD));
        coordinate_b = dot(p_b - p_d, j.gear_axis_d);
    }
    const float C = (coordinate_a + j.ratio * coordinate_b) - j.gear_constant;
    float impulse = 0.0f;
    if (mass > 0.0f) impulse = -C / mass;
    cA += j.inv_mass_a * impulse * jv_ac;
    aA += j.inv_ia * impulse * jw_a;
    cB += j.inv_mass_b * impulse * jv_bd;
    aB += j.inv_ib * impulse * jw_b;
    cC -= j.inv_mass_c * impulse * jv_ac;
    aC -= j.inv_ic * impulse * jw_c;
    cD -= j.inv_mass_d * impulse * jv_bd;
    aD -= j.inv_id * impulse * jw_d;
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    w.pos[j.index_c].c = cC;
    w.pos[j.index_c].a = aC;
    w.pos[j.index_d].c = cD;
    w.pos[j.index_d].a = aD;
    return true;  /* the linear error is never measured (:392-393) */
}

static void joint_init_velocity(World& w, Joint& j, const Step& step) {
    if (j.type == B2G_JOINT_GEAR) {
        gear_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_MOTOR) {
        motor_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_MOUSE) {
        mouse_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_PRISMATIC) {
        prismatic_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_WHEEL) {
        wheel_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_PULLEY) {
        pulley_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_FRICTION) {
        friction_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_WELD) {
        weld_init_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_DISTANCE) {
        distance_init_velocity(w, j, step);
        return;
    }
    const Body& A = w.bodies[j.body_a];
    const Body& B = w.bodies[j.body_b];
    j.index_a = A.island_index;
    j.index_b = B.island_index;
    j.lc_a = A.sweep.local_center;
    j.lc_b = B.sweep.local_center;
    j.inv_mass_a = A.inv_mass;
    j.inv_mass_b = B.inv_mass;
    j.inv_ia = A.inv_I;
    j.inv_ib = B.inv_I;
    const float aA = w.pos[j.index_a].a;
    const float aB = w.pos[j.index_b].a;
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const Rot qA = rot(aA), qB = rot(aB);
    j.r_a = mul(qA, j.local_anchor_a - j.lc_a);
    j.r_b = mul(qB, j.local_anchor_b - j.lc_b);
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    j.k.ex.x = mA + mB + j.r_a.y * j.r_a.y * iA + j.r_b.y * j.r_b.y * iB;
    j.k.ey.x = -j.r_a.y * j.r_a.x * iA - j.r_b.y * j.r_b.x * iB;
    j.k.ex.y = j.k.ey.x;
    j.k.ey.y = mA + mB + j.r_a.x * j.r_a.x * iA + j.r_b.x * j.r_b.x * iB;
    j.axial_mass = iA + iB;
    bool fixed_rotation;
    if (j.axial_mass > 0.0f) {
        j.axial_mass = 1.0f / j.axial_mass;
        fixed_rotation = false;
    } else {
        fixed_rotation = true;
    }
    j.angle = aB - aA - j.reference_angle;
    if (!j.enable_limit || fixed_rotation) {
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    if (!j.enable_motor || fixed_rotation) j.motor_impulse = 0.0f;
    if (step.warm) {
        j.impulse *= step.dt_ratio;
        j.motor_impulse *= step.dt_ratio;
        j.lower_impulse *= step.dt_ratio;
        j.upper_impulse *= step.dt_ratio;
        const float axial = j.motor_impulse + j.lower_impulse - j.upper_impulse;
        const Vec2 P = v2(j.impulse.x, j.impulse.y);
        vA -= mA * P;
        wA -= iA * (cross(j.r_a, P) + axial);
        vB += mB * P;
        wB += iB * (cross(j.r_b, P) + axial);
    } else {
        j.impulse = v2(0, 0);
        j.motor_impulse = 0.0f;
        j.lower_impulse = 0.0f;
        j.upper_impulse = 0.0f;
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* solve_velocity_constraints (:118-208): motor, lower and upper limits, point */
static void joint_solve_velocity(World& w, Joint& j, const Step& step) {
    if (j.type == B2G_JOINT_GEAR) {
        gear_solve_velocity(w, j);
        return;
    }
    if (j.type == B2G_JOINT_MOTOR) {
        motor_solve_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_MOUSE) {
        mouse_solve_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_PRISMATIC) {
        prismatic_solve_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_WHEEL) {
        wheel_solve_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_PULLEY) {
        pulley_solve_velocity(w, j);
        return;
    }
    if (j.type == B2G_JOINT_FRICTION) {
        friction_solve_velocity(w, j, step);
        return;
    }
    if (j.type == B2G_JOINT_WELD) {
        weld_solve_velocity(w, j);
        return;
    }
    if (j.type == B2G_JOINT_DISTANCE) {
        distance_solve_velocity(w, j, step);
        return;
    }
    Vec2 vA = w.vel[j.index_a].v;
    float wA = w.vel[j.index_a].w;
    Vec2 vB = w.vel[j.index_b].v;
    float wB = w.vel[j.index_b].w;
    const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
    const bool fixed_rotation = iA + iB == 0.0f;
    if (j.enable_motor && !fixed_rotation) {
        const float cdot = wB - wA - j.motor_speed;
        float impulse = -j.axial_mass * cdot;
        const float old_impulse = j.motor_impulse;
        const float max_impulse = step.dt * j.max_motor_torque;
        j.motor_impulse = bclamp(j.motor_impulse + impulse, -max_impulse, max_impulse);
        impulse = j.motor_impulse - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    if (j.enable_limit && !fixed_rotation) {
        {
            const float C = j.angle - j.lower_angle;
            const float cdot = wB - wA;
            float impulse = -j.axial_mass * (cdot + bmax(C, 0.0f) * step.inv_dt);
            const float old_impulse = j.lower_impulse;
            j.lower_impulse = bmax(j.lower_impulse + impulse, 0.0f);
            impulse = j.lower_impulse - old_impulse;
            wA -= iA * impulse;
            wB += iB * impulse;
        }
        {
            const float C = j.upper_angle - j.angle;
            const float cdot = wA - wB;
            float impulse = -j.axial_mass * (cdot + bmax(C, 0.0f) * step.inv_dt);
            const float old_impulse = j.upper_impulse;
            j.upper_impulse = bmax(j.upper_impulse + impulse, 0.0f);
            impulse = j.upper_impulse - old_impulse;
            wA += iA * impulse;
            wB -= iB * impulse;
        }
    }
    {
        const Vec2 cdot = vB + cross_sv(wB, j.r_b) - vA - cross_sv(wA, j.r_a);
        const Vec2 impulse = solve(j.k, -cdot);
        j.impulse.x += impulse.x;
        j.impulse.y += impulse.y;
        vA -= mA * impulse;
        wA -= iA * cross(j.r_a, impulse);
        vB += mB * impulse;
        wB += iB * cross(j.r_b, impulse);
    }
    w.vel[j.index_a].v = vA;
    w.vel[j.index_a].w = wA;
    w.vel[j.index_b].v = vB;
    w.vel[j.index_b].w = wB;
}

/* solve_position_constraints (:210-287): angular limit, then the point */
static bool joint_solve_position(World& w, Joint& j) {
    if (j.type == B2G_JOINT_GEAR) return gear_solve_position(w, j);
    if (j.type == B2G_JOINT_DISTANCE) return distance_solve_position(w, j);
    if (j.type == B2G_JOINT_WELD) return weld_solve_position(w, j);
    /* b2_friction_joint.rs, b2_motor_joint.rs and b2_mouse_joint.rs: no position correction */
    if (j.type == B2G_JOINT_FRICTION || j.type == B2G_JOINT_MOTOR || j.type == B2G_JOINT_MOUSE) return true;
    if (j.type == B2G_JOINT_PRISMATIC) return prismatic_solve_position(w, j);
    if (j.type == B2G_JOINT_WHEEL) return wheel_solve_position(w, j);
    if (j.type == B2G_JOINT_PULLEY) return pulley_solve_position(w, j);
    Vec2 cA = w.pos[j.index_a].c;
    float aA = w.pos[j.index_a].a;
    Vec2 cB = w.pos[j.index_b].c;
    float aB = w.pos[j.index_b].a;
    float angular_error = 0.0f;
    const bool fixed_rotation = j.inv_ia + j.inv_ib == 0.0f;
    if (j.enable_limit && !fixed_rotation) {
        const float angle = aB - aA - j.reference_angle;
        float C = 0.0f;
        if (std::fabs(j.upper_angle - j.lower_angle) < 2.0f * kAngularSlop) {
            C = bclamp(angle - j.lower_angle, -kMaxAngularCorrection, kMaxAngularCorrection);
        } else if (angle <= j.lower_angle) {
            C = bclamp(angle - j.lower_angle + kAngularSlop, -kMaxAngularCorrection, 0.0f);
        } else if (angle >= j.upper_angle) {
            C = bclamp(angle - j.upper_angle - kAngularSlop, 0.0f, kMaxAngularCorrection);
        }
        const float limit_impulse = -j.axial_mass * C;
        aA -= j.inv_ia * limit_impulse;
        aB += j.inv_ib * limit_impulse;
        angular_error = std::fabs(C);
    }
    float position_error;
    {
        const Rot qA = rot(aA), qB = rot(aB);
        const Vec2 rA = mul(qA, j.local_anchor_a - j.lc_a);
        const Vec2 rB = mul(qB, j.local_anchor_b - j.lc_b);
        const Vec2 C = cB + rB - cA - rA;
        position_error = length(C);
        const float mA = j.inv_mass_a, mB = j.inv_mass_b, iA = j.inv_ia, iB = j.inv_ib;
        Mat22 K;
        K.ex.x = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
        K.ex.y = -iA * rA.x * rA.y - iB * rB.x * rB.y;
        K.ey.x = K.ex.y;
        K.ey.y = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
        const Vec2 impulse = -solve(K, C);
        cA -= mA * impulse;
        aA -= iA * cross(rA, impulse);
        cB += mB * impulse;
        aB += iB * cross(rB, impulse);
    }
    w.pos[j.index_a].c = cA;
    w.pos[j.index_a].a = aA;
    w.pos[j.index_b].c = cB;
    w.pos[j.index_b].a = aB;
    return position_error <= kLinearSlop && angular_error <= kAngularSlop;
}

/* B2island::solve, b2_island_private.rs:129-328 */
static void solve_island(World& w, const Step& step) {
    float h = step.dt;
    int nb = (int)w.isl_bodies.size();
    w.pos.resize(nb);
    w.vel.resize(nb);
    for (int i = 0; i < nb; ++i) {
        Body& b = w.bodies[w.isl_bodies[i]];
        Vec2 c = b.sweep.c;
        float a = b.sweep.a;
        Vec2 v = b.v;
        float wv = b.w;
        b.sweep.c0 = b.sweep.c;
        b.sweep.a0 = b.sweep.a;
        if (b.type == DYNAMIC) {
            v += (h * b.inv_mass) * ((b.grav_scale * b.mass) * w.gravity + b.force);
            wv += h * b.inv_I * b.torque;
            v *= 1.0f / (1.0f + h * b.lin_damp);
            wv *= 1.0f / (1.0f + h * b.ang_damp);
        }
        w.pos[i].c = c;
        w.pos[i].a = a;
        w.vel[i].v = v;
        w.vel[i].w = wv;
    }
    init_constraints(w, step);
    if (step.warm) warm_start(w);
    for (int ji : w.isl_joints) joint_init_velocity(w, w.joints[ji], step);
    for (int it = 0; it < step.vi; ++it) {
        for (int ji : w.isl_joints) joint_solve_velocity(w, w.joints[ji], step);
        solve_velocity(w);
    }
    store_impulses(w);
    /* B2island::report (b2_island_private.rs:460-487): each island contact's impulses after the
     * velocity iterations, point count as solved (a 2-point manifold solved as 1 reports 1) */
    for (const VelocityConstraint& vc : w.vcs) {
        const Contact& c = w.contacts[w.isl_contacts[vc.contact]];
        b2g_contact_impulse r{};
        r.fixture_a = (uint32_t)c.fa;
        r.fixture_b = (uint32_t)c.fb;
        r.count = vc.count;
        for (int j = 0; j < vc.count; ++j) {
            r.normal_impulses[j] = vc.p[j].ni;
            r.tangent_impulses[j] = vc.p[j].ti;
        }
        w.post_solve.push_back(r);
    }
    for (int i = 0; i < nb; ++i) {
        Vec2 c = w.pos[i].c;
        float a = w.pos[i].a;
        Vec2 v = w.vel[i].v;
        float wv = w.vel[i].w;
        Vec2 translation = h * v;
        if (dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = kMaxTranslation / length(translation);
            v *= ratio;
        }
        float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = kMaxRotation / std::fabs(rotation);
            wv *= ratio;
        }
        c += h * v;
        a += h * wv;
        w.pos[i].c = c;
        w.pos[i].a = a;
        w.vel[i].v = v;
        w.vel[i].w = wv;
    }
    bool positionSolved = false;
    for (int it = 0; it < step.pi; ++it) {
        const bool contacts_okay = solve_position(w);
        bool joints_okay = true;
        for (int ji : w.isl_joints) {
            const bool ok = joint_solve_position(w, w.joints[ji]);
            joints_okay = joints_okay && ok;
        }
        if (contacts_okay && joints_okay) {
            positionSolved = true;
            break;
        }
    }
    for (int i = 0; i < nb; ++i) {
        Body& b = w.bodies[w.isl_bodies[i]];
        b.sweep.c = w.pos[i].c;
        b.sweep.a = w.pos[i].a;
        b.v = w.vel[i].v;
        b.w = w.vel[i].w;
        synchronize_transform(b);
    }
    if (w.allow_sleep) {
        float minSleepTime = kMaxFloat;
        const float linTolSqr = kLinearSleepTolerance * kLinearSleepTolerance;
        const float angTolSqr = kAngularSleepTolerance * kAngularSleepTolerance;
        for (int i = 0; i < nb; ++i) {
            Body& b = w.bodies[w.isl_bodies[i]];
            if (b.type == STATIC) continue;
            if (!b.auto_sleep || b.w * b.w > angTolSqr || dot(b.v, b.v) > linTolSqr) {
                b.sleep_time = 0.0f;
                minSleepTime = 0.0f;
            } else {
                b.sleep_time += h;
                minSleepTime = bmin(minSleepTime, b.sleep_time);
            }
        }
        if (minSleepTime >= kTimeToSleep && positionSolved) {
            for (int i = 0; i < nb; ++i) set_awake(w.bodies[w.isl_bodies[i]], false);
        }
    }
}

/* B2world::solve, private/dynamics/b2_world.rs:356-531 */
static void solve(World& w, const Step& step) {
    for (int b = w.body_head; b >= 0; b = w.bodies[b].next) w.bodies[b].island_flag = false;
    for (int c = w.contact_head; c >= 0; c = w.contacts[c].next) w.contacts[c].island_flag = false;
    for (int j = w.joint_head; j >= 0; j = w.joints[j].next) w.joints[j].island_flag = false;
    w.last_order.clear();
    w.islands_solved = 0;
    for (int seed = w.body_head; seed >= 0; seed = w.bodies[seed].next) {
        Body& S = w.bodies[seed];
        if (S.island_flag) continue;
        if (!S.awake || !S.enabled) continue;
        if (S.type == STATIC) continue;
        w.isl_bodies.clear();
        w.isl_contacts.clear();
        w.isl_joints.clear();
        w.stack.clear();
        w.stack.push_back(seed);
        S.island_flag = true;
        while (!w.stack.empty()) {
            int bi = w.stack.back();
            w.stack.pop_back();
            Body& b = w.bodies[bi];
            b.island_index = (int)w.isl_bodies.size();
            w.isl_bodies.push_back(bi);
            if (b.type == STATIC) continue;
            b.awake = true;
            for (int e = b.edge_head; e >= 0; e = w.edges[e].next) {
                int ci = w.edges[e].contact;
                Contact& c = w.contacts[ci];
                if (c.island_flag) continue;
                if (!c.enabled || !c.touching) continue;
                if (w.fixtures[c.fa].sensor || w.fixtures[c.fb].sensor) continue;
                w.isl_contacts.push_back(ci);
                c.island_flag = true;
                int other = w.edges[e].other;
                if (w.bodies[other].island_flag) continue;
                w.stack.push_back(other);
                w.bodies[other].island_flag = true;
            }
            for (int e = b.jedge_head; e >= 0; e = w.jedges[e].next) {
                Joint& J = w.joints[w.jedges[e].joint];
                if (J.island_flag) continue;
                const int other = w.jedges[e].other;
                if (!w.bodies[other].enabled) continue;
                w.isl_joints.push_back(w.jedges[e].joint);
                J.island_flag = true;
                if (w.bodies[other].island_flag) continue;
                w.stack.push_back(other);
                w.bodies[other].island_flag = true;
            }
        }
        if (!w.joint_rank.empty()) {
            /* joint ordering hook: this island's joints in the caller's order */
            std::stable_sort(w.isl_joints.begin(), w.isl_joints.end(),
                             [&](int x, int y) { return w.joint_rank[x] < w.joint_rank[y]; });
        }
        if (w.hook) {
            /* ordering hook: solve this island's contacts in the caller's order */
            std::stable_sort(w.isl_contacts.begin(), w.isl_contacts.end(), [&](int x, int y) {
                auto ix = w.hook_rank.find(pair_key(w.contacts[x].fa, w.contacts[x].fb));
                auto iy = w.hook_rank.find(pair_key(w.contacts[y].fa, w.contacts[y].fb));
                int rx = ix == w.hook_rank.end() ? 0x7fffffff : ix->second;
                int ry = iy == w.hook_rank.end() ? 0x7fffffff : iy->second;
                return rx < ry;
            });
            for (int ci : w.isl_contacts)
                if (w.hook_rank.find(pair_key(w.contacts[ci].fa, w.contacts[ci].fb)) == w.hook_rank.end()) ++w.hook_misses;
        }
        for (int ci : w.isl_contacts) w.last_order.push_back(pair_key(w.contacts[ci].fa, w.contacts[ci].fb));
        solve_island(w, step);
        ++w.islands_solved;
        for (int bi : w.isl_bodies)
            if (w.bodies[bi].type == STATIC) w.bodies[bi].island_flag = false;
    }
    auto t0 = std::chrono::steady_clock::now();
    for (int b = w.body_head; b >= 0; b = w.bodies[b].next) {
        Body& B = w.bodies[b];
        if (!B.island_flag) continue;
        if (B.type == STATIC) continue;
        synchronize_fixtures(w, B);
    }
    find_new_contacts(w);
    w.profile.broadphase = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

/* ---- continuous physics ---- */

/* B2Sweep::advance, src/b2_math.rs:773-779 */
static void sweep_advance(Sweep& s, float alpha) {
    const float beta = (alpha - s.alpha0) / (1.0f - s.alpha0);
    s.c0 += beta * (s.c - s.c0);
    s.a0 += beta * (s.a - s.a0);
    s.alpha0 = alpha;
}

/* B2body::advance, src/b2_body.rs:979-986 */
static void body_advance(Body& b, float alpha) {
    sweep_advance(b.sweep, alpha);
    b.sweep.c = b.sweep.c0;
    b.sweep.a = b.sweep.a0;
    b.xf.q = rot(b.sweep.a);
    b.xf.p = b.sweep.c - mul(b.xf.q, b.sweep.local_center);
}

/* the contact's key in the GPU's contact table: (smaller proxy id, larger proxy id) */
static uint64_t contact_proxy_key(const World& w, const Contact& c) {
    uint32_t p = (uint32_t)w.fixtures[c.fa].proxy, q = (uint32_t)w.fixtures[c.fb].proxy;
    if (p > q) std::swap(p, q);
    return ((uint64_t)p << 32) | q;
}

/* solve_toi_position_constraints, b2_contact_solver_private.rs:733-823: only the two bodies of
 * the event move */
static bool solve_toi_position(World& w, int toiA, int toiB) {
    float minSeparation = 0.0f;
    for (const PositionConstraint& pc : w.pcs) {
        Vec2 lcA = pc.lcA, lcB = pc.lcB;
        float mA = 0.0f, iA = 0.0f;
        if (pc.ia == toiA || pc.ia == toiB) {
            mA = pc.ma;
            iA = pc.IA;
        }
        float mB = 0.0f, iB = 0.0f;
        if (pc.ib == toiA || pc.ib == toiB) {
            mB = pc.mb;
            iB = pc.IB;
        }
        Vec2 cA = w.pos[pc.ia].c;
        float aA = w.pos[pc.ia].a;
        Vec2 cB = w.pos[pc.ib].c;
        float aB = w.pos[pc.ib].a;
        for (int j = 0; j < pc.count; ++j) {
            Xf xfA, xfB;
            xfA.q = rot(aA);
            xfB.q = rot(aB);
            xfA.p = cA - mul(xfA.q, lcA);
            xfB.p = cB - mul(xfB.q, lcB);
            Vec2 normal, point;
            float separation;
            position_manifold(pc, xfA, xfB, j, normal, point, separation);
            Vec2 rA = point - cA;
            Vec2 rB = point - cB;
            minSeparation = bmin(minSeparation, separation);
            float C = bclamp(kToiBaumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
            float rnA = cross(rA, normal);
            float rnB = cross(rB, normal);
            float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
            float impulse = K > 0.0f ? -C / K : 0.0f;
            Vec2 P = impulse * normal;
            cA -= mA * P;
            aA -= iA * cross(rA, P);
            cB += mB * P;
            aB += iB * cross(rB, P);
        }
        w.pos[pc.ia].c = cA;
        w.pos[pc.ia].a = aA;
        w.pos[pc.ib].c = cB;
        w.pos[pc.ib].a = aB;
    }
    return minSeparation >= -1.5f * kLinearSlop;
}

/* B2island::solve_toi, b2_island_private.rs:330-458 */
static void solve_toi_island(World& w, const Step& sub, int toiA, int toiB) {
    const int nb = (int)w.isl_bodies.size();
    w.pos.resize(nb);
    w.vel.resize(nb);
    for (int i = 0; i < nb; ++i) {
        const Body& b = w.bodies[w.isl_bodies[i]];
        w.pos[i].c = b.sweep.c;
        w.pos[i].a = b.sweep.a;
        w.vel[i].v = b.v;
        w.vel[i].w = b.w;
    }
    /* B2contactSolver::new (the velocity part is initialised again below, after the position
     * iterations move the bodies; without warm starting both passes start from zero impulses) */
    init_constraints(w, sub);
    for (int it = 0; it < sub.pi; ++it)
        if (solve_toi_position(w, toiA, toiB)) break;
    /* leap of faith to the new safe state */
    Body& A = w.bodies[w.isl_bodies[toiA]];
    Body& B = w.bodies[w.isl_bodies[toiB]];
    A.sweep.c0 = w.pos[toiA].c;
    A.sweep.a0 = w.pos[toiA].a;
    B.sweep.c0 = w.pos[toiB].c;
    B.sweep.a0 = w.pos[toiB].a;
    init_constraints(w, sub);
    for (int it = 0; it < sub.vi; ++it) solve_velocity(w);
    const float h = sub.dt;
    for (int i = 0; i < nb; ++i) {
        Vec2 c = w.pos[i].c;
        float a = w.pos[i].a;
        Vec2 v = w.vel[i].v;
        float wv = w.vel[i].w;
        Vec2 translation = h * v;
        if (dot(translation, translation) > kMaxTranslationSquared) {
            float ratio = kMaxTranslation / length(translation);
            v *= ratio;
        }
        float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            float ratio = kMaxRotation / std::fabs(rotation);
            wv *= ratio;
        }
        c += h * v;
        a += h * wv;
        w.pos[i].c = c;
        w.pos[i].a = a;
        w.vel[i].v = v;
        w.vel[i].w = wv;
        Body& b = w.bodies[w.isl_bodies[i]];
        b.sweep.c = c;
        b.sweep.a = a;
        b.v = v;
        b.w = wv;
        synchronize_transform(b);
    }
}

/* B2world::solve_toi, private/dynamics/b2_world.rs:534-901 (no sub-stepping: every step is
 * complete). With key_order set, two list-order choices follow the GPU's order instead: the
 * first time of impact is the smallest (alpha, contact key), and an event's island takes its
 * other contacts in key order. */
static void solve_toi(World& w, const Step& step) {
    for (int b = w.body_head; b >= 0; b = w.bodies[b].next) {
        w.bodies[b].island_flag = false;
        w.bodies[b].sweep.alpha0 = 0.0f;
    }
    for (int c = w.contact_head; c >= 0; c = w.contacts[c].next) {
        Contact& C = w.contacts[c];
        C.toi_flag = false;
        C.island_flag = false;
        C.toi_count = 0;
        C.toi = 1.0f;
    }
    const bool key_order = w.key_order;
    for (;;) {
        int minContact = -1;
        float minAlpha = 1.0f;
        uint64_t minKey = 0;
        for (int id = w.contact_head; id >= 0; id = w.contacts[id].next) {
            Contact& c = w.contacts[id];
            if (!c.enabled) continue;
            if (c.toi_count > kMaxSubSteps) continue;
            float alpha;
            if (c.toi_flag) {
                alpha = c.toi;
            } else {
                const Fixture& FA = w.fixtures[c.fa];
                const Fixture& FB = w.fixtures[c.fb];
                if (FA.sensor || FB.sensor) continue;
                Body& bA = w.bodies[FA.body];
                Body& bB = w.bodies[FB.body];
                const bool activeA = bA.awake && bA.type != STATIC;
                const bool activeB = bB.awake && bB.type != STATIC;
                if (!activeA && !activeB) continue;
                const bool collideA = bA.bullet || bA.type != DYNAMIC;
                const bool collideB = bB.bullet || bB.type != DYNAMIC;
                if (!collideA && !collideB) continue;
                float alpha0 = bA.sweep.alpha0;
                if (bA.sweep.alpha0 < bB.sweep.alpha0) {
                    alpha0 = bB.sweep.alpha0;
                    sweep_advance(bA.sweep, alpha0);
                } else if (bB.sweep.alpha0 < bA.sweep.alpha0) {
                    alpha0 = bA.sweep.alpha0;
                    sweep_advance(bB.sweep, alpha0);
                }
                int state;
                float beta;
                time_of_impact_shapes(FA.shape, bA.sweep, FB.shape, bB.sweep, 1.0f, state, beta);
                if (state == B2G_TOI_TOUCHING) alpha = bmin(alpha0 + (1.0f - alpha0) * beta, 1.0f);
                else alpha = 1.0f;
                c.toi = alpha;
                c.toi_flag = true;
            }
            if (alpha < minAlpha) {
                minContact = id;
                minAlpha = alpha;
                minKey = contact_proxy_key(w, c);
            } else if (key_order && minContact >= 0 && alpha == minAlpha) {
                const uint64_t k = contact_proxy_key(w, c);
                if (k < minKey) {
                    minContact = id;
                    minKey = k;
                }
            }
        }
        if (minContact < 0 || 1.0f - 10.0f * kEpsilon < minAlpha) break;

        Contact& mc = w.contacts[minContact];
        const int ia = w.fixtures[mc.fa].body, ib = w.fixtures[mc.fb].body;
        Body& bA = w.bodies[ia];
        Body& bB = w.bodies[ib];
        const Sweep backup1 = bA.sweep, backup2 = bB.sweep;
        body_advance(bA, minAlpha);
        body_advance(bB, minAlpha);
        update_contact(w, minContact);
        mc.toi_flag = false;
        ++mc.toi_count;
        if (!mc.enabled || !mc.touching) {
            mc.enabled = false;
            bA.sweep = backup1;
            bB.sweep = backup2;
            synchronize_transform(bA);
            synchronize_transform(bB);
            continue;
        }
        set_awake(bA, true);
        set_awake(bB, true);
        w.isl_bodies.clear();
        w.isl_contacts.clear();
        bA.island_index = 0;
        w.isl_bodies.push_back(ia);
        bB.island_index = 1;
        w.isl_bodies.push_back(ib);
        w.isl_contacts.push_back(minContact);
        bA.island_flag = true;
        bB.island_flag = true;
        mc.island_flag = true;

        /* the contacts of the event's dynamic bodies: (body, edge) in list order, body A's first */
        std::vector<std::pair<int, int>> cand;
        for (int bi : {ia, ib}) {
            if (w.bodies[bi].type != DYNAMIC) continue;
            for (int e = w.bodies[bi].edge_head; e >= 0; e = w.edges[e].next) cand.emplace_back(bi, e);
        }
        if (key_order) {
            /* each contact once (a second visit through the other body changes nothing), by key */
            std::vector<std::pair<int, int>> uniq;
            for (const auto& be : cand) {
                bool seen = false;
                for (const auto& u : uniq)
                    if (w.edges[u.second].contact == w.edges[be.second].contact) seen = true;
                if (!seen) uniq.push_back(be);
            }
            std::stable_sort(uniq.begin(), uniq.end(), [&](const std::pair<int, int>& x, const std::pair<int, int>& y) {
                return contact_proxy_key(w, w.contacts[w.edges[x.second].contact]) <
                       contact_proxy_key(w, w.contacts[w.edges[y.second].contact]);
            });
            cand.swap(uniq);
        }
        for (const auto& be : cand) {
            Body& body = w.bodies[be.first];
            const int ci = w.edges[be.second].contact;
            const int oi = w.edges[be.second].other;
            Contact& c = w.contacts[ci];
            if (c.island_flag) continue;
            Body& other = w.bodies[oi];
            if (other.type == DYNAMIC && !body.bullet && !other.bullet) continue;
            if (w.fixtures[c.fa].sensor || w.fixtures[c.fb].sensor) continue;
            const Sweep backup = other.sweep;
            if (!other.island_flag) body_advance(other, minAlpha);
            update_contact(w, ci);
            if (!c.enabled || !c.touching) {
                other.sweep = backup;
                synchronize_transform(other);
                continue;
            }
            c.island_flag = true;
            w.isl_contacts.push_back(ci);
            if (other.island_flag) continue;
            other.island_flag = true;
            if (other.type != STATIC) set_awake(other, true);
            other.island_index = (int)w.isl_bodies.size();
            w.isl_bodies.push_back(oi);
        }

        Step sub;
        sub.dt = (1.0f - minAlpha) * step.dt;
        sub.inv_dt = 1.0f / sub.dt;
        sub.dt_ratio = 1.0f;
        sub.pi = 20;
        sub.vi = step.vi;
        sub.warm = false;
        solve_toi_island(w, sub, bA.island_index, bB.island_index);
        ++w.toi_events;

        for (int bi : w.isl_bodies) {
            Body& b = w.bodies[bi];
            b.island_flag = false;
            if (b.type != DYNAMIC) continue;
            synchronize_fixtures(w, b);
            for (int e = b.edge_head; e >= 0; e = w.edges[e].next) {
                Contact& c = w.contacts[w.edges[e].contact];
                c.toi_flag = false;
                c.island_flag = false;
            }
        }
        find_new_contacts(w);
    }
}

/* B2world::step, private/dynamics/b2_world.rs:903-959 */
/* ---- destruction (src/b2_world.rs:72-91, src/b2_body.rs:259) and filtering (src/b2_fixture.rs:179-189) ---- */

/* B2world::destroy_joint, private/dynamics/b2_world.rs:278-340 */
static void destroy_joint(World& w, int id) {
    Joint& J = w.joints[id];
    if (J.prev >= 0) w.joints[J.prev].next = J.next;
    else w.joint_head = J.next;
    if (J.next >= 0) w.joints[J.next].prev = J.prev;
    J.prev = J.next = -1;
    set_awake(w.bodies[J.body_a], true);
    set_awake(w.bodies[J.body_b], true);
    for (int side = 0; side < 2; ++side) {  /* remove the joint edge from each body's singly linked list */
        const int b = side == 0 ? J.body_a : J.body_b;
        const int mine = 2 * id + side;
        int* link = &w.bodies[b].jedge_head;
        while (*link >= 0 && *link != mine) link = &w.jedges[*link].next;
        if (*link == mine) *link = w.jedges[mine].next;
    }
    J.alive = false;
    if (!J.collide_connected) {
        for (int e = w.bodies[J.body_b].edge_head; e >= 0; e = w.edges[e].next)
            if (w.edges[e].other == J.body_a) w.contacts[w.edges[e].contact].filter_flag = true;
    }
}

/* B2fixture::destroy_proxies, private/dynamics/b2_fixture.rs:135-145 */
static void destroy_proxies(World& w, Fixture& f) {
    if (f.proxy < 0) return;
    w.bp.destroy_proxy(f.proxy);
    f.proxy = -1;
}

/* B2body::destroy_fixture, private/dynamics/b2_body.rs:214-289 */
static void destroy_fixture(World& w, int fid) {
    Fixture& F = w.fixtures[fid];
    Body& b = w.bodies[F.body];
    int* link = &b.fixture_head;
    while (*link >= 0 && *link != fid) link = &w.fixtures[*link].next;
    if (*link == fid) *link = F.next;
    F.next = -1;
    /* the body's contacts of this fixture (B2contactManager::destroy) */
    for (int e = b.edge_head; e >= 0;) {
        const int next = w.edges[e].next;
        const Contact& c = w.contacts[w.edges[e].contact];
        if (c.fa == fid || c.fb == fid) destroy_contact(w, w.edges[e].contact);
        e = next;
    }
    if (b.enabled) destroy_proxies(w, F);
    F.alive = false;
    reset_mass_data(w, b);
}

/* B2world::destroy_body, private/dynamics/b2_world.rs:100-158 */
static void destroy_body(World& w, int bid) {
    Body& b = w.bodies[bid];
    while (b.jedge_head >= 0) destroy_joint(w, w.jedges[b.jedge_head].joint);
    while (b.edge_head >= 0) destroy_contact(w, w.edges[b.edge_head].contact);
    for (int f = b.fixture_head; f >= 0;) {
        const int next = w.fixtures[f].next;
        destroy_proxies(w, w.fixtures[f]);
        w.fixtures[f].alive = false;
        w.fixtures[f].next = -1;
        f = next;
    }
    b.fixture_head = -1;
    if (b.prev >= 0) w.bodies[b.prev].next = b.next;
    else w.body_head = b.next;
    if (b.next >= 0) w.bodies[b.next].prev = b.prev;
    b.prev = b.next = -1;
    b.alive = false;
    b.awake = false;  /* the slot reads as asleep, as the GPU's does */
}

/* B2fixture::set_filter_data + refilter, private/dynamics/b2_fixture.rs:175-211 */
static void set_filter_data(World& w, int fid, uint16_t category, uint16_t mask, int16_t group) {
    Fixture& F = w.fixtures[fid];
    F.category = category;
    F.mask = mask;
    F.group = group;
    for (int e = w.bodies[F.body].edge_head; e >= 0; e = w.edges[e].next) {
        Contact& c = w.contacts[w.edges[e].contact];
        if (c.fa == fid || c.fb == fid) c.filter_flag = true;
    }
    if (F.proxy >= 0) w.bp.touch_proxy(F.proxy);
}

static void step(World& w, float dt, int vi, int pi) {
    auto t0 = std::chrono::steady_clock::now();
    w.post_solve.clear();
    if (w.new_contacts) {
        find_new_contacts(w);
        w.new_contacts = false;
    }
    w.locked = true;
    Step s;
    s.dt = dt;
    s.vi = vi;
    s.pi = pi;
    s.inv_dt = dt > 0.0f ? 1.0f / dt : 0.0f;
    s.dt_ratio = w.inv_dt0 * dt;
    s.warm = w.warm_starting;
    auto t1 = std::chrono::steady_clock::now();
    collide(w);
    auto t2 = std::chrono::steady_clock::now();
    w.profile.collide = std::chrono::duration<float, std::milli>(t2 - t1).count();
    if (dt > 0.0f) {
        solve(w, s);
        w.profile.solve = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t2).count();
    }
    if (w.continuous && dt > 0.0f) {
        /* the recorded pair set stays the one of the step's own pair update */
        std::vector<Pair> pairs = w.last_pairs;
        std::vector<uint8_t> moved = w.last_moved;
        solve_toi(w, s);
        w.last_pairs.swap(pairs);
        w.last_moved.swap(moved);
    }
    if (dt > 0.0f) w.inv_dt0 = s.inv_dt;
    if (w.auto_clear) {
        for (int b = w.body_head; b >= 0; b = w.bodies[b].next) {
            w.bodies[b].force = v2(0, 0);
            w.bodies[b].torque = 0.0f;
        }
    }
    w.locked = false;
    w.profile.step = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace ora

using namespace ora;

extern "C" {

int ora_set_trig_libm(int flag) {
    g_trig_libm = flag != 0;
    return 0;
}

int ora_world_create(float gx, float gy, void** out) {
    World* w = new World();
    w->gravity = v2(gx, gy);
    *out = w;
    return 0;
}

int ora_world_destroy(void* p) {
    delete (World*)p;
    return 0;
}

int ora_set_flags(void* p, int allow_sleep, int warm_starting, int continuous, int auto_clear) {
    World& w = *(World*)p;
    w.allow_sleep = allow_sleep != 0;
    w.warm_starting = warm_starting != 0;
    w.continuous = continuous != 0;
    w.auto_clear = auto_clear != 0;
    return 0;
}

int ora_set_record_events(void* p, int flag) {
    ((World*)p)->record_events = flag != 0;
    return 0;
}

int ora_create_bodies(void* p, const b2g_body_def* defs, int n, uint32_t* ids) {
    World& w = *(World*)p;
    for (int i = 0; i < n; ++i) {
        int id = create_body(w, defs[i]);
        if (ids) ids[i] = (uint32_t)id;
    }
    return 0;
}

int ora_create_fixtures(void* p, const b2g_fixture_def* defs, int n, uint32_t* ids) {
    World& w = *(World*)p;
    for (int i = 0; i < n; ++i) {
        if (defs[i].body >= w.bodies.size()) return B2G_ERR_INVALID_ARG;
        int id = create_fixture(w, defs[i]);
        if (ids) ids[i] = (uint32_t)id;
    }
    return 0;
}

int ora_step(void* p, float dt, int vi, int pi) {
    step(*(World*)p, dt, vi, pi);
    return 0;
}

int ora_steps(void* p, float dt, int vi, int pi, int n) {
    for (int i = 0; i < n; ++i) step(*(World*)p, dt, vi, pi);
    return 0;
}

int ora_get_body_states(void* p, uint32_t first, uint32_t count, b2g_body_state* out) {
    World& w = *(World*)p;
    if ((size_t)first + count > w.bodies.size()) return B2G_ERR_INVALID_ARG;
    for (uint32_t i = 0; i < count; ++i) {
        const Body& b = w.bodies[first + i];
        b2g_body_state& s = out[i];
        s.position = b2g_vec2{b.xf.p.x, b.xf.p.y};
        s.angle = b.sweep.a;
        s.linear_velocity = b2g_vec2{b.v.x, b.v.y};
        s.angular_velocity = b.w;
        s.world_center = b2g_vec2{b.sweep.c.x, b.sweep.c.y};
    }
    return 0;
}

/* B2body::set_transform, private/dynamics/b2_body.rs:418-447 */
int ora_set_transform(void* p, uint32_t id, b2g_vec2 pos, float angle) {
    World& w = *(World*)p;
    if (id >= w.bodies.size()) return B2G_ERR_INVALID_ARG;
    Body& b = w.bodies[id];
    b.xf.q = rot(angle);
    b.xf.p = v2(pos.x, pos.y);
    b.sweep.c = mul(b.xf, b.sweep.local_center);
    b.sweep.a = angle;
    b.sweep.c0 = b.sweep.c;
    b.sweep.a0 = angle;
    for (int f = b.fixture_head; f >= 0; f = w.fixtures[f].next) synchronize_fixture(w, w.fixtures[f], b.xf, b.xf);
    w.new_contacts = true;
    return 0;
}

/* B2body::set_linear_velocity / set_angular_velocity (src/b2_body.rs:684-705) */
int ora_set_velocity(void* p, uint32_t id, b2g_vec2 v, float av) {
    World& w = *(World*)p;
    if (id >= w.bodies.size()) return B2G_ERR_INVALID_ARG;
    Body& b = w.bodies[id];
    if (b.type == STATIC) return 0;
    Vec2 vv = v2(v.x, v.y);
    if (dot(vv, vv) > 0.0f) set_awake(b, true);
    b.v = vv;
    if (av * av > 0.0f) set_awake(b, true);
    b.w = av;
    return 0;
}

int ora_get_counts(void* p, b2g_counts* out) {
    World& w = *(World*)p;
    memset(out, 0, sizeof(*out));
    out->bodies = (int)w.bodies.size();
    out->fixtures = (int)w.fixtures.size();
    out->proxies = w.bp.proxy_count;
    out->contacts = w.contact_count;
    int touching = 0;
    for (int c = w.contact_head; c >= 0; c = w.contacts[c].next) touching += w.contacts[c].touching ? 1 : 0;
    out->touching_contacts = touching;
    out->islands_solved = w.islands_solved;
    out->pairs = (int)w.last_pairs.size();
    return 0;
}

int ora_get_profile(void* p, b2g_profile* out) {
    *out = ((World*)p)->profile;
    return 0;
}

/* Contacts in world-list order (newest first). */
int ora_get_contacts(void* p, b2g_contact_info* out, int cap, int* n) {
    World& w = *(World*)p;
    int k = 0;
    for (int c = w.contact_head; c >= 0; c = w.contacts[c].next) {
        if (k < cap && out) {
            const Contact& C = w.contacts[c];
            b2g_contact_info& o = out[k];
            memset(&o, 0, sizeof(o));
            o.fixture_a = (uint32_t)C.fa;
            o.fixture_b = (uint32_t)C.fb;
            o.touching = C.touching ? 1 : 0;
            o.manifold_type = C.m.type;
            o.point_count = C.m.point_count;
            o.local_normal = b2g_vec2{C.m.local_normal.x, C.m.local_normal.y};
            o.local_point = b2g_vec2{C.m.local_point.x, C.m.local_point.y};
            for (int j = 0; j < 2; ++j) {
                o.point_local[j] = b2g_vec2{C.m.points[j].local_point.x, C.m.points[j].local_point.y};
                o.normal_impulse[j] = C.m.points[j].normal_impulse;
                o.tangent_impulse[j] = C.m.points[j].tangent_impulse;
                o.point_id[j] = C.m.points[j].id;
            }
            o.friction = C.friction;
            o.restitution = C.restitution;
            o.restitution_threshold = C.threshold;
        }
        ++k;
    }
    *n = k;
    return 0;
}

/* Pairs of the last update_pairs as fixture ids (min, max), in emission order (may repeat). */
int ora_get_pairs(void* p, uint32_t* out, int cap, int* n) {
    World& w = *(World*)p;
    int k = 0;
    for (const Pair& pr : w.last_pairs) {
        if (k < cap && out) {
            int fa = w.bp.tree.user(pr.a), fb = w.bp.tree.user(pr.b);
            out[2 * k] = (uint32_t)(fa < fb ? fa : fb);
            out[2 * k + 1] = (uint32_t)(fa < fb ? fb : fa);
        }
        ++k;
    }
    *n = k;
    return 0;
}

/* Fat AABB per fixture, whether it was in the move buffer at the last update_pairs, and its proxy id. */
int ora_get_proxies(void* p, float* aabbs, uint8_t* moved, int* proxy_ids, int cap) {
    World& w = *(World*)p;
    int n = (int)w.fixtures.size();
    for (int i = 0; i < n && i < cap; ++i) {
        const Fixture& f = w.fixtures[i];
        if (f.proxy < 0) {  /* no proxy (disabled or destroyed): an empty box, as the GPU reports it */
            const float inf = INFINITY;
            aabbs[4 * i + 0] = inf;
            aabbs[4 * i + 1] = inf;
            aabbs[4 * i + 2] = -inf;
            aabbs[4 * i + 3] = -inf;
            if (moved) moved[i] = 0;
            if (proxy_ids) proxy_ids[i] = -1;
            continue;
        }
        const AABB& a = w.bp.tree.fat_aabb(f.proxy);
        aabbs[4 * i + 0] = a.lo.x;
        aabbs[4 * i + 1] = a.lo.y;
        aabbs[4 * i + 2] = a.hi.x;
        aabbs[4 * i + 3] = a.hi.y;
        if (moved) moved[i] = w.last_moved[i];
        if (proxy_ids) proxy_ids[i] = f.proxy;
    }
    return 0;
}

/* Ordering hook: pairs (fixture_a, fixture_b) in the order islands must solve them; n = 0 clears. */
int ora_set_solver_order(void* p, const uint32_t* pairs, int n) {
    World& w = *(World*)p;
    w.hook_rank.clear();
    w.hook_misses = 0;
    w.hook = n > 0;
    w.hook_rank.reserve((size_t)n * 2);
    for (int i = 0; i < n; ++i) w.hook_rank[pair_key((int)pairs[2 * i], (int)pairs[2 * i + 1])] = i;
    return 0;
}

/* B2world::create_joint, private/dynamics/b2_world.rs:156-276 (revolute joints) */
int ora_create_joints(void* p, const b2g_joint_def* defs, int n, uint32_t* ids) {
    World& w = *(World*)p;
    for (int i = 0; i < n; ++i) {
        const b2g_joint_def& d = defs[i];
        if ((d.type != B2G_JOINT_REVOLUTE && d.type != B2G_JOINT_DISTANCE && d.type != B2G_JOINT_WELD &&
             d.type != B2G_JOINT_FRICTION && d.type != B2G_JOINT_MOTOR && d.type != B2G_JOINT_MOUSE &&
             d.type != B2G_JOINT_PRISMATIC && d.type != B2G_JOINT_WHEEL && d.type != B2G_JOINT_PULLEY &&
             d.type != B2G_JOINT_GEAR) ||
            (d.type == B2G_JOINT_GEAR && (d.joint1 >= w.joints.size() || d.joint2 >= w.joints.size())) ||
            d.body_a >= w.bodies.size() ||
            d.body_b >= w.bodies.size())
            return -1;
        const int id = (int)w.joints.size();
        Joint j;
        j.type = d.type;
        /* b2_distance_joint_new (b2_distance_joint.rs:42-76) */
        j.length = bmax(d.length, kLinearSlop);
        j.min_length = bmax(d.min_length, kLinearSlop);
        j.max_length = bmax(d.max_length, j.min_length);
        j.stiffness = d.stiffness;
        j.damping = d.damping;
        j.max_force = d.max_force;
        j.max_torque = d.max_torque;
        j.linear_offset = v2(d.linear_offset.x, d.linear_offset.y);
        j.angular_offset = d.angular_offset;
        j.correction_factor = d.correction_factor;
        j.target = v2(d.target.x, d.target.y);
        /* B2prismaticJoint::new (b2_prismatic_joint.rs:54-60) */
        j.local_xaxis_a = v2(d.local_axis_a.x, d.local_axis_a.y);
        normalize(j.local_xaxis_a);
        j.local_yaxis_a = cross_sv(1.0f, j.local_xaxis_a);
        j.lower_translation = d.lower_translation;
        j.upper_translation = d.upper_translation;
        j.max_motor_force = d.max_motor_force;
        /* b2_pulley_joint.rs:30-40 */
        j.ground_a = v2(d.ground_anchor_a.x, d.ground_anchor_a.y);
        j.ground_b = v2(d.ground_anchor_b.x, d.ground_anchor_b.y);
        j.ratio = d.ratio;
        j.pulley_constant = d.length_a + d.ratio * d.length_b;
        if (j.type == B2G_JOINT_WHEEL) {  /* b2_wheel_joint.rs:334-335: the axis as given */
            j.local_xaxis_a = v2(d.local_axis_a.x, d.local_axis_a.y);
            j.local_yaxis_a = cross_sv(1.0f, j.local_xaxis_a);
        }
        j.body_a = (int)d.body_a;
        j.body_b = (int)d.body_b;
        j.collide_connected = d.collide_connected != 0;
        j.local_anchor_a = v2(d.local_anchor_a.x, d.local_anchor_a.y);
        j.local_anchor_b = v2(d.local_anchor_b.x, d.local_anchor_b.y);
        /* b2_mouse_joint_new (src/joints/b2_mouse_joint.rs:140-160): the target in body B's frame */
        if (j.type == B2G_JOINT_MOUSE) j.local_anchor_b = mul_t(w.bodies[j.body_b].xf, j.target);
        if (j.type == B2G_JOINT_GEAR) {
            /* B2gearJoint::new (private/dynamics/joints/b2_gear_joint.rs:29-137): each side's anchors, axis,
             * reference angle and coordinate from its joint and the bodies' current transforms */
            float coordinate[2];
            for (int side = 0; side < 2; ++side) {
                const Joint& J = w.joints[side == 0 ? d.joint1 : d.joint2];
                const Body& F = w.bodies[J.body_a];
                const Body& S = w.bodies[J.body_b];
                const bool prismatic = J.type == B2G_JOINT_PRISMATIC;
                const Vec2 axis = prismatic ? J.local_xaxis_a : v2(0, 0);
                if (prismatic) {
                    const Vec2 p_second = mul_t(F.xf.q, mul(S.xf.q, J.local_anchor_b) + (S.xf.p - F.xf.p));
                    coordinate[side] = dot(p_second - J.local_anchor_a, axis);
                } else {
                    coordinate[side] = S.sweep.a - F.sweep.a - J.reference_angle;
                }
                if (side == 0) {
                    j.body_c = J.body_a;
                    j.gear_anchor_c = J.local_anchor_a;
                    j.gear_anchor_a = J.local_anchor_b;
                    j.gear_axis_c = axis;
                    j.gear_ref_a = J.reference_angle;
                    j.gear_prismatic_a = prismatic;
                } else {
                    j.body_d = J.body_a;
                    j.gear_anchor_d = J.local_anchor_a;
                    j.gear_anchor_b = J.local_anchor_b;
                    j.gear_axis_d = axis;
                    j.gear_ref_b = J.reference_angle;
                    j.gear_prismatic_b = prismatic;
                }
            }
            j.gear_constant = coordinate[0] + j.ratio * coordinate[1];
        }
        j.reference_angle = d.reference_angle;
        j.enable_limit = d.enable_limit != 0;
        j.lower_angle = d.lower_angle;
        j.upper_angle = d.upper_angle;
        j.enable_motor = d.enable_motor != 0;
        j.motor_speed = d.motor_speed;
        j.max_motor_torque = d.max_motor_torque;
        j.next = w.joint_head;
        if (w.joint_head >= 0) w.joints[w.joint_head].prev = id;
        w.joint_head = id;
        w.joints.push_back(j);
        w.jedges.push_back(JointEdge{id, j.body_b, w.bodies[j.body_a].jedge_head});
        w.bodies[j.body_a].jedge_head = 2 * id;
        w.jedges.push_back(JointEdge{id, j.body_a, w.bodies[j.body_b].jedge_head});
        w.bodies[j.body_b].jedge_head = 2 * id + 1;
        if (!j.collide_connected) {
            for (int e = w.bodies[j.body_b].edge_head; e >= 0; e = w.edges[e].next)
                if (w.edges[e].other == j.body_a) w.contacts[w.edges[e].contact].filter_flag = true;
        }
        if (ids) ids[i] = (uint32_t)id;
    }
    return 0;
}

/* per joint: impulse x, y, motor, lower, upper */
int ora_get_joint_impulses(void* p, uint32_t first, uint32_t count, float* out) {
    World& w = *(World*)p;
    if ((size_t)first + count > w.joints.size()) return -1;
    for (uint32_t i = 0; i < count; ++i) {
        const Joint& j = w.joints[first + i];
        if (j.type == B2G_JOINT_GEAR) {
            out[5 * i + 0] = j.gear_impulse;
            for (int k = 1; k < 5; ++k) out[5 * i + k] = 0.0f;
            continue;
        }
        if (j.type == B2G_JOINT_PULLEY) {
            out[5 * i + 0] = j.pulley_impulse;
            for (int k = 1; k < 5; ++k) out[5 * i + k] = 0.0f;
            continue;
        }
        if (j.type == B2G_JOINT_WHEEL) {
            out[5 * i + 0] = j.wheel_impulse;
            out[5 * i + 1] = j.spring_impulse;
            out[5 * i + 2] = j.motor_impulse;
            out[5 * i + 3] = j.lower_impulse;
            out[5 * i + 4] = j.upper_impulse;
            continue;
        }
        if (j.type == B2G_JOINT_FRICTION || j.type == B2G_JOINT_MOTOR || j.type == B2G_JOINT_MOUSE) {
            out[5 * i + 0] = j.linear_impulse.x;
            out[5 * i + 1] = j.linear_impulse.y;
            out[5 * i + 2] = j.angular_impulse;
            out[5 * i + 3] = 0.0f;
            out[5 * i + 4] = 0.0f;
            continue;
        }
        if (j.type == B2G_JOINT_WELD) {
            out[5 * i + 0] = j.weld_impulse[0];
            out[5 * i + 1] = j.weld_impulse[1];
            out[5 * i + 2] = j.weld_impulse[2];
            out[5 * i + 3] = 0.0f;
            out[5 * i + 4] = 0.0f;
            continue;
        }
        if (j.type == B2G_JOINT_DISTANCE) {
            out[5 * i + 0] = j.dist_impulse;
            out[5 * i + 1] = j.lower_impulse;
            out[5 * i + 2] = j.upper_impulse;
            out[5 * i + 3] = 0.0f;
            out[5 * i + 4] = 0.0f;
            continue;
        }
        out[5 * i + 0] = j.impulse.x;
        out[5 * i + 1] = j.impulse.y;
        out[5 * i + 2] = j.motor_impulse;
        out[5 * i + 3] = j.lower_impulse;
        out[5 * i + 4] = j.upper_impulse;
    }
    return 0;
}

/* Joint ordering hook: each island solves its joints in this order of joint ids (n = 0 clears) */
/* B2mouseJoint::set_target (src/joints/b2_mouse_joint.rs:114-119) */
int ora_set_mouse_target(void* p, uint32_t id, float x, float y) {
    World& w = *(World*)p;
    if (id >= w.joints.size() || w.joints[id].type != B2G_JOINT_MOUSE) return -1;
    Joint& j = w.joints[id];
    if (x != j.target.x || y != j.target.y) {
        set_awake(w.bodies[j.body_b], true);
        j.target = v2(x, y);
    }
    return 0;
}

int ora_set_joint_order(void* p, const uint32_t* order, int n) {
    World& w = *(World*)p;
    w.joint_rank.clear();
    if (n <= 0) return 0;
    w.joint_rank.assign(w.joints.size(), 0x7fffffff);
    for (int i = 0; i < n; ++i)
        if (order[i] < w.joint_rank.size()) w.joint_rank[order[i]] = i;
    return 0;
}

int ora_destroy_bodies(void* p, const uint32_t* ids, int n) {
    World& w = *(World*)p;
    for (int i = 0; i < n; ++i)
        if (ids[i] >= w.bodies.size() || !w.bodies[ids[i]].alive) return -1;
    for (int i = 0; i < n; ++i) destroy_body(w, (int)ids[i]);
    return 0;
}

int ora_destroy_fixtures(void* p, const uint32_t* ids, int n) {
    World& w = *(World*)p;
    for (int i = 0; i < n; ++i)
        if (ids[i] >= w.fixtures.size() || !w.fixtures[ids[i]].alive) return -1;
    for (int i = 0; i < n; ++i) destroy_fixture(w, (int)ids[i]);
    return 0;
}

int ora_destroy_joints(void* p, const uint32_t* ids, int n) {
    World& w = *(World*)p;
    for (int i = 0; i < n; ++i)
        if (ids[i] >= w.joints.size() || !w.joints[ids[i]].alive) return -1;
    for (int i = 0; i < n; ++i) destroy_joint(w, (int)ids[i]);
    return 0;
}

int ora_set_filter_data(void* p, uint32_t f, int category, int mask, int group) {
    World& w = *(World*)p;
    if (f >= w.fixtures.size() || !w.fixtures[f].alive) return -1;
    set_filter_data(w, (int)f, (uint16_t)category, (uint16_t)mask, (int16_t)group);
    return 0;
}

int ora_set_contact_filter(void* p, ContactFilterFn fn, void* user) {
    World& w = *(World*)p;
    w.filter_fn = fn;
    w.filter_user = user;
    return 0;
}

int ora_set_pre_solve(void* p, PreSolveFn fn, void* user) {
    World& w = *(World*)p;
    w.pre_solve_fn = fn;
    w.pre_solve_user = user;
    return 0;
}

int ora_get_post_solve(void* p, b2g_contact_impulse* out, int cap, int* n) {
    World& w = *(World*)p;
    *n = (int)w.post_solve.size();
    for (int i = 0; out && i < *n && i < cap; ++i) out[i] = w.post_solve[i];
    return 0;
}

int ora_get_hook_misses(void* p) { return ((World*)p)->hook_misses; }

/* solid time-of-impact events solved since the world was made */
int ora_get_toi_events(void* p) { return ((World*)p)->toi_events; }

/* Ordering hook for the contact list: collide goes through the contacts in key order, and in
 * solve_toi ties of the first time of impact go to the smallest contact key and an event's island
 * takes its other contacts in key order (the GPU's order), instead of the contact-list order. */
int ora_set_key_order(void* p, int flag) {
    ((World*)p)->key_order = flag != 0;
    return 0;
}

/* B2body::is_awake of bodies [first, first + count) */
int ora_get_awake(void* p, uint32_t first, uint32_t count, uint8_t* out) {
    World& w = *(World*)p;
    if ((size_t)first + count > w.bodies.size()) return -1;
    for (uint32_t i = 0; i < count; ++i) out[i] = w.bodies[first + i].awake ? 1 : 0;
    return 0;
}

int ora_get_solver_order(void* p, uint32_t* out, int cap, int* n) {
    World& w = *(World*)p;
    int k = 0;
    for (uint64_t key : w.last_order) {
        if (k < cap && out) {
            out[2 * k] = (uint32_t)(key >> 32);
            out[2 * k + 1] = (uint32_t)(key & 0xffffffffu);
        }
        ++k;
    }
    *n = k;
    return 0;
}

int ora_get_events(void* p, b2g_contact_event* out, int cap, int* n) {
    World& w = *(World*)p;
    int k = (int)w.events.size();
    *n = k;
    if (!out) return 0; /* size query: keep the events for the copying call */
    for (int i = 0; i < k && i < cap; ++i) out[i] = w.events[i];
    w.events.clear();
    return 0;
}

/* Replace the world's dynamic state with a snapshot taken after a step of another engine
 * (the GPU): body poses and velocities, every proxy's fat AABB (empty move buffer), the
 * contact list with manifolds, impulses and touching flags, and 1/dt of the last step.
 * Bodies and fixtures must have been created identically beforehand. Contacts are pushed
 * so that the world list ends up in the given order. */
int ora_import_state(void* p, const b2g_body_state* bodies, int nb, const float* fat, int nf,
                     const b2g_contact_info* contacts, int nc, float inv_dt0) {
    World& w = *(World*)p;
    if (nb != (int)w.bodies.size() || nf != (int)w.fixtures.size()) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < nb; ++i) {
        Body& b = w.bodies[i];
        if (b.type == STATIC) continue;
        const b2g_body_state& s = bodies[i];
        b.sweep.c = v2(s.world_center.x, s.world_center.y);
        b.sweep.a = s.angle;
        b.sweep.c0 = b.sweep.c;
        b.sweep.a0 = b.sweep.a;
        b.xf.p = v2(s.position.x, s.position.y);
        b.xf.q = rot(s.angle);
        b.v = v2(s.linear_velocity.x, s.linear_velocity.y);
        b.w = s.angular_velocity;
        b.force = v2(0, 0);
        b.torque = 0.0f;
        b.awake = true;
        b.sleep_time = 0.0f;
    }
    /* broadphase: rebuild the tree with the given fat AABBs in fixture order */
    w.bp = BroadPhase();
    w.proxy_to_fixture.clear();
    for (int f = 0; f < nf; ++f) {
        Fixture& F = w.fixtures[f];
        if (F.proxy < 0) continue;
        AABB a{v2(fat[4 * f], fat[4 * f + 1]), v2(fat[4 * f + 2], fat[4 * f + 3])};
        F.proxy = w.bp.create_proxy_fat(a, f);
        if ((int)w.proxy_to_fixture.size() <= F.proxy) w.proxy_to_fixture.resize((size_t)F.proxy + 1, -1);
        w.proxy_to_fixture[F.proxy] = f;
    }
    /* contacts: drop all, then recreate from the snapshot */
    w.contacts.clear();
    w.edges.clear();
    w.free_contacts.clear();
    w.contact_head = -1;
    w.contact_count = 0;
    for (Body& b : w.bodies) b.edge_head = -1;
    for (int i = nc - 1; i >= 0; --i) {
        const b2g_contact_info& c = contacts[i];
        const int fa = (int)c.fixture_a, fb = (int)c.fixture_b;
        if (fa < 0 || fa >= nf || fb < 0 || fb >= nf) return B2G_ERR_INVALID_ARG;
        const int before = w.contact_count;
        add_pair(w, fa, fb);
        if (w.contact_count == before) return B2G_ERR_INVALID_ARG;  /* rejected by add_pair */
        Contact& C = w.contacts[w.contact_head];
        if (C.fa != fa || C.fb != fb) return B2G_ERR_INVALID_ARG;  /* not in primary order */
        C.touching = c.touching != 0;
        C.m.type = c.manifold_type;
        C.m.point_count = c.point_count;
        C.m.local_normal = v2(c.local_normal.x, c.local_normal.y);
        C.m.local_point = v2(c.local_point.x, c.local_point.y);
        for (int j = 0; j < 2; ++j) {
            C.m.points[j].local_point = v2(c.point_local[j].x, c.point_local[j].y);
            C.m.points[j].normal_impulse = c.normal_impulse[j];
            C.m.points[j].tangent_impulse = c.tangent_impulse[j];
            C.m.points[j].id = c.point_id[j];
        }
    }
    w.inv_dt0 = inv_dt0;
    w.new_contacts = false;
    return 0;
}

/* Shape helpers exposed for known-answer tests (collision_test.rs / math_test.rs). */
int ora_polygon_mass(const b2g_fixture_def* d, float* out_centroid_mass_center_I) {
    Shape s;
    build_shape(*d, s);
    MassData md;
    compute_mass(s, d->density, md);
    out_centroid_mass_center_I[0] = s.centroid.x;
    out_centroid_mass_center_I[1] = s.centroid.y;
    out_centroid_mass_center_I[2] = md.mass;
    out_centroid_mass_center_I[3] = md.center.x;
    out_centroid_mass_center_I[4] = md.center.y;
    out_centroid_mass_center_I[5] = md.I;
    return s.count;
}

int ora_sincos(const float* x, float* s, float* c, int n) {
    for (int i = 0; i < n; ++i) {
        Rot q = rot(x[i]);
        s[i] = q.s;
        c[i] = q.c;
    }
    return 0;
}

/* Manifold of two standalone shapes at given transforms (narrowphase known-answer tests). */
int ora_collide(const b2g_fixture_def* da, const float* xfa, const b2g_fixture_def* db, const float* xfb,
                b2g_contact_info* out) {
    Shape sa, sb;
    build_shape(*da, sa);
    build_shape(*db, sb);
    Xf A{v2(xfa[0], xfa[1]), rot(xfa[2])}, B{v2(xfb[0], xfb[1]), rot(xfb[2])};
    Manifold m;
    int ta = sa.type, tb = sb.type;
    if (ta == SHAPE_CIRCLE && tb == SHAPE_CIRCLE) collide_circles(m, sa, A, sb, B);
    else if (ta == SHAPE_POLYGON && tb == SHAPE_CIRCLE) collide_polygon_circle(m, sa, A, sb, B);
    else if (ta == SHAPE_POLYGON && tb == SHAPE_POLYGON) collide_polygons(m, sa, A, sb, B);
    else if (ta == SHAPE_EDGE && tb == SHAPE_CIRCLE) collide_edge_circle(m, sa, A, sb, B);
    else if (ta == SHAPE_EDGE && tb == SHAPE_POLYGON) collide_edge_polygon(m, sa, A, sb, B);
    else return B2G_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    out->manifold_type = m.type;
    out->point_count = m.point_count;
    out->local_normal = b2g_vec2{m.local_normal.x, m.local_normal.y};
    out->local_point = b2g_vec2{m.local_point.x, m.local_point.y};
    for (int j = 0; j < 2; ++j) {
        out->point_local[j] = b2g_vec2{m.points[j].local_point.x, m.points[j].local_point.y};
        out->point_id[j] = m.points[j].id;
    }
    return 0;
}

}  // extern "C"

/* ---- world queries (B2world::query_aabb / ray_cast, private/dynamics/b2_world.rs:969-1056) ---- */

namespace {

/* fixture ray casts: B2circleShape (private/collision/b2_circle_shape.rs:26-59), B2polygonShape
 * (private/collision/b2_polygon_shape.rs:226-287, whose lower bound starts at 0.032), B2edgeShape
 * (private/collision/b2_edge_shape.rs:39-102) */
bool shape_ray_cast(const Shape& sh, const Xf& xf, Vec2 ip1, Vec2 ip2, float max_fraction, float* fraction,
                    Vec2* normal) {
    if (sh.type == SHAPE_CIRCLE) {
        const Vec2 position = xf.p + mul(xf.q, sh.p);
        const Vec2 s = ip1 - position;
        const float b = dot(s, s) - sh.radius * sh.radius;
        const Vec2 r = ip2 - ip1;
        const float c = dot(s, r);
        const float rr = dot(r, r);
        const float sigma = c * c - rr * b;
        if (sigma < 0.0f || rr < kEpsilon) return false;
        float a = -(c + std::sqrt(sigma));
        if (0.0f <= a && a <= max_fraction * rr) {
            a /= rr;
            *fraction = a;
            Vec2 n = s + a * r;
            normalize(n);
            *normal = n;
            return true;
        }
        return false;
    }
    const Vec2 p1 = mul_t(xf.q, ip1 - xf.p);
    const Vec2 p2 = mul_t(xf.q, ip2 - xf.p);
    const Vec2 d = p2 - p1;
    if (sh.type == SHAPE_POLYGON) {
        float lower = 0.032f, upper = max_fraction;
        int index = -1;
        for (int i = 0; i < sh.count; ++i) {
            const float numerator = dot(sh.normals[i], sh.verts[i] - p1);
            const float denominator = dot(sh.normals[i], d);
            if (denominator == 0.0f) {
                if (numerator < 0.0f) return false;
            } else {
                if (denominator < 0.0f && numerator < lower * denominator) {
                    lower = numerator / denominator;
                    index = i;
                } else if (denominator > 0.0f && numerator < upper * denominator) {
                    upper = numerator / denominator;
                }
            }
            if (upper < lower) return false;
        }
        if (index >= 0) {
            *fraction = lower;
            *normal = mul(xf.q, sh.normals[index]);
            return true;
        }
        return false;
    }
    /* edge */
    const Vec2 v1 = sh.v1, v2 = sh.v2;
    const Vec2 e = v2 - v1;
    Vec2 nrm{e.y, -e.x};
    normalize(nrm);
    const float numerator = dot(nrm, v1 - p1);
    if (sh.one_sided && numerator > 0.0f) return false;
    const float denominator = dot(nrm, d);
    if (denominator == 0.0f) return false;
    const float t = numerator / denominator;
    if (t < 0.0f || max_fraction < t) return false;
    const Vec2 q = p1 + t * d;
    const Vec2 r = v2 - v1;
    const float rr = dot(r, r);
    if (rr == 0.0f) return false;
    const float sf = dot(q - v1, r) / rr;
    if (sf < 0.0f || 1.0f < sf) return false;
    *fraction = t;
    *normal = numerator > 0.0f ? -mul(xf.q, nrm) : mul(xf.q, nrm);
    return true;
}

}  // namespace

extern "C" {

/* fixtures whose fat AABB overlaps the box, sorted; returns their number (writes at most cap) */
int ora_query_aabb(void* p, float lx, float ly, float ux, float uy, int* out, int cap) {
    World& w = *(World*)p;
    std::vector<int> hits;
    AABB box{Vec2{lx, ly}, Vec2{ux, uy}};
    w.bp.tree.query(box, [&](int proxy) {
        hits.push_back(w.bp.tree.user(proxy));
        return true;
    });
    std::sort(hits.begin(), hits.end());
    for (int i = 0; i < (int)hits.size() && i < cap; ++i) out[i] = hits[i];
    return (int)hits.size();
}

/* the closest hit along p1 -> p2, with the callback that clips the ray to each reported fraction:
 * out = fixture (as float bits; -1 if none), point x, y, normal x, y, fraction */
int ora_ray_cast_closest(void* p, float p1x, float p1y, float p2x, float p2y, float* out) {
    World& w = *(World*)p;
    const Vec2 p1{p1x, p1y}, p2{p2x, p2y};
    int hit_fixture = -1;
    Vec2 hit_point{0, 0}, hit_normal{0, 0};
    float hit_fraction = 1.0f;
    w.bp.tree.ray_cast(p1, p2, 1.0f, [&](float max_fraction, int proxy) -> float {
        const int fi = w.bp.tree.user(proxy);
        const Fixture& f = w.fixtures[fi];
        float fraction;
        Vec2 normal;
        if (!shape_ray_cast(f.shape, w.bodies[f.body].xf, p1, p2, max_fraction, &fraction, &normal))
            return max_fraction;
        hit_fixture = fi;
        hit_point = (1.0f - fraction) * p1 + fraction * p2;
        hit_normal = normal;
        hit_fraction = fraction;
        return fraction;
    });
    out[0] = (float)hit_fixture;
    out[1] = hit_point.x;
    out[2] = hit_point.y;
    out[3] = hit_normal.x;
    out[4] = hit_normal.y;
    out[5] = hit_fraction;
    return hit_fixture >= 0 ? 1 : 0;
}

}  // extern "C"
