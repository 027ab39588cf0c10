/*
 * api.cu — the C ABI of include/b2g.h and the host-side world that drives the kernels.
 *
 * Creation (B2world::create_body, B2body::create_fixture) runs on the host, because it
 * is rare and sequential: polygon hulls (B2polygonShape::set), mass data
 * (compute_mass + reset_mass_data) and the first fat AABB of each proxy are computed
 * here with the same f32 operation order as the reference, then uploaded. After the
 * first step the device copy is authoritative; setters launch small kernels.
 *
 * A step (B2world::step, src/private/dynamics/b2_world.rs:903-959) is a fixed sequence
 * of launches on the world's stream with no host synchronisation:
 *   [broadphase if fixtures were added] -> collide -> islands + constraints ->
 *   colouring (cooperative) -> solver (cooperative) -> broadphase + contact merge.
 * Counts that vary per step live in device memory and every kernel reads them there.
 *
 * Proxy ids: the reference's proxy id is the node-pool index of the proxy's leaf in its
 * dynamic tree (private/collision/b2_dynamic_tree.rs:28-99). That index depends only on the
 * order of creations and destructions, not on the tree's shape: an insertion into a non-empty
 * tree takes a leaf and an internal node from the pool's free list (or the next two fresh nodes),
 * a removal returns the leaf's parent and then the leaf (so the list's head is the leaf), a move
 * returns its parent and takes it back, and the root alone neither takes nor returns a parent.
 * So the free list is a stack of (leaf, parent) pairs with the leaf on top, and a new proxy gets
 * the most recently freed leaf id, else the next fresh node (0 for the first proxy, then two nodes
 * per proxy). alloc_refid / free_refid keep that stack; the ids serve the same purposes as in the
 * reference: which fixture of a same-type pair is A, the contact keys' order and the moved rule.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/b2g.h"
#include "b2g_internal.h"
#include "b2g_tape.h"

using namespace b2g;

namespace {

constexpr int kVersion = 1;

struct Timer {
    cudaEvent_t e[11] = {};
    bool valid = false;
};

/* What a captured step graph depends on besides device memory contents. */
struct GraphKey {
    float dt, dt_ratio, gx, gy;
    int vi, pi, flags;
    int generation, n_bodies, n_fixtures;
};

struct GraphSlot {
    cudaGraphExec_t exec = nullptr;
    unsigned long long kernels = 0;  /* kernel nodes in the graph */
    GraphKey key{};
};

/* launch configuration: the user's (b2g_set_launch_config), else the autotuner's choice for the
 * world's size bucket if one was made in this process, else the defaults */
struct LaunchCfg {
    int coop_per_sm = 1, collide_block = 128, traverse_block = 256, solver_block = 256, collide_group = kCollideGroup;
};

std::mutex g_tune_mutex;
std::vector<std::pair<int, LaunchCfg>> g_tuned;  /* (size bucket, configuration) */

/* The step tape of a world and the work buffers of its last backward pass. */
struct TapeHost {
    bool recording = false;
    bool valid = true;
    TapeDev d{};
    std::vector<void*> mem;
    int step_cap = 0;
    long long slot_cap = 0;
    int ckpt_every = 16;
    int steps = 0;                 /* steps with dt > 0 issued while recording */
    int n_bodies = 0;
    size_t bytes = 0;
    /* backward work buffers and the sizes they were made for */
    AdjWork work{};
    std::vector<void*> work_mem;
    size_t work_bytes = 0;
    int work_slots = 0, work_vi = 0, work_pi = 0;
    unsigned mismatches = 0;
};

/* What B2gearJoint::new (private/dynamics/joints/b2_gear_joint.rs:29-137) fixes when the joint is made:
 * bodies C and D, the four local anchors, the prismatic sides' axes, the revolute sides' reference
 * angles, the sides' types and the constant coordinate_a + ratio * coordinate_b. */
struct GearFrame {
    int body_c = 0, body_d = 0;
    bool prismatic_a = false, prismatic_b = false;
    V2 anchor_a{0, 0}, anchor_b{0, 0}, anchor_c{0, 0}, anchor_d{0, 0}, axis_c{0, 0}, axis_d{0, 0};
    float ref_a = 0.0f, ref_b = 0.0f, constant = 0.0f;
};

struct World {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;  /* the device's multiprocessors, queried when the world is made */
    b2g_vec2 gravity{0.0f, -10.0f};
    int num_worlds = 1;
    bool warm = true, continuous = false, allow_sleep = true, auto_clear = true;
    int toi_schedule = 0;  /* B2G_TOI_SCHEDULE_* */
    bool asleep_seen = false;  /* a body was created asleep or put to sleep by the caller */
    bool kinematic_or_bullet = false;  /* a kinematic or bullet body exists */
    /* joints: definitions, host copies of their impulses, the colouring, body -> joints */
    std::vector<b2g_joint_def> joints;
    std::vector<GearFrame> gear;       /* per joint: a gear joint's frame, fixed at creation */
    std::vector<float4> h_jimp, h_jimp2;
    std::vector<int> h_jorder, h_jcoff, h_jnt_off, h_jnt;
    bool joints_dirty = false;          /* joints changed since the device copy */
    bool joint_filter_pending = false;  /* contacts of newly joined bodies to flag for filtering */
    int joint_cap = 0;                  /* joints the device arrays hold */
    bool record_events = false, record_pairs = false;
    bool new_contacts = false;
    float inv_dt0 = 0.0f;
    std::string err;
    int steps = 0;
    /* host mirrors (authoritative until the first upload) */
    std::vector<float4> h_xf, h_pos, h_pos0, h_vel, h_force, h_mass, h_damp;
    std::vector<float2> h_lc;
    std::vector<uint32_t> h_flags, h_world;
    std::vector<std::vector<int>> body_fixtures;  /* newest first, like the reference's fixture list */
    std::vector<ShapeRec> h_shape;
    std::vector<int> h_fbody;
    std::vector<int> h_fix_off, h_fix;  /* body -> fixtures, uploaded with the fixtures */
    std::vector<float4> h_fmat, h_fat;
    std::vector<uint32_t> h_filter, h_group, h_refid;
    std::vector<uint8_t> h_moved;
    int proxies_created = 0;       /* live proxies */
    uint32_t next_node = 0;        /* the dynamic tree's next fresh node id */
    std::vector<uint32_t> free_refids;  /* freed leaf ids, most recent last */
    /* destroyed objects keep their ids (tombstones: a body turns static and disabled, a fixture
     * loses its proxy, a joint leaves the joint colouring) */
    std::vector<uint8_t> h_bdead, h_fdead, h_jdead;
    bool host_dirty = false;       /* host mirrors were edited: the next prepare uploads them */
    std::vector<int4> pending_events;  /* end events of destructions since the last b2g_get_events */
    /* host callbacks: the user's contact filter (replacing the default one) and pre_solve */
    b2g_contact_filter_fn filter_fn = nullptr;
    void* filter_user = nullptr;
    b2g_pre_solve_fn pre_solve_fn = nullptr;
    void* pre_solve_user = nullptr;
    int hook_rc = 0;               /* the first error of a host callback round trip during a step */
    /* device */
    DevWorld d{};
    bool allocated = false;
    int uploaded_bodies = 0, uploaded_fixtures = 0;
    bool device_authoritative = false;
    std::vector<void*> allocations;
    std::vector<size_t> alloc_bytes;  /* byte size of each entry of allocations */
    std::vector<void*> alloc_field;   /* the DevWorld member each entry was allocated into (its address) */
    bool auto_grow = false;           /* b2g_set_auto_grow: contact / pair capacity grows on overflow */
    int capacity_grows = 0;
    int user_contact_cap = 0, user_pair_cap = 0;
    Timer timer;
    b2g_profile profile{};
    int last_colours = 0;
    /* CUDA graphs of the steady-state step, one per contact-buffer parity */
    bool use_graphs = true;
    bool part_solve = true;       /* b2g_set_part_solve */
    int tuning_steps = 0;         /* steps of the last b2g_autotune */
    GraphSlot graphs[2];
    int swaps = 0;
    int alloc_generation = 0;
    int minsep_buffers = 2;  /* position-iteration separation buffers held in d.isl_minsep */
    int barrier_limit_units = 0;  /* grid-barrier wait limit / 1024 cycles (0: the kernels' default) */
    int barrier_hold = 0;         /* test hook: arrivals every grid barrier waits for in vain */
    int hierarchy_max_age = 16;   /* b2g_set_hierarchy_max_age */
    TapeHost* tape = nullptr;
    LaunchCfg cfg;
    bool cfg_set = false;    /* chosen by the user or the autotuner: no bucket lookup */
    bool pageable = false;   /* the device reads/writes pageable host memory coherently */
    b2g_body_state* d_states = nullptr;  /* packing buffer for b2g_get_body_states otherwise */
    int d_states_cap = 0;
    /* b2g_get_body_states_async: two device snapshots, copied out on a second stream */
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_packed[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    b2g_body_state* d_ring[2] = {nullptr, nullptr};
    int ring_cap = 0, ring_next = 0;
    bool ring_used[2] = {false, false};
};

/* bucket: log2 of the bodies per world (batched worlds of uneven size use the mean), and
 * whether the world is a batch */
int size_bucket(const World* w) {
    const size_t nb = w->h_flags.size();
    const size_t per = nb / (size_t)(w->num_worlds > 0 ? w->num_worlds : 1);
    int b = 0;
    while ((size_t(1) << (b + 1)) <= per) ++b;
    return b * 2 + (w->num_worlds > 1 ? 1 : 0);
}

void apply_launch_config(World* w) {
    if (!w->cfg_set) {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        const int b = size_bucket(w);
        for (auto& e : g_tuned)
            if (e.first == b) w->cfg = e.second;
    }
    w->d.cfg_coop_per_sm = w->cfg.coop_per_sm;
    w->d.cfg_collide_block = w->cfg.collide_block;
    w->d.cfg_traverse_block = w->cfg.traverse_block;
    w->d.cfg_solver_block = w->cfg.coop_per_sm == 1 ? w->cfg.solver_block : 256;
    w->d.cfg_collide_group = w->cfg.collide_group;
}


/* an edit between taped steps that the tape cannot represent */
void tape_touch(World* w) {
    if (w->tape && w->tape->recording) w->tape->valid = false;
}

void tape_free_work(TapeHost* t) {
    for (void* p : t->work_mem) cudaFree(p);
    t->work_mem.clear();
    t->work_bytes = 0;
    t->work_slots = t->work_vi = t->work_pi = 0;
}

void tape_free(World* w) {
    if (!w->tape) return;
    cudaStreamSynchronize(w->stream);
    for (void* p : w->tape->mem) cudaFree(p);
    tape_free_work(w->tape);
    delete w->tape;
    w->tape = nullptr;
}

void drop_graphs(World* w) {
    for (GraphSlot& g : w->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
}

int fail(World* w, int code, const char* msg) {
    if (w) w->err = msg;
    return code;
}
int fail(World* w, int code, const std::string& msg) { return fail(w, code, msg.c_str()); }

#define CUDA_OK(w, call)                                                       \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) {                                               \
            (w)->err = std::string(#call) + ": " + cudaGetErrorString(e_);     \
            return B2G_ERR_CUDA;                                               \
        }                                                                      \
    } while (0)

/* Host-to-device copies of a world go on its stream (cudaMemcpyAsync): a plain cudaMemcpy from pageable
 * memory may return before its transfer lands and is not ordered with the world's non-blocking stream. */

template <class T>
int dalloc(World* w, T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        w->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return B2G_ERR_OUT_OF_MEMORY;
    }
    w->allocations.push_back((void*)*p);
    w->alloc_bytes.push_back(n * sizeof(T));
    w->alloc_field.push_back((void*)p);
    cudaMemsetAsync(*p, 0, n * sizeof(T), w->stream);
    return B2G_OK;
}

/* forgets entry k of the allocation list (the caller frees the memory) */
void drop_allocation(World* w, size_t k) {
    w->alloc_bytes.erase(w->alloc_bytes.begin() + k);
    w->alloc_field.erase(w->alloc_field.begin() + k);
    w->allocations.erase(w->allocations.begin() + k);
}

void drop_graphs(World* w);

/* frees one dalloc'd buffer */
template <class T>
void dfree(World* w, T** p) {
    if (!*p) return;
    auto it = std::find(w->allocations.begin(), w->allocations.end(), (void*)*p);
    if (it != w->allocations.end()) drop_allocation(w, (size_t)(it - w->allocations.begin()));
    cudaFree(*p);
    *p = nullptr;
}

void free_all(World* w) {
    drop_graphs(w);
    for (void* p : w->allocations) cudaFree(p);
    w->allocations.clear();
    w->alloc_bytes.clear();
    w->alloc_field.clear();
    w->joint_cap = 0;
    w->d.j_body = nullptr;  /* the joint arrays went with the rest */
    w->allocated = false;
    ++w->alloc_generation;
}

int bits_for(uint64_t v) {
    int b = 1;
    while ((1ull << b) <= v) ++b;
    return b;
}

/* ---- creation-time geometry (host) ---- */

/* B2polygonShape::set_as_box, private/collision/b2_polygon_shape.rs:12-23 */
void polygon_box(ShapeRec& s, float hx, float hy) {
    s.v[0] = mk(-hx, -hy);
    s.v[1] = mk(hx, -hy);
    s.v[2] = mk(hx, hy);
    s.v[3] = mk(-hx, hy);
    s.n[0] = mk(0.0f, -1.0f);
    s.n[1] = mk(1.0f, 0.0f);
    s.n[2] = mk(0.0f, 1.0f);
    s.n[3] = mk(-1.0f, 0.0f);
    s.centroid = mk(0.0f, 0.0f);
    s.meta = SHAPE_POLYGON | (4 << 8);
}

/* polygon centroid, b2_polygon_shape.rs:53-77 */
V2 polygon_centroid(const V2* vs, int count) {
    V2 c = mk(0.0f, 0.0f);
    float area = 0.0f;
    const V2 s = vs[0];
    const float inv3 = 1.0f / 3.0f;
    for (int i = 0; i < count; ++i) {
        V2 p1 = sub(vs[0], s);
        V2 p2 = sub(vs[i], s);
        V2 p3 = (i + 1 < count) ? sub(vs[i + 1], s) : sub(vs[0], s);
        V2 e1 = sub(p2, p1);
        V2 e2 = sub(p3, p1);
        float d = cross(e1, e2);
        float tri = 0.5f * d;
        area += tri;
        c = add(c, scale(tri * inv3, add(add(p1, p2), p3)));
    }
    return add(scale(1.0f / area, c), s);
}

/* B2polygonShape::set (gift wrapping), b2_polygon_shape.rs:96-211; false -> unit box fallback */
bool polygon_hull(ShapeRec& s, const b2g_vec2* in, int count) {
    if (count < 3) {
        polygon_box(s, 1.0f, 1.0f);
        return false;
    }
    int n = count < kMaxPolygonVertices ? count : kMaxPolygonVertices;
    V2 ps[kMaxPolygonVertices];
    int temp = 0;
    for (int i = 0; i < n; ++i) {
        V2 v = mk(in[i].x, in[i].y);
        bool unique = true;
        for (int j = 0; j < temp; ++j) {
            if (dist_sq(v, ps[j]) < ((0.5f * kLinearSlop) * (0.5f * kLinearSlop))) {
                unique = false;
                break;
            }
        }
        if (unique) ps[temp++] = v;
    }
    n = temp;
    if (n < 3) {
        polygon_box(s, 1.0f, 1.0f);
        return false;
    }
    int i0 = 0;
    float x0 = ps[0].x;
    for (int i = 1; i < n; ++i) {
        float x = ps[i].x;
        if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) {
            i0 = i;
            x0 = x;
        }
    }
    int hull[kMaxPolygonVertices];
    int m = 0, ih = i0;
    for (;;) {
        if (m >= kMaxPolygonVertices) {
            polygon_box(s, 1.0f, 1.0f);
            return false;
        }
        hull[m] = ih;
        int ie = 0;
        for (int j = 1; j < n; ++j) {
            if (ie == ih) {
                ie = j;
                continue;
            }
            V2 r = sub(ps[ie], ps[hull[m]]);
            V2 v = sub(ps[j], ps[hull[m]]);
            float c = cross(r, v);
            if (c < 0.0f) ie = j;
            if (c == 0.0f && length_sq(v) > length_sq(r)) ie = j;
        }
        ++m;
        ih = ie;
        if (ie == i0) break;
    }
    if (m < 3) {
        polygon_box(s, 1.0f, 1.0f);
        return false;
    }
    for (int i = 0; i < m; ++i) s.v[i] = ps[hull[i]];
    for (int i = 0; i < m; ++i) {
        int i2 = (i + 1 < m) ? i + 1 : 0;
        s.n[i] = cross_vs(sub(s.v[i2], s.v[i]), 1.0f);
        normalize(s.n[i]);
    }
    s.centroid = polygon_centroid(s.v, m);
    s.meta = SHAPE_POLYGON | (m << 8);
    return true;
}

void build_shape(const b2g_fixture_def& d, ShapeRec& s) {
    memset(&s, 0, sizeof(s));
    s.radius = d.radius;
    if (d.shape_type == B2G_SHAPE_CIRCLE) {
        s.v[0] = mk(d.vertices[0].x, d.vertices[0].y);
        s.meta = SHAPE_CIRCLE | (1 << 8);
    } else if (d.shape_type == B2G_SHAPE_EDGE) {
        for (int i = 0; i < 4; ++i) s.v[i] = mk(d.vertices[i].x, d.vertices[i].y);
        s.meta = SHAPE_EDGE | (2 << 8) | ((d.one_sided ? 1 : 0) << 16);
    } else {
        if (d.polygon_mode == B2G_POLYGON_BOX) {
            polygon_box(s, d.box_half_extents.x, d.box_half_extents.y);
        } else if (d.polygon_mode == B2G_POLYGON_BOX_ORIENTED) {
            /* set_as_box_angle, b2_polygon_shape.rs:25-50 */
            polygon_box(s, d.box_half_extents.x, d.box_half_extents.y);
            Xf xf;
            xf.p = mk(d.box_center.x, d.box_center.y);
            xf.q = rot(d.box_angle);
            s.centroid = xf.p;
            for (int i = 0; i < 4; ++i) {
                s.v[i] = mul(xf, s.v[i]);
                s.n[i] = mul(xf.q, s.n[i]);
            }
        } else {
            polygon_hull(s, d.vertices, d.vertex_count);
        }
        s.radius = d.radius;
    }
}

/* compute_mass of each shape: b2_polygon_shape.rs:314-390, b2_circle_shape.rs:79-86, b2_edge_shape.rs:126-132 */
void shape_mass(const ShapeRec& s, float density, float& mass, V2& center, float& I) {
    const int t = shape_type(s);
    if (t == SHAPE_CIRCLE) {
        mass = density * kPi * s.radius * s.radius;
        center = s.v[0];
        I = mass * (0.5f * s.radius * s.radius + dot(s.v[0], s.v[0]));
    } else if (t == SHAPE_EDGE) {
        mass = 0.0f;
        center = scale(0.5f, add(s.v[1], s.v[2]));
        I = 0.0f;
    } else {
        const int n = shape_count(s);
        V2 c = mk(0.0f, 0.0f);
        float area = 0.0f, inert = 0.0f;
        const V2 o = s.v[0];
        const float inv3 = 1.0f / 3.0f;
        for (int i = 0; i < n; ++i) {
            V2 e1 = sub(s.v[i], o);
            V2 e2 = (i + 1 < n) ? sub(s.v[i + 1], o) : sub(s.v[0], o);
            float d = cross(e1, e2);
            float tri = 0.5f * d;
            area += tri;
            c = add(c, scale(tri * inv3, add(e1, e2)));
            float intx2 = e1.x * e1.x + e2.x * e1.x + e2.x * e2.x;
            float inty2 = e1.y * e1.y + e2.y * e1.y + e2.y * e2.y;
            inert += ((0.25f * inv3) * d) * (intx2 + inty2);
        }
        mass = density * area;
        c = scale(1.0f / area, c);
        center = add(c, o);
        I = density * inert;
        I += mass * (dot(center, center) - dot(c, c));
    }
}

Xf host_xf(const World* w, int b) {
    Xf x;
    x.p = mk(w->h_xf[b].x, w->h_xf[b].y);
    x.q.s = w->h_xf[b].z;
    x.q.c = w->h_xf[b].w;
    return x;
}

/* reset_mass_data, private/dynamics/b2_body.rs:292-350 */
void reset_mass_data(World* w, int b) {
    float4& pos = w->h_pos[b];
    float4& pos0 = w->h_pos0[b];
    float4& m = w->h_mass[b];
    float4& v = w->h_vel[b];
    const uint32_t fl = w->h_flags[b];
    const Xf xf = host_xf(w, b);
    m = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w->h_lc[b] = make_float2(0.0f, 0.0f);
    const int type = (int)(fl & BF_TYPE_MASK);
    if (type != BODY_DYNAMIC) {
        pos = make_float4(xf.p.x, xf.p.y, pos.z, 0.0f);
        pos0 = make_float4(xf.p.x, xf.p.y, pos.z, 0.0f);
        return;
    }
    V2 lc = mk(0.0f, 0.0f);
    float mass = 0.0f, I = 0.0f, inv_mass = 0.0f, inv_I = 0.0f;
    for (int f : w->body_fixtures[b]) {
        const float density = w->h_fmat[f].w;
        if (density == 0.0f) continue;
        float fm, fi;
        V2 fc;
        shape_mass(w->h_shape[f], density, fm, fc, fi);
        mass += fm;
        lc = add(lc, scale(fm, fc));
        I += fi;
    }
    if (mass > 0.0f) {
        inv_mass = 1.0f / mass;
        lc.x *= inv_mass;
        lc.y *= inv_mass;
    }
    if (I > 0.0f && !(fl & BF_FIXED_ROTATION)) {
        I -= mass * dot(lc, lc);
        inv_I = 1.0f / I;
    } else {
        I = 0.0f;
        inv_I = 0.0f;
    }
    m = make_float4(mass, inv_mass, I, inv_I);
    const V2 old_center = mk(pos.x, pos.y);
    w->h_lc[b] = make_float2(lc.x, lc.y);
    const V2 c0 = mul(xf, lc);
    pos = make_float4(c0.x, c0.y, pos.z, 0.0f);
    pos0 = make_float4(c0.x, c0.y, pos0.z, 0.0f);
    const V2 dv = cross_sv(v.z, sub(c0, old_center));
    v.x += dv.x;
    v.y += dv.y;
}

/* a new proxy's id: the most recently freed leaf, else the next fresh node (a leaf and, unless the tree
 * is empty, its parent) */
uint32_t alloc_refid(World* w) {
    uint32_t id;
    if (!w->free_refids.empty()) {
        id = w->free_refids.back();
        w->free_refids.pop_back();
    } else {
        id = w->next_node;
        w->next_node += w->proxies_created == 0 ? 1u : 2u;
    }
    ++w->proxies_created;
    return id;
}

void free_refid(World* w, uint32_t id) {
    w->free_refids.push_back(id);
    --w->proxies_created;
}

/* host copy of the fat-AABB rule of B2dynamicTree::move_proxy (private/collision/b2_dynamic_tree.rs:109-168) */
void host_move_proxy(World* w, int f, const AABB& aabb, V2 disp) {
    const V2 r = mk(kAabbExtension, kAabbExtension);
    AABB fat;
    fat.lo = sub(aabb.lo, r);
    fat.hi = add(aabb.hi, r);
    const V2 d = scale(kAabbMultiplier, disp);
    if (d.x < 0.0f) fat.lo.x += d.x; else fat.hi.x += d.x;
    if (d.y < 0.0f) fat.lo.y += d.y; else fat.hi.y += d.y;
    const float4 t = w->h_fat[f];
    AABB tree;
    tree.lo = mk(t.x, t.y);
    tree.hi = mk(t.z, t.w);
    if (contains(tree, aabb)) {
        AABB huge;
        huge.lo = sub(fat.lo, scale(4.0f, r));
        huge.hi = add(fat.hi, scale(4.0f, r));
        if (contains(huge, tree)) return;
    }
    w->h_fat[f] = make_float4(fat.lo.x, fat.lo.y, fat.hi.x, fat.hi.y);
    w->h_moved[f] = 1;
}

/* ---- device allocation, upload and download ---- */

/* the grid-barrier settings into the device's counter block (read by every grid barrier) */
int write_barrier_settings(World* w) {
    if (!w->allocated) return B2G_OK;
    const int v[2] = {w->barrier_limit_units, w->barrier_hold};
    CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_BARRIER_LIMIT, v, sizeof(v), cudaMemcpyHostToDevice, w->stream));
    const int age = w->hierarchy_max_age;
    CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_BP_MAX_AGE, &age, sizeof(age), cudaMemcpyHostToDevice, w->stream));
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    return B2G_OK;
}

/* keep_body_cap / keep_fix_cap (when > 0): the body and fixture capacities to keep, so that a
 * reallocation that only grows the contact and pair capacities keeps every per-body and per-fixture
 * array's layout */
int allocate(World* w, int nb, int nf, int keep_body_cap = 0, int keep_fix_cap = 0) {
    DevWorld& d = w->d;
    const int body_cap = keep_body_cap > 0 ? keep_body_cap : nb + nb / 4 + 1024;
    const int fix_cap = keep_fix_cap > 0 ? keep_fix_cap : nf + nf / 4 + 1024;
    /* a capacity given in b2g_world_def is used as is; 0 picks one proportional to the fixtures */
    const int contact_cap = w->user_contact_cap > 0 ? w->user_contact_cap : 6 * fix_cap + 4096;
    const int pair_cap = w->user_pair_cap > 0 ? w->user_pair_cap : 4 * fix_cap + 4096;
    d.body_cap = body_cap;
    d.fix_cap = fix_cap;
    d.contact_cap = contact_cap;
    d.pair_cap = pair_cap;
    d.event_cap = contact_cap;
    d.cons_cap = contact_cap;
    d.num_worlds = w->num_worlds;
    apply_launch_config(w);
    int rc = B2G_OK;
#define A(ptr, n)                                      \
    do {                                               \
        if ((rc = dalloc(w, &(ptr), (size_t)(n))) != B2G_OK) return rc; \
    } while (0)
    A(d.b_xf, body_cap); A(d.b_pos, body_cap); A(d.b_pos0, body_cap); A(d.b_vel, body_cap);
    A(d.b_force, body_cap); A(d.b_mass, body_cap); A(d.b_damp, body_cap); A(d.b_lc, body_cap);
    A(d.b_flags, body_cap); A(d.b_world, body_cap); A(d.b_island, body_cap); A(d.b_rank, body_cap);
    A(d.b_part, body_cap); A(d.b_cidx, body_cap);
    A(d.b_cmin, 4 * (size_t)body_cap); A(d.b_cmask, 2 * (size_t)body_cap);
    /* one per-island separation buffer per position iteration (at least 2: the island pass
     * uses the second as its "has an awake member" flag) */
    w->minsep_buffers = std::max(2, w->minsep_buffers);
    A(d.isl_minsep, (size_t)w->minsep_buffers * body_cap); A(d.isl_done, body_cap); A(d.isl_sleep, body_cap);
    A(d.b_wake, body_cap); A(d.b_dwake, body_cap); A(d.c_done, contact_cap);
    cudaMemsetAsync(d.b_wake, 0x7f, (size_t)body_cap * sizeof(int), w->stream);  /* kNoWake */
    A(d.f_shape, fix_cap); A(d.f_vn, (size_t)kMaxPolygonVertices * fix_cap); A(d.f_hdr, fix_cap);
    A(d.f_body, fix_cap); A(d.f_mat, fix_cap); A(d.f_filter, fix_cap); A(d.f_group, fix_cap);
    A(d.f_refid, fix_cap); A(d.f_fat, fix_cap); A(d.f_moved, fix_cap);
    Contacts* cs[2] = {&d.c, &d.c_alt};
    for (Contacts* c : cs) {
        A(c->key, contact_cap); A(c->fix, contact_cap); A(c->body, contact_cap); A(c->flags, contact_cap);
        A(c->mat, contact_cap); A(c->mgeo, contact_cap); A(c->mpts, contact_cap); A(c->mimp, contact_cap);
        A(c->mids, contact_cap);
    }
    A(d.c_rank, contact_cap); A(d.c_row, 2 * (size_t)fix_cap + 2); A(d.c_row_end, 2 * (size_t)fix_cap + 2);
    A(d.n_key, pair_cap); A(d.n_fix, pair_cap); A(d.n_idx, pair_cap); A(d.n_key_alt, pair_cap); A(d.n_idx_alt, pair_cap);
    A(d.cons_contact, contact_cap); A(d.cons_colour, contact_cap); A(d.cons_island, contact_cap);
    A(d.s_contact, contact_cap); A(d.s_cons, contact_cap); A(d.s_fix, contact_cap);
    A(d.cons_part, contact_cap); A(d.col_tail, kColourTail);
    A(d.col_off, kMaxColours + 1); A(d.col_hist, (size_t)(kMaxParts + 1) * kMaxColours);
    A(d.part_off, (size_t)kMaxParts * (kMaxColours + 1)); A(d.part_ncol, kMaxParts); A(d.part_tot, kMaxParts + 1);
    A(d.rank_x, fix_cap); A(d.blk_tot, std::max(kMaxParts, 8 * w->num_sms)); A(d.cache_body, fix_cap);
    A(d.part_cbeg, kMaxParts); A(d.part_cend, kMaxParts); A(d.part_rbeg, kMaxParts);
    A(d.vc_idx, contact_cap); A(d.vc_inv, contact_cap); A(d.vc_nf, contact_cap); A(d.vc_r0, contact_cap);
    A(d.vc_r1, contact_cap); A(d.vc_m0, contact_cap); A(d.vc_m1, contact_cap); A(d.vc_imp, contact_cap);
    A(d.vc_k, contact_cap); A(d.vc_island, contact_cap); A(d.vc_code, contact_cap);
    A(d.pc_lp, contact_cap); A(d.pc_geo, contact_cap); A(d.pc_lc, contact_cap); A(d.pc_inv, contact_cap);
    A(d.pc_meta, contact_cap);
    A(d.bp_key, fix_cap); A(d.bp_val, fix_cap); A(d.bp_key_alt, fix_cap); A(d.bp_val_alt, fix_cap);
    A(d.bp_leaf, fix_cap); A(d.bp_node_b0, fix_cap); A(d.bp_node_b1, fix_cap); A(d.bp_node_child, fix_cap);
    A(d.bp_parent, 2 * (size_t)fix_cap); A(d.bp_flag, fix_cap);
    A(d.bp_quad_box, 4 * (size_t)fix_cap); A(d.bp_quad_child, fix_cap);
    A(d.bp_world_root, 2 * (size_t)w->num_worlds); A(d.bp_world_first, 2 * (size_t)w->num_worlds);
    A(d.b_fix_off, (size_t)body_cap + 1); A(d.b_fix, fix_cap);
    A(d.b_jnt_off, (size_t)body_cap + 1);
    A(d.b_alpha0, body_cap); A(d.b_stamp, body_cap); A(d.b_event, body_cap); A(d.b_inval, body_cap);
    A(d.b_cx, body_cap); A(d.b_sync, body_cap); A(d.b_best, body_cap); A(d.b_bkey, body_cap);
    A(d.f_leaf, fix_cap);
    A(d.t_toi, contact_cap); A(d.t_when, contact_cap); A(d.t_count, contact_cap);
    A(d.t_elig, contact_cap); A(d.t_hits, contact_cap); A(d.t_hitx, contact_cap); A(d.t_sync, body_cap);
    A(d.t_moved, fix_cap); A(d.t_nkey, kToiNewCap); A(d.t_nslot, kToiNewCap);
    A(d.ev_contact, kToiEvCap); A(d.ev_alpha, kToiEvCap); A(d.ev_solid, kToiEvCap);
    A(d.ev_cand, (size_t)kToiEvCap * (kToiCand + 1));
    A(d.tw_alpha, w->num_worlds); A(d.tw_key, w->num_worlds); A(d.tw_salpha, w->num_worlds); A(d.tw_skey, w->num_worlds);
    A(d.s_xf, body_cap); A(d.s_pos, body_cap); A(d.s_pos0, body_cap); A(d.s_vel, body_cap); A(d.s_flags, body_cap);
    A(d.s_fat, fix_cap);
    A(d.events, d.event_cap);
    A(d.pairs, pair_cap);
    A(d.scan_tmp, 2 * (size_t)contact_cap + scan_tmp_size(contact_cap) + 64);
    const size_t hist = radix_sort_hist_size(std::max(fix_cap, pair_cap));
    A(d.sort_hist, hist);
    A(d.cnt, CNT_SIZE);
#undef A
    w->allocated = true;
    return write_barrier_settings(w);
}

int upload(World* w) {
    DevWorld& d = w->d;
    const int nb = (int)w->h_flags.size();
    const int nf = (int)w->h_fbody.size();
    cudaStream_t s = w->stream;
#define U(dst, src) CUDA_OK(w, cudaMemcpyAsync((dst), (src).data(), (src).size() * sizeof((src)[0]), cudaMemcpyHostToDevice, s))
    if (nb > 0) {
        U(d.b_xf, w->h_xf); U(d.b_pos, w->h_pos); U(d.b_pos0, w->h_pos0); U(d.b_vel, w->h_vel);
        U(d.b_force, w->h_force); U(d.b_mass, w->h_mass); U(d.b_damp, w->h_damp); U(d.b_lc, w->h_lc);
        U(d.b_flags, w->h_flags); U(d.b_world, w->h_world);
    }
    if (nf > 0) {
        U(d.f_shape, w->h_shape); U(d.f_body, w->h_fbody); U(d.f_mat, w->h_fmat); U(d.f_filter, w->h_filter);
        U(d.f_group, w->h_group); U(d.f_refid, w->h_refid); U(d.f_fat, w->h_fat); U(d.f_moved, w->h_moved);
        launch_shape_rows(d, nf, s);  /* the narrowphase's structure-of-arrays copy of f_shape */
    }
    /* body -> fixtures (the continuous pass synchronises an island body's proxies) */
    w->h_fix_off.assign((size_t)nb + 1, 0);
    for (int f = 0; f < nf; ++f) ++w->h_fix_off[(size_t)w->h_fbody[f] + 1];
    for (int b = 0; b < nb; ++b) w->h_fix_off[(size_t)b + 1] += w->h_fix_off[b];
    w->h_fix.assign((size_t)std::max(nf, 1), 0);
    {
        std::vector<int> fill(w->h_fix_off.begin(), w->h_fix_off.end() - 1);
        for (int f = 0; f < nf; ++f) w->h_fix[(size_t)fill[w->h_fbody[f]]++] = f;
    }
    U(d.b_fix_off, w->h_fix_off);
    if (nf > 0) U(d.b_fix, w->h_fix);
#undef U
    /* proxies may have changed (created, destroyed, moved or re-filtered on the host): the next
     * broadphase pass rebuilds its hierarchy */
    CUDA_OK(w, cudaMemsetAsync(d.cnt + CNT_BP_FORCE, 1, sizeof(int), s));
    CUDA_OK(w, cudaStreamSynchronize(s));
    w->uploaded_bodies = nb;
    w->uploaded_fixtures = nf;
    w->host_dirty = false;
    d.n_bodies = nb;
    d.n_fixtures = nf;
    return B2G_OK;
}

/* device -> host mirrors for bodies and fixtures (before host-side edits after stepping). With host edits
 * pending (host_dirty) the mirrors are already current: every device-side operation uploads them first. */
int download_state(World* w) {
    if (w->host_dirty) return B2G_OK;
    DevWorld& d = w->d;
    const int nb = w->uploaded_bodies;
    const int nf = w->uploaded_fixtures;
    cudaStream_t s = w->stream;
#define D(src, dst, n) CUDA_OK(w, cudaMemcpyAsync((dst).data(), (src), (size_t)(n) * sizeof((dst)[0]), cudaMemcpyDeviceToHost, s))
    if (nb > 0) {
        D(d.b_xf, w->h_xf, nb); D(d.b_pos, w->h_pos, nb); D(d.b_pos0, w->h_pos0, nb); D(d.b_vel, w->h_vel, nb);
        D(d.b_force, w->h_force, nb); D(d.b_flags, w->h_flags, nb);
    }
    if (nf > 0) {
        D(d.f_fat, w->h_fat, nf); D(d.f_moved, w->h_moved, nf);
    }
#undef D
    CUDA_OK(w, cudaStreamSynchronize(s));
    return B2G_OK;
}

inline float __uint_as_float_host(uint32_t u) {
    float f;
    memcpy(&f, &u, sizeof(f));
    return f;
}

/* The joints' impulses from the device into the host copies (before the device arrays change) */
int download_joint_impulses(World* w) {
    const int n = w->d.n_joints;
    if (w->joint_cap == 0 || n == 0 || !w->device_authoritative) return B2G_OK;
    CUDA_OK(w, cudaMemcpy(w->h_jimp.data(), w->d.j_imp, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(w->h_jimp2.data(), w->d.j_imp2, n * sizeof(float4), cudaMemcpyDeviceToHost));
    return B2G_OK;
}

/* (Re)allocates the joint table for cap joints (its contents start at zero). */
int alloc_joint_arrays(World* w, int cap) {
    DevWorld& d = w->d;
    dfree(w, &d.j_body); dfree(w, &d.j_body2); dfree(w, &d.j_anchor); dfree(w, &d.j_lim); dfree(w, &d.j_par);
    dfree(w, &d.j_imp); dfree(w, &d.j_imp2); dfree(w, &d.j_rr); dfree(w, &d.j_k); dfree(w, &d.j_m); dfree(w, &d.j_s);
    dfree(w, &d.j_x); dfree(w, &d.j_order); dfree(w, &d.j_coff); dfree(w, &d.b_jnt);
    int rc = B2G_OK;
    if ((rc = dalloc(w, &d.j_body, cap)) || (rc = dalloc(w, &d.j_body2, cap)) || (rc = dalloc(w, &d.j_anchor, cap)) ||
        (rc = dalloc(w, &d.j_lim, cap)) || (rc = dalloc(w, &d.j_par, cap)) || (rc = dalloc(w, &d.j_imp, cap)) ||
        (rc = dalloc(w, &d.j_imp2, cap)) || (rc = dalloc(w, &d.j_rr, cap)) || (rc = dalloc(w, &d.j_k, cap)) ||
        (rc = dalloc(w, &d.j_m, cap)) || (rc = dalloc(w, &d.j_s, cap)) || (rc = dalloc(w, &d.j_x, cap)) ||
        (rc = dalloc(w, &d.j_order, cap)) || (rc = dalloc(w, &d.j_coff, kMaxJointColours + 1)) ||
        (rc = dalloc(w, &d.b_jnt, 2 * (size_t)cap)))
        return rc;
    w->joint_cap = cap;
    drop_graphs(w);
    ++w->alloc_generation;
    return B2G_OK;
}

/* Grows the contact and pair capacities in place: every buffer is reallocated with the same body and
 * fixture capacities and the old contents copied to the front of its successor, matched by the
 * DevWorld member that holds it (the contact tables trade members at every swap), so the contact
 * table, the colouring and partition state and every other persistent array carry over unchanged. */
int grow_capacities(World* w, int contact_cap, int pair_cap) {
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    const std::vector<void*> old_ptr = w->allocations, old_field = w->alloc_field;
    const std::vector<size_t> old_bytes = w->alloc_bytes;
    /* the buffer each member holds now and its size */
    std::vector<void*> held(old_field.size());
    std::vector<size_t> held_bytes(old_field.size(), 0);
    for (size_t i = 0; i < old_field.size(); ++i) {
        held[i] = *(void**)old_field[i];
        const auto it = std::find(old_ptr.begin(), old_ptr.end(), held[i]);
        if (it != old_ptr.end()) held_bytes[i] = old_bytes[(size_t)(it - old_ptr.begin())];
    }
    const int joint_cap = w->joint_cap;
    drop_graphs(w);
    w->allocations.clear();
    w->alloc_bytes.clear();
    w->alloc_field.clear();
    DevWorld& d = w->d;
    /* the old joint buffers are still referenced by d: forget them so the reallocation frees nothing */
    d.j_body = d.j_body2 = nullptr;
    d.j_anchor = d.j_lim = d.j_par = d.j_imp = d.j_imp2 = d.j_rr = d.j_k = d.j_m = d.j_x = nullptr;
    d.j_s = nullptr;
    d.j_order = d.j_coff = d.b_jnt = nullptr;
    w->joint_cap = 0;
    w->allocated = false;
    w->user_contact_cap = contact_cap;
    w->user_pair_cap = pair_cap;
    int rc = allocate(w, d.n_bodies, d.n_fixtures, d.body_cap, d.fix_cap);
    if (rc == B2G_OK && joint_cap > 0) rc = alloc_joint_arrays(w, joint_cap);
    if (rc == B2G_OK) {
        /* keep the relation between the swap parity and the table buffers that a saved state records:
         * with an odd number of swaps the current table is the one allocated second */
        if (w->swaps & 1) std::swap(d.c, d.c_alt);
        /* on the world's stream, after the new buffers' zero fill and before any later launch */
        for (size_t i = 0; i < w->allocations.size() && rc == B2G_OK; ++i) {
            size_t k = old_field.size();  /* the member that holds this buffer now */
            for (size_t f = 0; f < old_field.size() && k == old_field.size(); ++f)
                if (*(void**)old_field[f] == w->allocations[i]) k = f;
            if (k == old_field.size() || !held[k] || held_bytes[k] == 0) continue;
            const cudaError_t e = cudaMemcpyAsync(w->allocations[i], held[k], std::min(held_bytes[k], w->alloc_bytes[i]),
                                                  cudaMemcpyDeviceToDevice, w->stream);
            if (e != cudaSuccess) rc = fail(w, B2G_ERR_CUDA, cudaGetErrorString(e));
        }
        const cudaError_t e = cudaStreamSynchronize(w->stream);
        if (rc == B2G_OK && e != cudaSuccess) rc = fail(w, B2G_ERR_CUDA, cudaGetErrorString(e));
    }
    for (void* p : old_ptr) cudaFree(p);
    if (rc != B2G_OK) return rc;
    ++w->capacity_grows;
    ++w->alloc_generation;
    return write_barrier_settings(w);
}

/* Uploads the joints: definitions, impulses, the colouring (greedy, in creation order: a joint takes
 * the first colour no earlier joint on one of its dynamic bodies has, so joints of a colour share no
 * body the solver writes) and body -> joints. */
int upload_joints(World* w) {
    DevWorld& d = w->d;
    const int nj = (int)w->joints.size();
    const int nb = (int)w->h_flags.size();
    cudaStream_t s = w->stream;
    if (nj > w->joint_cap) {
        const int rc = alloc_joint_arrays(w, nj);
        if (rc != B2G_OK) return rc;
    }
    std::vector<int> colour(nj, 0);
    std::vector<uint64_t> used(nb, 0);
    int ncol = 0;
    int nlive = 0;
    for (int j = 0; j < nj; ++j) {
        if (w->h_jdead[j]) continue;  /* a destroyed joint is in no colour */
        ++nlive;
        /* the bodies the joint writes: A and B, and a gear joint's C and D */
        uint32_t jb[4] = {w->joints[j].body_a, w->joints[j].body_b, 0u, 0u};
        int nbj = 2;
        if (w->joints[j].type == B2G_JOINT_GEAR) {
            jb[2] = (uint32_t)w->gear[j].body_c;
            jb[3] = (uint32_t)w->gear[j].body_d;
            nbj = 4;
        }
        uint64_t busy = 0;
        for (int k = 0; k < nbj; ++k)
            if ((w->h_flags[jb[k]] & BF_TYPE_MASK) == BODY_DYNAMIC) busy |= used[jb[k]];
        int c = 0;
        while (c < kMaxJointColours && (busy >> c) & 1ull) ++c;
        if (c == kMaxJointColours) return fail(w, B2G_ERR_CAPACITY, "a body has more joints than the joint colouring holds (64)");
        colour[j] = c;
        for (int k = 0; k < nbj; ++k)
            if ((w->h_flags[jb[k]] & BF_TYPE_MASK) == BODY_DYNAMIC) used[jb[k]] |= 1ull << c;
        ncol = std::max(ncol, c + 1);
    }
    w->h_jcoff.assign(kMaxJointColours + 1, 0);
    for (int j = 0; j < nj; ++j)
        if (!w->h_jdead[j]) ++w->h_jcoff[colour[j] + 1];
    for (int c = 0; c < kMaxJointColours; ++c) w->h_jcoff[c + 1] += w->h_jcoff[c];
    w->h_jorder.assign(nlive, 0);
    {
        std::vector<int> fill(w->h_jcoff.begin(), w->h_jcoff.end() - 1);
        for (int j = 0; j < nj; ++j)
            if (!w->h_jdead[j]) w->h_jorder[fill[colour[j]]++] = j;
    }
    w->h_jnt_off.assign((size_t)nb + 1, 0);
    for (int j = 0; j < nj; ++j) {
        if (w->h_jdead[j]) continue;
        ++w->h_jnt_off[(size_t)w->joints[j].body_a + 1];
        ++w->h_jnt_off[(size_t)w->joints[j].body_b + 1];
    }
    for (int b = 0; b < nb; ++b) w->h_jnt_off[(size_t)b + 1] += w->h_jnt_off[b];
    w->h_jnt.assign(std::max(2 * nj, 1), 0);
    {
        std::vector<int> fill(w->h_jnt_off.begin(), w->h_jnt_off.end() - 1);
        for (int j = 0; j < nj; ++j) {
            if (w->h_jdead[j]) continue;
            w->h_jnt[(size_t)fill[w->joints[j].body_a]++] = j;
            w->h_jnt[(size_t)fill[w->joints[j].body_b]++] = j;
        }
    }
#define U(dst, src, n) CUDA_OK(w, cudaMemcpyAsync((dst), (src), (size_t)(n) * sizeof(*(dst)), cudaMemcpyHostToDevice, s))
    U(d.b_jnt_off, w->h_jnt_off.data(), nb + 1);
    if (nj > 0) {
        std::vector<int2> jb(nj), jb2(nj);
        std::vector<float4> an(nj), lim(nj), par(nj), jx(nj);
        std::vector<float2> js(nj);
        for (int j = 0; j < nj; ++j) {
            const b2g_joint_def& jd = w->joints[j];
            /* a destroyed joint joins no islands: its body pair is (a, a) */
            jb[j] = w->h_jdead[j] ? make_int2((int)jd.body_a, (int)jd.body_a) : make_int2((int)jd.body_a, (int)jd.body_b);
            jb2[j] = jb[j];
            jx[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            js[j] = make_float2(0.0f, 0.0f);
            an[j] = make_float4(jd.local_anchor_a.x, jd.local_anchor_a.y, jd.local_anchor_b.x, jd.local_anchor_b.y);
            uint32_t fl = ((uint32_t)jd.type << JF_TYPE_SHIFT) | (jd.collide_connected ? JF_COLLIDE : 0u);
            if (jd.type == B2G_JOINT_GEAR) {
                const GearFrame& g = w->gear[j];
                jb2[j] = make_int2(g.body_c, g.body_d);
                an[j] = make_float4(g.anchor_a.x, g.anchor_a.y, g.anchor_b.x, g.anchor_b.y);
                lim[j] = make_float4(g.anchor_c.x, g.anchor_c.y, g.anchor_d.x, g.anchor_d.y);
                jx[j] = make_float4(g.axis_c.x, g.axis_c.y, g.axis_d.x, g.axis_d.y);
                js[j] = make_float2(g.ref_a, g.ref_b);
                fl |= (g.prismatic_a ? JF_GEAR_A_PRISMATIC : 0u) | (g.prismatic_b ? JF_GEAR_B_PRISMATIC : 0u);
                par[j] = make_float4(jd.ratio, __uint_as_float_host(fl), g.constant, 0.0f);
                continue;
            }
            if (jd.type == B2G_JOINT_PULLEY) {
                /* the constant length_a + ratio * length_b (b2_pulley_joint.rs:33) is formed on the device */
                lim[j] = make_float4(jd.ground_anchor_a.x, jd.ground_anchor_a.y, jd.ground_anchor_b.x, jd.ground_anchor_b.y);
                par[j] = make_float4(jd.ratio, __uint_as_float_host(fl), jd.length_a, jd.length_b);
            } else if (jd.type == B2G_JOINT_WHEEL) {
                lim[j] = make_float4(jd.lower_translation, jd.upper_translation, jd.motor_speed, jd.max_motor_torque);
                fl |= (jd.enable_limit ? JF_LIMIT : 0u) | (jd.enable_motor ? JF_MOTOR : 0u);
                par[j] = make_float4(jd.stiffness, __uint_as_float_host(fl), jd.local_axis_a.x, jd.local_axis_a.y);
            } else if (jd.type == B2G_JOINT_PRISMATIC) {
                /* B2prismaticJoint::new (private/dynamics/joints/b2_prismatic_joint.rs:54-60): unit axis */
                V2 ax = mk(jd.local_axis_a.x, jd.local_axis_a.y);
                normalize(ax);
                lim[j] = make_float4(jd.lower_translation, jd.upper_translation, jd.motor_speed, jd.max_motor_force);
                fl |= (jd.enable_limit ? JF_LIMIT : 0u) | (jd.enable_motor ? JF_MOTOR : 0u);
                par[j] = make_float4(jd.reference_angle, __uint_as_float_host(fl), ax.x, ax.y);
            } else if (jd.type == B2G_JOINT_MOUSE) {
                an[j] = make_float4(jd.target.x, jd.target.y, jd.local_anchor_b.x, jd.local_anchor_b.y);
                lim[j] = make_float4(jd.max_force, jd.stiffness, jd.damping, 0.0f);
                par[j] = make_float4(0.0f, __uint_as_float_host(fl), 0.0f, 0.0f);
            } else if (jd.type == B2G_JOINT_MOTOR) {
                an[j] = make_float4(jd.linear_offset.x, jd.linear_offset.y, 0.0f, 0.0f);
                lim[j] = make_float4(jd.max_force, jd.max_torque, jd.correction_factor, jd.angular_offset);
                par[j] = make_float4(0.0f, __uint_as_float_host(fl), 0.0f, 0.0f);
            } else if (jd.type == B2G_JOINT_FRICTION) {
                lim[j] = make_float4(jd.max_force, jd.max_torque, 0.0f, 0.0f);
                par[j] = make_float4(0.0f, __uint_as_float_host(fl), 0.0f, 0.0f);
            } else if (jd.type == B2G_JOINT_WELD) {
                lim[j] = make_float4(jd.reference_angle, jd.stiffness, jd.damping, 0.0f);
                par[j] = make_float4(0.0f, __uint_as_float_host(fl), 0.0f, 0.0f);
            } else if (jd.type == B2G_JOINT_DISTANCE) {
                /* b2_distance_joint_new (private/dynamics/joints/b2_distance_joint.rs:42-76) */
                const float len = std::max(jd.length, kLinearSlop);
                const float lo = std::max(jd.min_length, kLinearSlop);
                const float hi = std::max(jd.max_length, lo);
                lim[j] = make_float4(len, lo, hi, jd.stiffness);
                par[j] = make_float4(jd.damping, __uint_as_float_host(fl), 0.0f, 0.0f);
            } else {
                lim[j] = make_float4(jd.reference_angle, jd.lower_angle, jd.upper_angle, jd.motor_speed);
                fl |= (jd.enable_limit ? JF_LIMIT : 0u) | (jd.enable_motor ? JF_MOTOR : 0u);
                par[j] = make_float4(jd.max_motor_torque, __uint_as_float_host(fl), 0.0f, 0.0f);
            }
        }
        U(d.j_body, jb.data(), nj);
        U(d.j_body2, jb2.data(), nj);
        U(d.j_x, jx.data(), nj);
        U(d.j_s, js.data(), nj);
        U(d.j_anchor, an.data(), nj);
        U(d.j_lim, lim.data(), nj);
        U(d.j_par, par.data(), nj);
        U(d.j_imp, w->h_jimp.data(), nj);
        U(d.j_imp2, w->h_jimp2.data(), nj);
        if (nlive > 0) U(d.j_order, w->h_jorder.data(), nlive);
        U(d.j_coff, w->h_jcoff.data(), kMaxJointColours + 1);
        U(d.b_jnt, w->h_jnt.data(), 2 * nj);
    }
#undef U
    CUDA_OK(w, cudaStreamSynchronize(s));
    d.n_joints = nj;
    if (d.n_jcolours != ncol) drop_graphs(w);  /* captured launches hold the colour count */
    d.n_jcolours = ncol;
    w->joints_dirty = false;
    return B2G_OK;
}

/* Makes the device hold every created body and fixture; grows capacities by rebuilding. */
int prepare(World* w) {
    const int nb = (int)w->h_flags.size();
    const int nf = (int)w->h_fbody.size();
    if (w->allocated && nb == w->uploaded_bodies && nf == w->uploaded_fixtures && !w->host_dirty) {
        if (!w->joints_dirty) return B2G_OK;
        /* only joints were added: the device's bodies and fixtures stay as they are */
        int rc = download_joint_impulses(w);
        if (rc != B2G_OK) return rc;
        return upload_joints(w);
    }
    {
        int rc = download_joint_impulses(w);
        if (rc != B2G_OK) return rc;
    }
    if (w->allocated && (nb > w->d.body_cap || nf > w->d.fix_cap)) {
        /* rebuild: keep the current contact table (its keys and impulses) across the reallocation */
        CUDA_OK(w, cudaStreamSynchronize(w->stream));
        int n_contacts = 0;
        CUDA_OK(w, cudaMemcpy(&n_contacts, w->d.cnt + CNT_CONTACTS, sizeof(int), cudaMemcpyDeviceToHost));
        Contacts old = w->d.c;
        const int old_cap = w->d.contact_cap;
        std::vector<unsigned long long> key(n_contacts);
        std::vector<int2> fix(n_contacts), body(n_contacts);
        std::vector<uint32_t> flags(n_contacts);
        std::vector<float4> mat(n_contacts), mgeo(n_contacts), mpts(n_contacts), mimp(n_contacts);
        std::vector<uint4> mids(n_contacts);
        if (n_contacts > 0) {
            cudaMemcpy(key.data(), old.key, n_contacts * sizeof(uint64_t), cudaMemcpyDeviceToHost);
            cudaMemcpy(fix.data(), old.fix, n_contacts * sizeof(int2), cudaMemcpyDeviceToHost);
            cudaMemcpy(body.data(), old.body, n_contacts * sizeof(int2), cudaMemcpyDeviceToHost);
            cudaMemcpy(flags.data(), old.flags, n_contacts * sizeof(uint32_t), cudaMemcpyDeviceToHost);
            cudaMemcpy(mat.data(), old.mat, n_contacts * sizeof(float4), cudaMemcpyDeviceToHost);
            cudaMemcpy(mgeo.data(), old.mgeo, n_contacts * sizeof(float4), cudaMemcpyDeviceToHost);
            cudaMemcpy(mpts.data(), old.mpts, n_contacts * sizeof(float4), cudaMemcpyDeviceToHost);
            cudaMemcpy(mimp.data(), old.mimp, n_contacts * sizeof(float4), cudaMemcpyDeviceToHost);
            CUDA_OK(w, cudaMemcpy(mids.data(), old.mids, n_contacts * sizeof(uint4), cudaMemcpyDeviceToHost));
        }
        (void)old_cap;
        const int old_key_bits = w->d.key_bits;
        free_all(w);
        int rc = allocate(w, nb, nf);
        if (rc != B2G_OK) return rc;
        /* keep the swap parity's relation to the table buffers (a saved state records it) */
        if (w->swaps & 1) std::swap(w->d.c, w->d.c_alt);
        if (n_contacts > 0) {
            Contacts& c = w->d.c;
            cudaMemcpyAsync(c.key, key.data(), n_contacts * sizeof(uint64_t), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.fix, fix.data(), n_contacts * sizeof(int2), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.body, body.data(), n_contacts * sizeof(int2), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.flags, flags.data(), n_contacts * sizeof(uint32_t), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.mat, mat.data(), n_contacts * sizeof(float4), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.mgeo, mgeo.data(), n_contacts * sizeof(float4), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.mpts, mpts.data(), n_contacts * sizeof(float4), cudaMemcpyHostToDevice, w->stream);
            cudaMemcpyAsync(c.mimp, mimp.data(), n_contacts * sizeof(float4), cudaMemcpyHostToDevice, w->stream);
            CUDA_OK(w, cudaMemcpyAsync(c.mids, mids.data(), n_contacts * sizeof(uint4), cudaMemcpyHostToDevice, w->stream));
            CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_CONTACTS, &n_contacts, sizeof(int), cudaMemcpyHostToDevice, w->stream));
            CUDA_OK(w, cudaStreamSynchronize(w->stream));
        }
        w->d.key_bits = old_key_bits;
    } else if (!w->allocated) {
        int rc = allocate(w, nb, nf);
        if (rc != B2G_OK) return rc;
    }
    /* contact keys are refid_min << key_bits | refid_max; widening key_bits keeps their order */
    const int kb = bits_for((uint64_t)std::max(1u, w->next_node));
    if (kb != w->d.key_bits) {
        if (w->d.key_bits != 0) {
            /* re-key the current table: decode with the old width, encode with the new one */
            int n_contacts = 0;
            CUDA_OK(w, cudaMemcpy(&n_contacts, w->d.cnt + CNT_CONTACTS, sizeof(int), cudaMemcpyDeviceToHost));
            if (n_contacts > 0) {
                std::vector<unsigned long long> key(n_contacts);
                CUDA_OK(w, cudaMemcpy(key.data(), w->d.c.key, n_contacts * sizeof(uint64_t), cudaMemcpyDeviceToHost));
                const uint64_t mask = (1ull << w->d.key_bits) - 1;
                for (unsigned long long& k : key) k = ((k >> w->d.key_bits) << kb) | (k & mask);
                CUDA_OK(w, cudaMemcpyAsync(w->d.c.key, key.data(), n_contacts * sizeof(uint64_t), cudaMemcpyHostToDevice, w->stream));
            }
        }
        w->d.key_bits = kb;
    }
    w->d.morton_world_bits = bits_for((uint64_t)(2 * w->num_worlds - 1));  /* key worlds: 2 per world */
    int rc = upload(w);
    if (rc != B2G_OK) return rc;
    return upload_joints(w);
}

/* Host copy of the first n entries of the current contact table (n = the device's contact count). A
 * contact destroyed between steps stays in the table, flagged CF_DEAD, until the next merge. */
struct HostContacts {
    int n = 0;
    std::vector<int2> fix, body;
    std::vector<uint32_t> flags;
    std::vector<float4> mat, mgeo, mpts, mimp;
    std::vector<uint4> mids;
};

int download_contacts(World* w, HostContacts& h, bool manifolds) {
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    CUDA_OK(w, cudaMemcpy(&h.n, w->d.cnt + CNT_CONTACTS, sizeof(int), cudaMemcpyDeviceToHost));
    const int n = h.n;
    const Contacts& c = w->d.c;
    h.flags.resize(n);
    h.fix.resize(n);
    h.body.resize(n);
    if (n == 0) return B2G_OK;
    CUDA_OK(w, cudaMemcpy(h.flags.data(), c.flags, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(h.fix.data(), c.fix, n * sizeof(int2), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(h.body.data(), c.body, n * sizeof(int2), cudaMemcpyDeviceToHost));
    if (!manifolds) return B2G_OK;
    h.mat.resize(n);
    h.mgeo.resize(n);
    h.mpts.resize(n);
    h.mimp.resize(n);
    h.mids.resize(n);
    CUDA_OK(w, cudaMemcpy(h.mat.data(), c.mat, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(h.mgeo.data(), c.mgeo, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(h.mpts.data(), c.mpts, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(h.mimp.data(), c.mimp, n * sizeof(float4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(h.mids.data(), c.mids, n * sizeof(uint4), cudaMemcpyDeviceToHost));
    return B2G_OK;
}

void contact_info(const HostContacts& h, int i, b2g_contact_info& o) {
    memset(&o, 0, sizeof(o));
    o.fixture_a = (uint32_t)h.fix[i].x;
    o.fixture_b = (uint32_t)h.fix[i].y;
    o.touching = (h.flags[i] & CF_TOUCHING) ? 1 : 0;
    o.manifold_type = (int)(h.mids[i].z & 0xffu);
    o.point_count = (int)((h.mids[i].z >> 8) & 0xffu);
    o.local_normal = b2g_vec2{h.mgeo[i].x, h.mgeo[i].y};
    o.local_point = b2g_vec2{h.mgeo[i].z, h.mgeo[i].w};
    o.point_local[0] = b2g_vec2{h.mpts[i].x, h.mpts[i].y};
    o.point_local[1] = b2g_vec2{h.mpts[i].z, h.mpts[i].w};
    o.normal_impulse[0] = h.mimp[i].x;
    o.tangent_impulse[0] = h.mimp[i].y;
    o.normal_impulse[1] = h.mimp[i].z;
    o.tangent_impulse[1] = h.mimp[i].w;
    o.point_id[0] = h.mids[i].x;
    o.point_id[1] = h.mids[i].y;
    o.friction = h.mat[i].x;
    o.restitution = h.mat[i].y;
    o.restitution_threshold = h.mat[i].z;
}

/* readers of a stepped world after a host-side edit: the edited mirrors go to the device first */
int sync_host_edits(World* w) {
    if (w->device_authoritative && w->host_dirty) return prepare(w);
    return B2G_OK;
}

int status_error(World* w, int status);

int check_status(World* w) {
    if (!w->allocated) return B2G_OK;
    int status = 0;
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    CUDA_OK(w, cudaMemcpy(&status, w->d.cnt + CNT_STATUS, sizeof(int), cudaMemcpyDeviceToHost));
    return status_error(w, status);
}

/* the error for a device status word read after the stream drained (0: none); clears it */
int status_error(World* w, int status) {
    if (status == 0) return B2G_OK;
    const int zero = 0;
    cudaMemcpyAsync(w->d.cnt + CNT_STATUS, &zero, sizeof(int), cudaMemcpyHostToDevice, w->stream);
    if (status & ST_BARRIER_TIMEOUT) {
        /* the barrier counters may be left mid-count: reset them */
        const int z2[2] = {0, 0};
        cudaMemcpyAsync(w->d.cnt + CNT_BARRIER, z2, sizeof(z2), cudaMemcpyHostToDevice, w->stream);
        return fail(w, B2G_ERR_TIMEOUT, "a grid barrier wait timed out; the step's results are void");
    }
    if (status & (ST_CONTACT_OVERFLOW | ST_PAIR_OVERFLOW | ST_STACK_OVERFLOW | ST_COLOUR_OVERFLOW)) {
        std::string what;
        if (status & ST_CONTACT_OVERFLOW) what += " contacts";
        if (status & ST_PAIR_OVERFLOW) what += " new-pairs";
        if (status & ST_STACK_OVERFLOW) what += " traversal-stack";
        if (status & ST_COLOUR_OVERFLOW) what += " colours";
        return fail(w, B2G_ERR_CAPACITY,
                    "a device capacity overflowed (" + what.substr(1) +
                        "); raise contact_capacity / pair_capacity in b2g_world_def");
    }
    if (status & ST_EVENT_OVERFLOW) return fail(w, B2G_ERR_CAPACITY, "contact event buffer overflowed");
    if (status & ST_RECORD_OVERFLOW) return fail(w, B2G_ERR_CAPACITY, "recorded pair buffer overflowed");
    if (status & ST_TOI_OVERFLOW)
        return fail(w, B2G_ERR_CAPACITY,
                    "a list of the continuous pass overflowed (time-of-impact island of more than 64 bodies or 64 "
                    "partner contacts, or more than 4096 new contacts or moved proxies in one step)");
    if (status & ST_PART_MISMATCH)
        return fail(w, B2G_ERR_CUDA, "the solver ran with a block count other than its colouring's");
    return B2G_OK;
}

void swap_contacts(World* w) {
    std::swap(w->d.c, w->d.c_alt);
    ++w->swaps;
}

StepParams make_params(World* w, float dt, int vi, int pi) {
    StepParams sp{};
    sp.dt = dt;
    sp.inv_dt = dt > 0.0f ? 1.0f / dt : 0.0f;
    sp.dt_ratio = w->inv_dt0 * dt;
    sp.gx = w->gravity.x;
    sp.gy = w->gravity.y;
    sp.vi = vi;
    sp.pi = pi;
    sp.warm = w->warm ? 1 : 0;
    sp.allow_sleep = w->allow_sleep ? 1 : 0;
    sp.auto_clear = w->auto_clear ? 1 : 0;
    sp.record_events = w->record_events ? 1 : 0;
    sp.record_pairs = w->record_pairs ? 1 : 0;
    sp.toi_schedule = w->toi_schedule;
    sp.toi_may_conflict = w->kinematic_or_bullet ? 1 : 0;
    sp.custom_filter = w->filter_fn ? 1 : 0;
    sp.pre_solve = w->pre_solve_fn ? 1 : 0;
    return sp;
}

/* ---- host callbacks inside a step ----
 * The reference calls its contact filter from add_pair and from collide (for a flagged contact), and
 * pre_solve from each contact's update. Here a world with such a callback runs its steps without
 * graphs and stops at three points to run them on the host: before collide (the flagged contacts,
 * whose answer goes to the device as CF_REJECT; the manifolds are also copied for pre_solve's old
 * manifold), after collide (pre_solve of every updated, touching contact, in table order; its edits go
 * back to the device before the solver), and after the broadphase's traversal (the new pairs, before
 * they are sorted and merged). Each stop synchronises the world's stream: a slow path. */

/* self.should_collide(other) on the host mirrors (B2body::should_collide, private/dynamics/b2_body.rs:391-416) */
bool host_should_collide(const World* w, int self, int other) {
    if ((w->h_flags[self] & BF_TYPE_MASK) != BODY_DYNAMIC && (w->h_flags[other] & BF_TYPE_MASK) != BODY_DYNAMIC)
        return false;
    for (size_t j = 0; j < w->joints.size(); ++j) {
        if (w->h_jdead[j] || w->joints[j].collide_connected) continue;
        const int a = (int)w->joints[j].body_a, b = (int)w->joints[j].body_b;
        if ((a == self && b == other) || (a == other && b == self)) return false;
    }
    return true;
}

int hook_before_collide(World* w, HostContacts& old) {
    int rc = download_contacts(w, old, w->pre_solve_fn != nullptr);
    if (rc != B2G_OK || !w->filter_fn) return rc;
    bool changed = false;
    for (int i = 0; i < old.n; ++i) {
        const uint32_t f = old.flags[i];
        if (!(f & CF_FILTER) || (f & CF_DEAD)) continue;
        if (!host_should_collide(w, old.body[i].y, old.body[i].x)) continue;  /* collide destroys it anyway */
        const bool keep = w->filter_fn(w->filter_user, (uint32_t)old.fix[i].x, (uint32_t)old.fix[i].y) != 0;
        const uint32_t nf = keep ? (f & ~CF_REJECT) : (f | CF_REJECT);
        if (nf != f) {
            old.flags[i] = nf;
            changed = true;
        }
    }
    if (changed && old.n > 0)
        CUDA_OK(w, cudaMemcpyAsync(w->d.c.flags, old.flags.data(), old.n * sizeof(uint32_t), cudaMemcpyHostToDevice, w->stream));
    return B2G_OK;
}

int hook_pre_solve(World* w, const HostContacts& old) {
    HostContacts now;
    int rc = download_contacts(w, now, true);
    if (rc != B2G_OK) return rc;
    bool changed = false;
    for (int i = 0; i < now.n; ++i) {
        const uint32_t f = now.flags[i];
        if (!(f & CF_UPDATED) || !(f & CF_TOUCHING) || (f & CF_DEAD)) continue;
        b2g_contact_info info, prev;
        contact_info(now, i, info);
        if (i < old.n) contact_info(old, i, prev);
        else memset(&prev, 0, sizeof(prev));
        b2g_contact_edit e;
        e.enabled = (f & CF_ENABLED) ? 1 : 0;
        e.friction = now.mat[i].x;
        e.restitution = now.mat[i].y;
        e.restitution_threshold = now.mat[i].z;
        e.tangent_speed = now.mat[i].w;
        w->pre_solve_fn(w->pre_solve_user, &info, &prev, &e);
        const uint32_t nf = e.enabled ? (f | CF_ENABLED) : (f & ~CF_ENABLED);
        const float4 nm = make_float4(e.friction, e.restitution, e.restitution_threshold, e.tangent_speed);
        if (nf != f || memcmp(&nm, &now.mat[i], sizeof(nm)) != 0) {
            now.flags[i] = nf;
            now.mat[i] = nm;
            changed = true;
        }
    }
    if (changed) {
        CUDA_OK(w, cudaMemcpyAsync(w->d.c.flags, now.flags.data(), now.n * sizeof(uint32_t), cudaMemcpyHostToDevice, w->stream));
        CUDA_OK(w, cudaMemcpyAsync(w->d.c.mat, now.mat.data(), now.n * sizeof(float4), cudaMemcpyHostToDevice, w->stream));
    }
    return B2G_OK;
}

/* add_pair's call of the contact filter for the broadphase's new pairs (the fixtures of the smaller and
 * the larger proxy id, as the pair was found); the pairs it rejects are removed before the merge */
int hook_new_pairs(World* w) {
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    int n = 0;
    CUDA_OK(w, cudaMemcpy(&n, w->d.cnt + CNT_NEW, sizeof(int), cudaMemcpyDeviceToHost));
    n = std::min(n, w->d.pair_cap);
    if (n <= 0) return B2G_OK;
    std::vector<unsigned long long> key(n);
    std::vector<int2> fix(n);
    CUDA_OK(w, cudaMemcpy(key.data(), w->d.n_key, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(fix.data(), w->d.n_fix, n * sizeof(int2), cudaMemcpyDeviceToHost));
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const int fa = fix[i].x, fb = fix[i].y;
        const bool a_first = w->h_refid[fa] < w->h_refid[fb];
        const bool keep = w->filter_fn(w->filter_user, (uint32_t)(a_first ? fa : fb), (uint32_t)(a_first ? fb : fa)) != 0;
        if (!keep) continue;
        key[m] = key[i];
        fix[m] = fix[i];
        ++m;
    }
    if (m == n) return B2G_OK;
    std::vector<uint32_t> idx(std::max(m, 1));
    for (int i = 0; i < m; ++i) idx[i] = (uint32_t)i;
    if (m > 0) {
        CUDA_OK(w, cudaMemcpyAsync(w->d.n_key, key.data(), m * sizeof(unsigned long long), cudaMemcpyHostToDevice, w->stream));
        CUDA_OK(w, cudaMemcpyAsync(w->d.n_fix, fix.data(), m * sizeof(int2), cudaMemcpyHostToDevice, w->stream));
        CUDA_OK(w, cudaMemcpyAsync(w->d.n_idx, idx.data(), m * sizeof(uint32_t), cudaMemcpyHostToDevice, w->stream));
    }
    CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_NEW, &m, sizeof(int), cudaMemcpyHostToDevice, w->stream));
    return B2G_OK;
}

/* The launch sequence of one step on the world's stream (captured into a graph or run directly).
 * Under capture the profile events become external event-record nodes, so the host can still
 * time the graph's phases with cudaEventElapsedTime. */
void issue_step(World* w, const StepParams& sp, float dt, bool capturing = false) {
    cudaStream_t s = w->stream;
    Timer& t = w->timer;
    auto mark = [&](cudaEvent_t e) {
        if (capturing) cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
        else cudaEventRecord(e, s);
    };
    /* host callbacks (never under capture): the first failure is kept and the rest of the step skipped */
    auto hook = [&](int rc) {
        if (rc != B2G_OK && w->hook_rc == B2G_OK) w->hook_rc = rc;
    };
    auto pair_hook = [&](int k) {
        if (k == 2 && w->filter_fn && w->hook_rc == B2G_OK) hook(hook_new_pairs(w));
    };
    cudaMemsetAsync(w->d.cnt + CNT_EVENTS, 0, sizeof(int), s);
    mark(t.e[0]);
    if (w->new_contacts) {
        launch_broadphase(w->d, sp, s, w->num_sms, pair_hook);
        swap_contacts(w);
        w->new_contacts = false;
    }
    mark(t.e[1]);
    HostContacts before;
    if ((w->filter_fn || w->pre_solve_fn) && w->hook_rc == B2G_OK) hook(hook_before_collide(w, before));
    launch_collide(w->d, sp, s, w->allow_sleep || w->asleep_seen, w->num_sms);
    if (w->pre_solve_fn && w->hook_rc == B2G_OK) hook(hook_pre_solve(w, before));
    mark(t.e[2]);
    if (dt > 0.0f) {
        launch_islands_and_constraints(w->d, sp, s);
        mark(t.e[6]);
        const bool taping = w->tape && w->tape->recording;
        launch_colouring(w->d, s, w->num_sms, w->part_solve);
        if (taping) launch_tape_record(w->d, w->tape->d, sp, s, w->num_sms);
        mark(t.e[3]);
        launch_solver(w->d, sp, s, w->num_sms, w->part_solve);
        if (taping) launch_tape_post(w->d, w->tape->d, sp, s, w->num_sms);
        mark(t.e[4]);
        launch_broadphase(w->d, sp, s, w->num_sms, [&](int k) {
            mark(t.e[k == 0 ? 9 : k == 1 ? 10 : 7]);
            pair_hook(k);
        });
        swap_contacts(w);
        mark(t.e[8]);
        /* B2world::solve_toi (private/dynamics/b2_world.rs:946-950); the pass moves hierarchy leaves
         * in place without the four-way records, so the next broadphase pass rebuilds */
        if (w->continuous) {
            launch_continuous(w->d, sp, s, w->num_sms);
            cudaMemsetAsync(w->d.cnt + CNT_BP_FORCE, 1, sizeof(int), s);
        }
        mark(t.e[5]);
        w->inv_dt0 = sp.inv_dt;
    } else {
        mark(t.e[6]);
        mark(t.e[3]);
        mark(t.e[4]);
        mark(t.e[9]);
        mark(t.e[10]);
        mark(t.e[7]);
        if (w->auto_clear) launch_clear_forces(w->d, s);
        mark(t.e[8]);
        mark(t.e[5]);
    }
}

/* More position iterations than separation buffers: replace that one allocation. */
int ensure_minsep_buffers(World* w, int pi) {
    if (pi <= w->minsep_buffers) return B2G_OK;
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    auto it = std::find(w->allocations.begin(), w->allocations.end(), (void*)w->d.isl_minsep);
    if (it != w->allocations.end()) drop_allocation(w, (size_t)(it - w->allocations.begin()));
    cudaFree(w->d.isl_minsep);
    w->minsep_buffers = pi;
    int rc = dalloc(w, &w->d.isl_minsep, (size_t)pi * w->d.body_cap);
    if (rc != B2G_OK) return rc;
    drop_graphs(w);
    ++w->alloc_generation;
    return B2G_OK;
}

/* With auto-grow on: after a broadphase pass whose new pairs or merged contacts overflowed (the world's
 * stream drained), the table it started from is made current again, the capacities grow (doubled, as
 * often as needed) and the pass runs again with every proxy queried. The pass is the last thing that
 * touched the contact table, and querying every proxy instead of the moved ones finds the same new
 * contacts (a pair of unmoved overlapping proxies already has its contact or was rejected by add_pair's
 * rules, which reject it again), so the world continues exactly as one that had the capacity from the
 * start. Other device errors are reported as usual. */
int recover_overflow(World* w, const StepParams& sp) {
    const int growable = ST_CONTACT_OVERFLOW | ST_PAIR_OVERFLOW | ST_RECORD_OVERFLOW;
    for (int attempt = 0; attempt < 16; ++attempt) {
        CUDA_OK(w, cudaStreamSynchronize(w->stream));
        int cnt[CNT_SIZE];
        CUDA_OK(w, cudaMemcpy(cnt, w->d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
        const int status = cnt[CNT_STATUS];
        if (!(status & growable) || (status & ~growable)) return status_error(w, status);
        const int zero = 0, from = cnt[CNT_MERGE_FROM];
        CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_STATUS, &zero, sizeof(int), cudaMemcpyHostToDevice, w->stream));
        swap_contacts(w);
        CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_CONTACTS, &from, sizeof(int), cudaMemcpyHostToDevice, w->stream));
        const int cc = (status & ST_CONTACT_OVERFLOW) ? 2 * w->d.contact_cap : w->d.contact_cap;
        const int pc = (status & (ST_PAIR_OVERFLOW | ST_RECORD_OVERFLOW)) ? 2 * w->d.pair_cap : w->d.pair_cap;
        int rc = grow_capacities(w, cc, pc);
        if (rc != B2G_OK) return rc;
        launch_touch_all_proxies(w->d, w->stream);
        launch_broadphase(w->d, sp, w->stream, w->num_sms, nullptr, BP_REPEAT);
        swap_contacts(w);
        CUDA_OK(w, cudaGetLastError());
    }
    return fail(w, B2G_ERR_CAPACITY, "capacities still overflow after repeated growth");
}

/* B2world::step, src/private/dynamics/b2_world.rs:903-959 */
int step(World* w, float dt, int vi, int pi) {
    if (w->h_flags.empty()) return B2G_OK;
    if (vi < 0 || pi < 0 || !(dt >= 0.0f)) return fail(w, B2G_ERR_INVALID_ARG, "dt must be >= 0 and iterations >= 0");
    int rc = prepare(w);
    if (rc != B2G_OK) return rc;
    rc = ensure_minsep_buffers(w, pi);
    if (rc != B2G_OK) return rc;
    if (w->joint_filter_pending) {
        /* B2world::create_joint flags the contacts of the joined bodies (b2_world.rs:258-271) */
        launch_flag_joint_contacts(w->d, w->stream, w->num_sms);
        w->joint_filter_pending = false;
    }
    w->device_authoritative = true;
    if (w->tape && w->tape->recording) {
        if (dt > 0.0f) ++w->tape->steps;
        else w->tape->valid = false;  /* a collide-only step re-matches impulses outside the tape */
    }
    StepParams sp = make_params(w, dt, vi, pi);
    cudaStream_t s = w->stream;
    Timer& t = w->timer;
    if (!t.valid) {
        for (auto& e : t.e) cudaEventCreate(&e);
        t.valid = true;
    }
    const bool grow = w->auto_grow && !(w->tape && w->tape->recording) && !w->filter_fn;
    if (grow && w->new_contacts) {
        /* the initial pass of new fixtures on its own, checked before the step collides its contacts */
        launch_broadphase(w->d, sp, s, w->num_sms);
        swap_contacts(w);
        w->new_contacts = false;
        rc = recover_overflow(w, sp);
        if (rc != B2G_OK) return rc;
    }
    /* Steady state (no fixtures added since the last step, dt > 0, warm-start ratio already
     * set): the step's launch sequence depends only on the parameters, the allocation and the
     * contact-buffer parity, so it runs as one of two captured CUDA graphs. */
    const bool graphable = w->use_graphs && !w->new_contacts && dt > 0.0f && w->steps > 0 && !w->filter_fn &&
                           !w->pre_solve_fn;
    if (graphable) {
        GraphKey key{};
        key.dt = dt;
        key.dt_ratio = sp.dt_ratio;
        key.gx = sp.gx;
        key.gy = sp.gy;
        key.vi = vi;
        key.pi = pi;
        key.flags = sp.warm | (sp.allow_sleep << 1) | (sp.auto_clear << 2) | (sp.record_events << 3) |
                    (sp.record_pairs << 4) | ((w->tape && w->tape->recording) ? (1 << 5) : 0) |
                    (w->continuous ? (1 << 6) : 0) | (sp.toi_schedule << 7) | (w->asleep_seen ? (1 << 9) : 0) |
                    (sp.toi_may_conflict << 10);
        key.generation = w->alloc_generation;
        key.n_bodies = w->d.n_bodies;
        key.n_fixtures = w->d.n_fixtures;
        const int parity = w->swaps & 1;
        GraphSlot& g = w->graphs[parity];
        if (!g.exec || memcmp(&g.key, &key, sizeof(key)) != 0) {
            if (g.exec) {
                cudaGraphExecDestroy(g.exec);
                g.exec = nullptr;
            }
            DevWorld saved = w->d;
            const int saved_swaps = w->swaps;
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                const unsigned long long before = g_kernel_launches;
                issue_step(w, sp, dt, true);
                g.kernels = g_kernel_launches - before;  /* counted per replay instead */
                g_kernel_launches = before;
                e = cudaStreamEndCapture(s, &graph);
            }
            w->d = saved;  /* the capture recorded the launches; the real swap happens below */
            w->swaps = saved_swaps;
            if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                /* capture unsupported here: fall back to direct launches for this world */
                cudaGetLastError();
                g.exec = nullptr;
                w->use_graphs = false;
                issue_step(w, sp, dt);
                CUDA_OK(w, cudaGetLastError());
                ++w->steps;
                return B2G_OK;
            }
            g.key = key;
        }
        CUDA_OK(w, cudaGraphLaunch(g.exec, s));
        B2G_LAUNCHED(g.kernels);
        swap_contacts(w);
        w->inv_dt0 = sp.inv_dt;
    } else {
        w->hook_rc = B2G_OK;
        issue_step(w, sp, dt);
        if (w->hook_rc != B2G_OK) {
            ++w->steps;
            return w->hook_rc;
        }
    }
    CUDA_OK(w, cudaGetLastError());
    ++w->steps;
    if (grow && dt > 0.0f) return recover_overflow(w, sp);
    return B2G_OK;
}

World* W(void* p) { return (World*)p; }

/* b2g_body_state of bodies [first, first + count); thread 0 also copies the status word to
 * *status (host memory the device writes coherently) so the caller needs no second copy */
__global__ void k_pack_states(DevWorld d, uint32_t first, uint32_t count, b2g_body_state* out, int* status) {
    if (status && blockIdx.x == 0 && threadIdx.x == 0) *status = ((volatile int*)d.cnt)[CNT_STATUS];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float4 xf = d.b_xf[first + i], pos = d.b_pos[first + i], vel = d.b_vel[first + i];
        b2g_body_state s;
        s.position = b2g_vec2{xf.x, xf.y};
        s.angle = pos.z;
        s.linear_velocity = b2g_vec2{vel.x, vel.y};
        s.angular_velocity = vel.z;
        s.world_center = b2g_vec2{pos.x, pos.y};
        out[i] = s;
    }
}

/* the snapshot of b2g_get_body_states_async into the caller's buffer (host memory the device
 * reaches coherently), 16 bytes per thread */
__global__ void k_copy_states(const float4* __restrict__ in, float4* out, size_t n4) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

/* small body edits after the device became authoritative */
/* One edit of one body (src/b2_body.rs): 0 set_linear_velocity (:684-694), 1 set_angular_velocity
 * (:696-705), 2 apply_force, 3 apply_linear_impulse, 4 apply_force_to_center, 5 apply_torque,
 * 6 apply_linear_impulse_to_center, 7 apply_angular_impulse (:870-980), 8 set_awake (:783-801).
 * v.w holds the sleep time; f.z the torque. Shared by the device kernel and the host mirrors. */
B2G_HD void edit_body(int op, uint32_t& fl, float4& v, float4& f, const float4& p, const float4& m, float x, float y,
                      float z, float px, float py, int wake) {
    const int type = (int)(fl & BF_TYPE_MASK);
    if (op == 0 || op == 1) {
        if (type == BODY_STATIC) return;
        const bool nonzero = op == 0 ? x * x + y * y > 0.0f : z * z > 0.0f;
        if (nonzero && !(fl & BF_AWAKE)) {
            fl |= BF_AWAKE;
            v.w = 0.0f;
        }
        if (op == 0) {
            v.x = x;
            v.y = y;
        } else {
            v.z = z;
        }
        return;
    }
    if (op == 8) {
        if (type == BODY_STATIC) return;
        if (wake) {
            fl |= BF_AWAKE;
            v.w = 0.0f;
        } else {
            fl &= ~BF_AWAKE;
            v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            f = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        return;
    }
    if (type != BODY_DYNAMIC) return;
    if (wake && !(fl & BF_AWAKE)) {
        fl |= BF_AWAKE;
        v.w = 0.0f;
    }
    if (!(fl & BF_AWAKE)) return;  /* a sleeping body accumulates nothing */
    const float cr = (px - p.x) * y - (py - p.y) * x;  /* b2_cross(point - c, vector) */
    switch (op) {
        case 2: f.x += x; f.y += y; f.z += cr; break;
        case 3: v.x += m.y * x; v.y += m.y * y; v.z += m.w * cr; break;
        case 4: f.x += x; f.y += y; break;
        case 5: f.z += z; break;
        case 6: v.x += m.y * x; v.y += m.y * y; break;
        case 7: v.z += m.w * z; break;
        default: break;
    }
}

__global__ void k_body_op(DevWorld d, int op, int b, float x, float y, float z, float px, float py, int wake) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t fl = d.b_flags[b];
    float4 v = d.b_vel[b], f = d.b_force[b];
    edit_body(op, fl, v, f, d.b_pos[b], d.b_mass[b], x, y, z, px, py, wake);
    d.b_flags[b] = fl;
    d.b_vel[b] = v;
    d.b_force[b] = f;
}

int body_op(World* w, int op, uint32_t b, float x, float y, float z, float px, float py, int wake) {
    if (b >= w->h_flags.size() || w->h_bdead[b]) return fail(w, B2G_ERR_INVALID_ARG, "body id out of range or destroyed");
    tape_touch(w);
    if (w->device_authoritative) {
        int rc = prepare(w);
        if (rc != B2G_OK) return rc;
        k_body_op<<<1, 32, 0, w->stream>>>(w->d, op, (int)b, x, y, z, px, py, wake); B2G_LAUNCHED(1);
        CUDA_OK(w, cudaGetLastError());
        return B2G_OK;
    }
    edit_body(op, w->h_flags[b], w->h_vel[b], w->h_force[b], w->h_pos[b], w->h_mass[b], x, y, z, px, py, wake);
    return B2G_OK;
}

}  // namespace

extern "C" {

int b2g_version(void) { return kVersion; }

int64_t b2g_get_launch_count(void) { return (int64_t)g_kernel_launches; }

int b2g_world_create(const b2g_world_def* def, void** out) {
    if (!def || !out) return B2G_ERR_INVALID_ARG;
    if (def->num_worlds < 1) return B2G_ERR_INVALID_ARG;
    World* w = new World();
    w->device = def->device;
    w->gravity = def->gravity;
    w->num_worlds = def->num_worlds;
    w->user_contact_cap = def->contact_capacity;
    w->user_pair_cap = def->pair_capacity;
    if (cudaSetDevice(w->device) != cudaSuccess) {
        delete w;
        return B2G_ERR_CUDA;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, w->device) != cudaSuccess || cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete w;
        return B2G_ERR_CUDA;
    }
    w->num_sms = prop.multiProcessorCount;
    w->d.num_sms = w->num_sms;
    w->pageable = prop.pageableMemoryAccess != 0;
    if (!prop.cooperativeLaunch) {
        cudaStreamDestroy(w->stream);
        delete w;
        return B2G_ERR_UNSUPPORTED;
    }
    *out = w;
    return B2G_OK;
}

int b2g_world_destroy(void* p) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    cudaStreamSynchronize(w->stream);
    if (w->copy_stream) {
        cudaStreamSynchronize(w->copy_stream);
        for (int i = 0; i < 2; ++i) {
            if (w->d_ring[i]) cudaFree(w->d_ring[i]);
            cudaEventDestroy(w->ev_packed[i]);
            cudaEventDestroy(w->ev_copied[i]);
        }
        cudaStreamDestroy(w->copy_stream);
    }
    tape_free(w);
    if (w->d_states) cudaFree(w->d_states);
    free_all(w);
    if (w->timer.valid)
        for (auto& e : w->timer.e) cudaEventDestroy(e);
    cudaStreamDestroy(w->stream);
    delete w;
    return B2G_OK;
}

const char* b2g_last_error(const void* p) { return p ? W((void*)p)->err.c_str() : "null world"; }

/* B2world::create_body -> b2_body (private/dynamics/b2_body.rs:15-78) */
int b2g_create_bodies(void* p, const b2g_body_def* defs, int32_t n, uint32_t* ids) {
    World* w = W(p);
    if (!w || (!defs && n > 0) || n < 0) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const b2g_body_def& d = defs[i];
        if (d.type < 0 || d.type > 2) return fail(w, B2G_ERR_INVALID_ARG, "body type must be 0, 1 or 2");
        if ((int)d.world_index >= w->num_worlds) return fail(w, B2G_ERR_INVALID_ARG, "world_index >= num_worlds");
        if (!(d.linear_damping >= 0.0f) || !(d.angular_damping >= 0.0f))
            return fail(w, B2G_ERR_INVALID_ARG, "damping must be >= 0");
    }
    if (n > 0) tape_touch(w);
    if (w->device_authoritative) {
        int rc = download_state(w);
        if (rc != B2G_OK) return rc;
    }
    for (int i = 0; i < n; ++i) {
        const b2g_body_def& d = defs[i];
        uint32_t fl = (uint32_t)d.type;
        if (d.awake && d.type != B2G_STATIC_BODY) fl |= BF_AWAKE;
        if (!d.awake && d.type != B2G_STATIC_BODY) w->asleep_seen = true;
        if (d.enabled) fl |= BF_ENABLED;
        if (d.allow_sleep) fl |= BF_AUTO_SLEEP;
        if (d.fixed_rotation) fl |= BF_FIXED_ROTATION;
        if (d.bullet) fl |= BF_BULLET;
        if (d.type == B2G_KINEMATIC_BODY || (d.type == B2G_DYNAMIC_BODY && d.bullet)) w->kinematic_or_bullet = true;
        const Rot q = rot(d.angle);
        const int id = (int)w->h_flags.size();
        w->h_flags.push_back(fl);
        w->h_world.push_back(d.world_index);
        w->h_xf.push_back(make_float4(d.position.x, d.position.y, q.s, q.c));
        w->h_pos.push_back(make_float4(d.position.x, d.position.y, d.angle, 0.0f));
        w->h_pos0.push_back(make_float4(d.position.x, d.position.y, d.angle, 0.0f));
        w->h_vel.push_back(make_float4(d.linear_velocity.x, d.linear_velocity.y, d.angular_velocity, 0.0f));
        w->h_force.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        w->h_mass.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        w->h_damp.push_back(make_float4(d.linear_damping, d.angular_damping, d.gravity_scale, 0.0f));
        w->h_lc.push_back(make_float2(0.0f, 0.0f));
        w->body_fixtures.emplace_back();
        w->h_bdead.push_back(0);
        if (ids) ids[i] = (uint32_t)id;
    }
    return B2G_OK;
}

/* B2body::create_fixture (private/dynamics/b2_body.rs:155-200) + create_proxies (b2_fixture.rs:114-133) */
int b2g_create_fixtures(void* p, const b2g_fixture_def* defs, int32_t n, uint32_t* ids) {
    World* w = W(p);
    if (!w || (!defs && n > 0) || n < 0) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const b2g_fixture_def& d = defs[i];
        if (d.body >= w->h_flags.size()) return fail(w, B2G_ERR_INVALID_ARG, "fixture body id out of range");
        if (w->h_bdead[d.body]) return fail(w, B2G_ERR_INVALID_ARG, "fixture body was destroyed");
        if (d.shape_type < 0 || d.shape_type > 2)
            return fail(w, B2G_ERR_UNSUPPORTED, "shape type must be circle, edge or polygon (chain shapes are not supported)");
        if (!(d.density >= 0.0f) || !(d.friction >= 0.0f) || !(d.restitution >= 0.0f))
            return fail(w, B2G_ERR_INVALID_ARG, "density, friction and restitution must be >= 0");
    }
    if (n > 0) tape_touch(w);
    if (w->device_authoritative) {
        int rc = download_state(w);
        if (rc != B2G_OK) return rc;
    }
    for (int i = 0; i < n; ++i) {
        const b2g_fixture_def& d = defs[i];
        const int b = (int)d.body;
        const int f = (int)w->h_fbody.size();
        ShapeRec s;
        build_shape(d, s);
        w->h_shape.push_back(s);
        w->h_fbody.push_back(b);
        w->h_fmat.push_back(make_float4(d.friction, d.restitution, d.restitution_threshold, d.density));
        w->h_filter.push_back((uint32_t)d.category_bits | ((uint32_t)d.mask_bits << 16));
        w->h_group.push_back((uint32_t)(uint16_t)d.group_index | (d.is_sensor ? 0x10000u : 0u));
        if (w->h_flags[b] & BF_ENABLED) {
            AABB a;
            shape_aabb(s, host_xf(w, b), a);
            const V2 r = mk(kAabbExtension, kAabbExtension);
            const V2 lo = sub(a.lo, r), hi = add(a.hi, r);
            w->h_fat.push_back(make_float4(lo.x, lo.y, hi.x, hi.y));
            w->h_moved.push_back(1);
            w->h_refid.push_back(alloc_refid(w));
        } else {
            const float inf = INFINITY;
            w->h_fat.push_back(make_float4(inf, inf, -inf, -inf));
            w->h_moved.push_back(0);
            w->h_refid.push_back(0xffffffffu);
        }
        w->body_fixtures[b].insert(w->body_fixtures[b].begin(), f);
        w->h_fdead.push_back(0);
        if (d.density > 0.0f) reset_mass_data(w, b);
        w->new_contacts = true;
        if (ids) ids[i] = (uint32_t)f;
    }
    return B2G_OK;
}

}  // extern "C"

namespace {

/* one side of B2gearJoint::new (b2_gear_joint.rs:62-82 / :91-111): the joint's local anchors, axis,
 * reference angle and the side's coordinate on the bodies' current transforms */
void gear_side(World* w, const b2g_joint_def& jd, V2& anchor_first, V2& anchor_second, V2& axis, float& ref,
               bool& prismatic, float& coordinate) {
    const int first = (int)jd.body_a, second = (int)jd.body_b;
    anchor_first = mk(jd.local_anchor_a.x, jd.local_anchor_a.y);
    anchor_second = mk(jd.local_anchor_b.x, jd.local_anchor_b.y);
    ref = jd.reference_angle;
    prismatic = jd.type == B2G_JOINT_PRISMATIC;
    const Xf xf_second = host_xf(w, second), xf_first = host_xf(w, first);
    if (!prismatic) {
        axis = mk(0.0f, 0.0f);
        coordinate = w->h_pos[second].z - w->h_pos[first].z - ref;
        return;
    }
    /* the prismatic joint's unit axis (B2prismaticJoint::new, b2_prismatic_joint.rs:54-60) */
    axis = mk(jd.local_axis_a.x, jd.local_axis_a.y);
    normalize(axis);
    const V2 p_second = mul_t(xf_first.q, add(mul(xf_second.q, anchor_second), sub(xf_second.p, xf_first.p)));
    coordinate = dot(sub(p_second, anchor_first), axis);
}

GearFrame gear_frame(World* w, const b2g_joint_def& d) {
    GearFrame g;
    const b2g_joint_def& j1 = w->joints[d.joint1];
    const b2g_joint_def& j2 = w->joints[d.joint2];
    float coordinate_a = 0.0f, coordinate_b = 0.0f;
    g.body_c = (int)j1.body_a;
    g.body_d = (int)j2.body_a;
    gear_side(w, j1, g.anchor_c, g.anchor_a, g.axis_c, g.ref_a, g.prismatic_a, coordinate_a);
    gear_side(w, j2, g.anchor_d, g.anchor_b, g.axis_d, g.ref_b, g.prismatic_b, coordinate_b);
    g.constant = coordinate_a + d.ratio * coordinate_b;
    return g;
}

}  // namespace

extern "C" {

int b2g_create_joints(void* p, const b2g_joint_def* defs, int32_t n, uint32_t* ids) {
    World* w = W(p);
    if (!w || (!defs && n > 0) || n < 0) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i) {
        const b2g_joint_def& d = defs[i];
        if (d.type != B2G_JOINT_REVOLUTE && d.type != B2G_JOINT_DISTANCE && d.type != B2G_JOINT_WELD &&
            d.type != B2G_JOINT_FRICTION && d.type != B2G_JOINT_MOTOR && d.type != B2G_JOINT_MOUSE &&
            d.type != B2G_JOINT_PRISMATIC && d.type != B2G_JOINT_WHEEL && d.type != B2G_JOINT_PULLEY &&
            d.type != B2G_JOINT_GEAR)
            return fail(w, B2G_ERR_UNSUPPORTED, "unknown joint type");
        if (d.body_a >= w->h_flags.size() || d.body_b >= w->h_flags.size() || d.body_a == d.body_b)
            return fail(w, B2G_ERR_INVALID_ARG, "joint body ids out of range or equal");
        if (w->h_bdead[d.body_a] || w->h_bdead[d.body_b]) return fail(w, B2G_ERR_INVALID_ARG, "a joint body was destroyed");
        if (d.type == B2G_JOINT_GEAR) {
            /* B2gearJoint::new asserts (b2_gear_joint.rs:29-60, 83-87): two revolute or prismatic joints made
             * earlier; the gear's bodies are their second bodies, which must be dynamic */
            const size_t made = w->joints.size() + (size_t)i;
            if (d.joint1 >= made || d.joint2 >= made || (d.joint1 < w->joints.size() && w->h_jdead[d.joint1]) ||
                (d.joint2 < w->joints.size() && w->h_jdead[d.joint2]))
                return fail(w, B2G_ERR_INVALID_ARG, "a gear joint's joints must exist before it");
            const b2g_joint_def& j1 = d.joint1 < w->joints.size() ? w->joints[d.joint1] : defs[d.joint1 - w->joints.size()];
            const b2g_joint_def& j2 = d.joint2 < w->joints.size() ? w->joints[d.joint2] : defs[d.joint2 - w->joints.size()];
            if ((j1.type != B2G_JOINT_REVOLUTE && j1.type != B2G_JOINT_PRISMATIC) ||
                (j2.type != B2G_JOINT_REVOLUTE && j2.type != B2G_JOINT_PRISMATIC))
                return fail(w, B2G_ERR_INVALID_ARG, "a gear joint couples revolute or prismatic joints");
            if (d.body_a != j1.body_b || d.body_b != j2.body_b)
                return fail(w, B2G_ERR_INVALID_ARG, "a gear joint's body_a / body_b must be its joints' body_b");
            if ((w->h_flags[j1.body_b] & BF_TYPE_MASK) != BODY_DYNAMIC || (w->h_flags[j2.body_b] & BF_TYPE_MASK) != BODY_DYNAMIC)
                return fail(w, B2G_ERR_INVALID_ARG, "a gear joint's joints must have a dynamic body_b");
        }
        /* B2pulleyJointDef::initialize asserts ratio > B2_EPSILON (src/joints/b2_pulley_joint.rs:81) and
         * the joint's constructor ratio != 0 (private/dynamics/joints/b2_pulley_joint.rs:30) */
        if (d.type == B2G_JOINT_PULLEY && !(d.ratio > FLT_EPSILON))
            return fail(w, B2G_ERR_INVALID_ARG, "a pulley joint's ratio must be greater than FLT_EPSILON");
    }
    if (n > 0) tape_touch(w);
    if (w->device_authoritative) {
        int rc = download_joint_impulses(w);
        if (rc != B2G_OK) return rc;
        for (int i = 0; i < n && rc == B2G_OK; ++i)
            if (defs[i].type == B2G_JOINT_MOUSE || defs[i].type == B2G_JOINT_GEAR)
                rc = download_state(w);  /* the bodies' transforms */
        if (rc != B2G_OK) return rc;
    }
    for (int i = 0; i < n; ++i) {
        if (ids) ids[i] = (uint32_t)w->joints.size();
        w->joints.push_back(defs[i]);
        w->h_jdead.push_back(0);
        w->gear.emplace_back();
        if (defs[i].type == B2G_JOINT_GEAR) w->gear.back() = gear_frame(w, defs[i]);
        if (defs[i].type == B2G_JOINT_MOUSE) {
            /* b2_mouse_joint_new (src/joints/b2_mouse_joint.rs:140-160): the target in body B's frame */
            const V2 la = mul_t(host_xf(w, (int)defs[i].body_b), mk(defs[i].target.x, defs[i].target.y));
            w->joints.back().local_anchor_b = b2g_vec2{la.x, la.y};
        }
        w->h_jimp.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        /* the wheel joint's damping rides in the w slot of its second impulse record */
        w->h_jimp2.push_back(make_float4(0.0f, 0.0f, 0.0f, defs[i].type == B2G_JOINT_WHEEL ? defs[i].damping : 0.0f));
        if (!defs[i].collide_connected) w->joint_filter_pending = true;
    }
    if (n > 0) w->joints_dirty = true;
    return B2G_OK;
}

}  // extern "C"

namespace {

/* The world's host mirrors made current before a host-side edit of a stepped world: first the edit's
 * contact changes on the device (destroyed contacts, filtering flags), which may wake bodies, then the
 * device's bodies and proxies are downloaded; the edited mirrors are uploaded by the next prepare. */
int begin_host_edit(World* w, const std::vector<uint8_t>* fix_mark, const std::vector<int2>* body_pairs) {
    if (!w->device_authoritative) {
        w->host_dirty = true;
        return B2G_OK;
    }
    int rc = prepare(w);
    if (rc != B2G_OK) return rc;
    rc = check_status(w);
    if (rc != B2G_OK) return rc;
    const bool any_mark = fix_mark && std::any_of(fix_mark->begin(), fix_mark->end(), [](uint8_t m) { return m != 0; });
    const bool any_pair = body_pairs && !body_pairs->empty();
    if (any_mark || any_pair) {
        const int nf = (int)w->h_fbody.size();
        const int np = any_pair ? (int)body_pairs->size() : 0;
        uint8_t* d_mark = nullptr;
        int2* d_pairs = nullptr;
        if (cudaMalloc(&d_mark, (size_t)std::max(nf, 1)) != cudaSuccess ||
            (np > 0 && cudaMalloc(&d_pairs, (size_t)np * sizeof(int2)) != cudaSuccess)) {
            cudaFree(d_mark);
            cudaGetLastError();
            return fail(w, B2G_ERR_OUT_OF_MEMORY, "cudaMalloc for a contact edit failed");
        }
        int n_events0 = 0;
        CUDA_OK(w, cudaMemcpy(&n_events0, w->d.cnt + CNT_EVENTS, sizeof(int), cudaMemcpyDeviceToHost));
        cudaMemsetAsync(d_mark, 0, (size_t)std::max(nf, 1), w->stream);
        if (any_mark) cudaMemcpyAsync(d_mark, fix_mark->data(), (size_t)nf, cudaMemcpyHostToDevice, w->stream);
        if (np > 0) cudaMemcpyAsync(d_pairs, body_pairs->data(), (size_t)np * sizeof(int2), cudaMemcpyHostToDevice, w->stream);
        launch_edit_contacts(w->d, d_mark, d_pairs, np, w->record_events, w->stream);
        const cudaError_t e = cudaStreamSynchronize(w->stream);
        cudaFree(d_mark);
        cudaFree(d_pairs);
        if (e != cudaSuccess) return fail(w, B2G_ERR_CUDA, cudaGetErrorString(e));
        /* the destroyed contacts' end events wait on the host for the next b2g_get_events; the
         * device list keeps only the last step's */
        int n_events1 = 0;
        CUDA_OK(w, cudaMemcpy(&n_events1, w->d.cnt + CNT_EVENTS, sizeof(int), cudaMemcpyDeviceToHost));
        n_events1 = std::min(n_events1, w->d.event_cap);
        if (n_events1 > n_events0) {
            const size_t k = w->pending_events.size();
            w->pending_events.resize(k + (size_t)(n_events1 - n_events0));
            CUDA_OK(w, cudaMemcpy(w->pending_events.data() + k, w->d.events + n_events0,
                                  (size_t)(n_events1 - n_events0) * sizeof(int4), cudaMemcpyDeviceToHost));
            CUDA_OK(w, cudaMemcpyAsync(w->d.cnt + CNT_EVENTS, &n_events0, sizeof(int), cudaMemcpyHostToDevice, w->stream));
        }
        int status = 0;
        CUDA_OK(w, cudaMemcpy(&status, w->d.cnt + CNT_STATUS, sizeof(int), cudaMemcpyDeviceToHost));
        rc = status_error(w, status);
        if (rc != B2G_OK) return rc;
    }
    rc = download_state(w);
    if (rc != B2G_OK) return rc;
    w->host_dirty = true;
    return B2G_OK;
}

/* set_awake(true) on a host mirror (src/b2_body.rs:783-801): not for static bodies; sleep time 0 */
void host_wake(World* w, int b) {
    if ((w->h_flags[b] & BF_TYPE_MASK) == BODY_STATIC) return;
    w->h_flags[b] |= BF_AWAKE;
    w->h_vel[b].w = 0.0f;
}

/* a fixture's proxy is destroyed (B2fixture::destroy_proxies, private/dynamics/b2_fixture.rs:135-145) */
void drop_proxy(World* w, int f) {
    if (w->h_refid[f] != 0xffffffffu) free_refid(w, w->h_refid[f]);
    w->h_refid[f] = 0xffffffffu;
    const float inf = INFINITY;
    w->h_fat[f] = make_float4(inf, inf, -inf, -inf);
    w->h_moved[f] = 0;
}

bool has_duplicates(const uint32_t* ids, int n) {
    std::vector<uint32_t> v(ids, ids + n);
    std::sort(v.begin(), v.end());
    return std::adjacent_find(v.begin(), v.end()) != v.end();
}

}  // namespace

extern "C" {

/* B2world::destroy_joint, private/dynamics/b2_world.rs:278-340, for each joint in the given order:
 * both bodies woken, the joint leaves the solver and the islands, and without collide_connected the
 * contacts between its bodies are flagged for filtering at the next collide. */
int b2g_destroy_joints(void* p, const uint32_t* ids, int32_t n) {
    World* w = W(p);
    if (!w || n < 0 || (n > 0 && !ids)) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i)
        if (ids[i] >= w->joints.size() || w->h_jdead[ids[i]])
            return fail(w, B2G_ERR_INVALID_ARG, "joint id out of range or already destroyed");
    if (has_duplicates(ids, n)) return fail(w, B2G_ERR_INVALID_ARG, "a joint id appears twice");
    if (n == 0) return B2G_OK;
    tape_touch(w);
    std::vector<int2> pairs;
    for (int i = 0; i < n; ++i) {
        const b2g_joint_def& j = w->joints[ids[i]];
        if (!j.collide_connected) pairs.push_back(make_int2((int)j.body_a, (int)j.body_b));
    }
    int rc = download_joint_impulses(w);
    if (rc != B2G_OK) return rc;
    rc = begin_host_edit(w, nullptr, &pairs);
    if (rc != B2G_OK) return rc;
    for (int i = 0; i < n; ++i) {
        const b2g_joint_def& j = w->joints[ids[i]];
        host_wake(w, (int)j.body_a);
        host_wake(w, (int)j.body_b);
        w->h_jdead[ids[i]] = 1;
    }
    w->joints_dirty = true;
    return B2G_OK;
}

/* B2body::destroy_fixture, private/dynamics/b2_body.rs:214-289, for each fixture in the given order:
 * its contacts are destroyed (end events, wakes), its proxy is destroyed (the id returns to the
 * tree's free list), it leaves its body's fixture list and the body's mass data is reset. */
int b2g_destroy_fixtures(void* p, const uint32_t* ids, int32_t n) {
    World* w = W(p);
    if (!w || n < 0 || (n > 0 && !ids)) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i)
        if (ids[i] >= w->h_fbody.size() || w->h_fdead[ids[i]])
            return fail(w, B2G_ERR_INVALID_ARG, "fixture id out of range or already destroyed");
    if (has_duplicates(ids, n)) return fail(w, B2G_ERR_INVALID_ARG, "a fixture id appears twice");
    if (n == 0) return B2G_OK;
    tape_touch(w);
    std::vector<uint8_t> mark(w->h_fbody.size(), 0);
    for (int i = 0; i < n; ++i) mark[ids[i]] = 1;
    int rc = begin_host_edit(w, &mark, nullptr);
    if (rc != B2G_OK) return rc;
    for (int i = 0; i < n; ++i) {
        const int f = (int)ids[i];
        const int b = w->h_fbody[f];
        std::vector<int>& list = w->body_fixtures[b];
        list.erase(std::remove(list.begin(), list.end(), f), list.end());
        drop_proxy(w, f);
        w->h_fdead[f] = 1;
        reset_mass_data(w, b);
    }
    return B2G_OK;
}

/* B2world::destroy_body, private/dynamics/b2_world.rs:100-158, for each body in the given order: its
 * joints are destroyed (newest first, waking their bodies), its contacts are destroyed (end events,
 * wakes), its fixtures' proxies are destroyed in the body's fixture-list order (newest first). The
 * body keeps its id as a static, disabled body without fixtures; its last state stays readable. */
int b2g_destroy_bodies(void* p, const uint32_t* ids, int32_t n) {
    World* w = W(p);
    if (!w || n < 0 || (n > 0 && !ids)) return B2G_ERR_INVALID_ARG;
    for (int i = 0; i < n; ++i)
        if (ids[i] >= w->h_flags.size() || w->h_bdead[ids[i]])
            return fail(w, B2G_ERR_INVALID_ARG, "body id out of range or already destroyed");
    if (has_duplicates(ids, n)) return fail(w, B2G_ERR_INVALID_ARG, "a body id appears twice");
    if (n == 0) return B2G_OK;
    tape_touch(w);
    std::vector<uint8_t> dead_body(w->h_flags.size(), 0), mark(w->h_fbody.size(), 0);
    for (int i = 0; i < n; ++i) dead_body[ids[i]] = 1;
    for (size_t f = 0; f < w->h_fbody.size(); ++f)
        if (!w->h_fdead[f] && dead_body[w->h_fbody[f]]) mark[f] = 1;
    int rc = download_joint_impulses(w);
    if (rc != B2G_OK) return rc;
    rc = begin_host_edit(w, &mark, nullptr);
    if (rc != B2G_OK) return rc;
    bool joints_gone = false;
    for (int i = 0; i < n; ++i) {
        const uint32_t b = ids[i];
        /* the body's joint list is newest first */
        for (int j = (int)w->joints.size() - 1; j >= 0; --j) {
            if (w->h_jdead[j] || (w->joints[j].body_a != b && w->joints[j].body_b != b)) continue;
            host_wake(w, (int)w->joints[j].body_a);
            host_wake(w, (int)w->joints[j].body_b);
            w->h_jdead[j] = 1;
            joints_gone = true;
        }
        for (int f : w->body_fixtures[b]) {
            drop_proxy(w, f);
            w->h_fdead[f] = 1;
        }
        w->body_fixtures[b].clear();
        w->h_bdead[b] = 1;
        w->h_flags[b] = (uint32_t)BODY_STATIC;  /* static, disabled, asleep: no step touches it */
        w->h_mass[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (joints_gone) w->joints_dirty = true;
    return B2G_OK;
}

/* B2fixture::set_filter_data + refilter (private/dynamics/b2_fixture.rs:175-211): the fixture's
 * contacts are flagged for filtering at the next collide (destroyed there if the bodies or the
 * filter no longer allow them) and its proxy is touched, so the next broadphase queries it and
 * pairs the new filter allows are made. */
int b2g_set_filter_data(void* p, uint32_t f, uint16_t category_bits, uint16_t mask_bits, int16_t group_index) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (f >= w->h_fbody.size() || w->h_fdead[f]) return fail(w, B2G_ERR_INVALID_ARG, "fixture id out of range or destroyed");
    tape_touch(w);
    std::vector<uint8_t> mark(w->h_fbody.size(), 0);
    mark[f] = 2;
    int rc = begin_host_edit(w, &mark, nullptr);
    if (rc != B2G_OK) return rc;
    w->h_filter[f] = (uint32_t)category_bits | ((uint32_t)mask_bits << 16);
    w->h_group[f] = (uint32_t)(uint16_t)group_index | (w->h_group[f] & 0x10000u);
    if (w->h_refid[f] != 0xffffffffu) w->h_moved[f] = 1;
    return B2G_OK;
}

int b2g_refilter(void* p, uint32_t f) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (f >= w->h_fbody.size() || w->h_fdead[f]) return fail(w, B2G_ERR_INVALID_ARG, "fixture id out of range or destroyed");
    const uint32_t x = w->h_filter[f];
    return b2g_set_filter_data(p, f, (uint16_t)(x & 0xffffu), (uint16_t)(x >> 16), (int16_t)(w->h_group[f] & 0xffffu));
}

int b2g_get_joint_impulses(void* p, uint32_t first, uint32_t count, float* out) {
    World* w = W(p);
    if (!w || (!out && count)) return B2G_ERR_INVALID_ARG;
    if ((size_t)first + count > w->joints.size()) return fail(w, B2G_ERR_INVALID_ARG, "joint range out of bounds");
    if (count == 0) return B2G_OK;
    if (w->device_authoritative && !w->joints_dirty) {
        int rc = check_status(w);
        if (rc != B2G_OK) return rc;
        rc = download_joint_impulses(w);
        if (rc != B2G_OK) return rc;
    }
    for (uint32_t i = 0; i < count; ++i) {
        const float4 a = w->h_jimp[first + i], b = w->h_jimp2[first + i];
        const int jt = w->joints[first + i].type;
        if (jt != B2G_JOINT_REVOLUTE && jt != B2G_JOINT_PRISMATIC && jt != B2G_JOINT_WHEEL) {
            out[5 * i + 0] = a.x;
            out[5 * i + 1] = a.y;
            out[5 * i + 2] = a.z;
            out[5 * i + 3] = 0.0f;
            out[5 * i + 4] = 0.0f;
            continue;
        }
        out[5 * i + 0] = a.x;
        out[5 * i + 1] = a.y;
        out[5 * i + 2] = a.z;
        out[5 * i + 3] = a.w;
        out[5 * i + 4] = b.x;
    }
    return B2G_OK;
}

int b2g_get_joint_order(void* p, uint32_t* out, int32_t cap, int32_t* n) {
    World* w = W(p);
    if (!w || !n || (!out && cap > 0)) return B2G_ERR_INVALID_ARG;
    if (!w->h_flags.empty()) {
        int rc = prepare(w);
        if (rc != B2G_OK) return rc;
    }
    const int nj = (int)w->h_jorder.size();
    *n = nj;
    if (cap < nj) return fail(w, B2G_ERR_CAPACITY, "joint order buffer too small");
    for (int i = 0; i < nj; ++i) out[i] = (uint32_t)w->h_jorder[i];
    return B2G_OK;
}

int b2g_step(void* p, float dt, int32_t vi, int32_t pi) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (w->continuous && w->tape && w->tape->recording)
        return fail(w, B2G_ERR_UNSUPPORTED, "the tape does not record the continuous pass; call b2g_set_continuous_physics(world, 0) while taping");
    return step(w, dt, vi, pi);
}

int b2g_synchronize(void* p) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    return check_status(w);
}

int b2g_get_body_states_async(void* p, uint32_t first, uint32_t count, b2g_body_state* out) {
    World* w = W(p);
    if (!w || (!out && count > 0)) return B2G_ERR_INVALID_ARG;
    const int synced = sync_host_edits(w);
    if (synced != B2G_OK) return synced;
    if ((size_t)first + count > w->h_flags.size()) return fail(w, B2G_ERR_INVALID_ARG, "body range out of bounds");
    if (count == 0) return B2G_OK;
    if (!(w->device_authoritative && (int)(first + count) <= w->uploaded_bodies))
        return b2g_get_body_states(p, first, count, out);  /* the host holds the state: nothing to overlap */
    if (!w->copy_stream) {
        CUDA_OK(w, cudaStreamCreateWithFlags(&w->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < 2; ++i) {
            CUDA_OK(w, cudaEventCreateWithFlags(&w->ev_packed[i], cudaEventDisableTiming));
            CUDA_OK(w, cudaEventCreateWithFlags(&w->ev_copied[i], cudaEventDisableTiming));
        }
    }
    if (w->ring_cap < (int)count) {
        CUDA_OK(w, cudaStreamSynchronize(w->copy_stream));
        for (int i = 0; i < 2; ++i) {
            if (w->d_ring[i]) cudaFree(w->d_ring[i]);
            w->d_ring[i] = nullptr;
            w->ring_used[i] = false;
        }
        w->ring_cap = 0;
        for (int i = 0; i < 2; ++i) CUDA_OK(w, cudaMalloc((void**)&w->d_ring[i], count * sizeof(b2g_body_state)));
        w->ring_cap = (int)count;
    }
    const int i = w->ring_next;
    w->ring_next ^= 1;
    /* the snapshot is taken in stream order after the last issued step; the copy out of this
     * buffer two requests ago must have finished before it is overwritten */
    if (w->ring_used[i]) CUDA_OK(w, cudaStreamWaitEvent(w->stream, w->ev_copied[i], 0));
    const int grid = grid_for((int)count, 256, w->num_sms * 8);
    k_pack_states<<<grid, 256, 0, w->stream>>>(w->d, first, count, w->d_ring[i], nullptr);
    B2G_LAUNCHED(1);
    CUDA_OK(w, cudaEventRecord(w->ev_packed[i], w->stream));
    CUDA_OK(w, cudaStreamWaitEvent(w->copy_stream, w->ev_packed[i], 0));
    if (w->pageable) {
        const size_t n4 = (size_t)count * sizeof(b2g_body_state) / sizeof(float4);
        k_copy_states<<<grid_for((int)std::min<size_t>(n4, 1u << 30), 256, w->num_sms * 4), 256, 0, w->copy_stream>>>(
            (const float4*)w->d_ring[i], (float4*)out, n4);
        B2G_LAUNCHED(1);
    } else {
        CUDA_OK(w, cudaMemcpyAsync(out, w->d_ring[i], count * sizeof(b2g_body_state), cudaMemcpyDeviceToHost,
                                   w->copy_stream));
    }
    CUDA_OK(w, cudaEventRecord(w->ev_copied[i], w->copy_stream));
    w->ring_used[i] = true;
    CUDA_OK(w, cudaGetLastError());
    return B2G_OK;
}

int b2g_wait_body_states(void* p) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (w->copy_stream) CUDA_OK(w, cudaStreamSynchronize(w->copy_stream));
    return check_status(w);
}

int b2g_get_body_states(void* p, uint32_t first, uint32_t count, b2g_body_state* out) {
    World* w = W(p);
    if (!w || (!out && count > 0)) return B2G_ERR_INVALID_ARG;
    const int synced = sync_host_edits(w);
    if (synced != B2G_OK) return synced;
    if ((size_t)first + count > w->h_flags.size()) return fail(w, B2G_ERR_INVALID_ARG, "body range out of bounds");
    if (count == 0) return B2G_OK;
    if (w->device_authoritative && (int)(first + count) <= w->uploaded_bodies) {
        /* one kernel packs the caller's layout; with coherent access to pageable host memory
         * (Grace's C2C link) it writes straight into the caller's buffer, else into a device
         * buffer that is copied out in one piece */
        const int grid = grid_for((int)count, 256, w->num_sms * 8);
        if (w->pageable) {
            int status = 0;
            k_pack_states<<<grid, 256, 0, w->stream>>>(w->d, first, count, out, &status);
            B2G_LAUNCHED(1);
            CUDA_OK(w, cudaGetLastError());
            CUDA_OK(w, cudaStreamSynchronize(w->stream));
            return status_error(w, ((volatile int*)&status)[0]);
        } else {
            if (w->d_states_cap < (int)count) {
                if (w->d_states) cudaFree(w->d_states);
                w->d_states = nullptr;
                w->d_states_cap = 0;
                CUDA_OK(w, cudaMalloc((void**)&w->d_states, count * sizeof(b2g_body_state)));
                w->d_states_cap = (int)count;
            }
            k_pack_states<<<grid, 256, 0, w->stream>>>(w->d, first, count, w->d_states, nullptr);
            B2G_LAUNCHED(1);
            CUDA_OK(w, cudaMemcpyAsync(out, w->d_states, count * sizeof(b2g_body_state), cudaMemcpyDeviceToHost,
                                       w->stream));
        }
        return check_status(w);  /* waits for the stream and reports device-side errors */
    }
    std::vector<float4> xf(count), pos(count), vel(count);
    {
        if (w->device_authoritative) {
            int rc = download_state(w);
            if (rc != B2G_OK) return rc;
        }
        for (uint32_t i = 0; i < count; ++i) {
            xf[i] = w->h_xf[first + i];
            pos[i] = w->h_pos[first + i];
            vel[i] = w->h_vel[first + i];
        }
    }
    for (uint32_t i = 0; i < count; ++i) {
        b2g_body_state& s = out[i];
        s.position = b2g_vec2{xf[i].x, xf[i].y};
        s.angle = pos[i].z;
        s.linear_velocity = b2g_vec2{vel[i].x, vel[i].y};
        s.angular_velocity = vel[i].z;
        s.world_center = b2g_vec2{pos[i].x, pos[i].y};
    }
    return B2G_OK;
}

/* B2body::get_mass_data / get_local_center (src/b2_body.rs): per body mass, 1/mass, rotational
 * inertia about the centre of mass (m_I; get_inertia adds mass * |local centre|^2), its inverse,
 * local centre x, y. */
int b2g_get_mass_data(void* p, uint32_t first, uint32_t count, float* out) {
    World* w = W(p);
    if (!w || (!out && count > 0)) return B2G_ERR_INVALID_ARG;
    const int synced = sync_host_edits(w);
    if (synced != B2G_OK) return synced;
    if ((size_t)first + count > w->h_flags.size()) return fail(w, B2G_ERR_INVALID_ARG, "body range out of bounds");
    std::vector<float4> m(count);
    std::vector<float2> lc(count);
    if (w->device_authoritative && (int)(first + count) <= w->uploaded_bodies) {
        CUDA_OK(w, cudaStreamSynchronize(w->stream));
        CUDA_OK(w, cudaMemcpy(m.data(), w->d.b_mass + first, count * sizeof(float4), cudaMemcpyDeviceToHost));
        CUDA_OK(w, cudaMemcpy(lc.data(), w->d.b_lc + first, count * sizeof(float2), cudaMemcpyDeviceToHost));
    } else {
        for (uint32_t i = 0; i < count; ++i) {
            m[i] = w->h_mass[first + i];
            lc[i] = w->h_lc[first + i];
        }
    }
    for (uint32_t i = 0; i < count; ++i) {
        float* o = out + 6 * (size_t)i;
        o[0] = m[i].x;
        o[1] = m[i].y;
        o[2] = m[i].z;
        o[3] = m[i].w;
        o[4] = lc[i].x;
        o[5] = lc[i].y;
    }
    return B2G_OK;
}

/* B2body::set_transform, private/dynamics/b2_body.rs:418-447 */
int b2g_set_transform(void* p, uint32_t b, b2g_vec2 position, float angle) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (b >= w->h_flags.size() || w->h_bdead[b]) return fail(w, B2G_ERR_INVALID_ARG, "body id out of range or destroyed");
    tape_touch(w);
    if (w->device_authoritative) {
        int rc = prepare(w);
        if (rc != B2G_OK) return rc;
        launch_set_transform(w->d, (int)b, position.x, position.y, angle, w->stream);
        CUDA_OK(w, cudaGetLastError());
    } else {
        const Rot q = rot(angle);
        w->h_xf[b] = make_float4(position.x, position.y, q.s, q.c);
        const Xf xf = host_xf(w, (int)b);
        const V2 c = mul(xf, mk(w->h_lc[b].x, w->h_lc[b].y));
        w->h_pos[b] = make_float4(c.x, c.y, angle, 0.0f);
        w->h_pos0[b] = make_float4(c.x, c.y, angle, 0.0f);
        for (int f : w->body_fixtures[b]) {
            if (w->h_refid[f] == 0xffffffffu) continue;
            AABB a1, a2;
            shape_aabb(w->h_shape[f], xf, a1);
            shape_aabb(w->h_shape[f], xf, a2);
            const AABB swept = combine(a1, a2);
            host_move_proxy(w, f, swept, sub(center(a2), center(a1)));
        }
    }
    w->new_contacts = true;
    return B2G_OK;
}

int b2g_set_linear_velocity(void* p, uint32_t b, b2g_vec2 v) {
    return p ? body_op(W(p), 0, b, v.x, v.y, 0.0f, 0.0f, 0.0f, 0) : B2G_ERR_INVALID_ARG;
}
int b2g_set_angular_velocity(void* p, uint32_t b, float av) {
    return p ? body_op(W(p), 1, b, 0.0f, 0.0f, av, 0.0f, 0.0f, 0) : B2G_ERR_INVALID_ARG;
}
int b2g_apply_force(void* p, uint32_t b, b2g_vec2 force, b2g_vec2 point, int32_t wake) {
    return p ? body_op(W(p), 2, b, force.x, force.y, 0.0f, point.x, point.y, wake) : B2G_ERR_INVALID_ARG;
}
int b2g_apply_linear_impulse(void* p, uint32_t b, b2g_vec2 impulse, b2g_vec2 point, int32_t wake) {
    return p ? body_op(W(p), 3, b, impulse.x, impulse.y, 0.0f, point.x, point.y, wake) : B2G_ERR_INVALID_ARG;
}
int b2g_apply_force_to_center(void* p, uint32_t b, b2g_vec2 force, int32_t wake) {
    return p ? body_op(W(p), 4, b, force.x, force.y, 0.0f, 0.0f, 0.0f, wake) : B2G_ERR_INVALID_ARG;
}
int b2g_apply_torque(void* p, uint32_t b, float torque, int32_t wake) {
    return p ? body_op(W(p), 5, b, 0.0f, 0.0f, torque, 0.0f, 0.0f, wake) : B2G_ERR_INVALID_ARG;
}
int b2g_apply_linear_impulse_to_center(void* p, uint32_t b, b2g_vec2 impulse, int32_t wake) {
    return p ? body_op(W(p), 6, b, impulse.x, impulse.y, 0.0f, 0.0f, 0.0f, wake) : B2G_ERR_INVALID_ARG;
}
int b2g_apply_angular_impulse(void* p, uint32_t b, float impulse, int32_t wake) {
    return p ? body_op(W(p), 7, b, 0.0f, 0.0f, impulse, 0.0f, 0.0f, wake) : B2G_ERR_INVALID_ARG;
}
int b2g_set_mouse_target(void* p, uint32_t j, b2g_vec2 target) {
    World* w = W(p);
    if (!w || j >= w->joints.size() || w->joints[j].type != B2G_JOINT_MOUSE)
        return w ? fail(w, B2G_ERR_INVALID_ARG, "not a mouse joint") : B2G_ERR_INVALID_ARG;
    b2g_joint_def& jd = w->joints[j];
    if (target.x == jd.target.x && target.y == jd.target.y) return B2G_OK;
    tape_touch(w);
    int rc = body_op(w, 8, jd.body_b, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1);  /* set_awake(true) */
    if (rc != B2G_OK) return rc;
    if (w->device_authoritative && !w->joints_dirty) {
        rc = download_joint_impulses(w);
        if (rc != B2G_OK) return rc;
    }
    jd.target = target;
    w->joints_dirty = true;
    return B2G_OK;
}

int b2g_set_awake(void* p, uint32_t b, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    if (!flag) W(p)->asleep_seen = true;
    return body_op(W(p), 8, b, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, flag);
}

int b2g_get_awake(void* p, uint32_t first, uint32_t count, uint8_t* out) {
    World* w = W(p);
    if (!w || (!out && count)) return B2G_ERR_INVALID_ARG;
    const int synced = sync_host_edits(w);
    if (synced != B2G_OK) return synced;
    if ((size_t)first + count > w->h_flags.size()) return fail(w, B2G_ERR_INVALID_ARG, "body range out of bounds");
    if (count == 0) return B2G_OK;
    std::vector<uint32_t> fl(count);
    if (w->device_authoritative) {
        int rc = check_status(w);
        if (rc != B2G_OK) return rc;
        CUDA_OK(w, cudaMemcpy(fl.data(), w->d.b_flags + first, count * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    } else {
        std::copy(w->h_flags.begin() + first, w->h_flags.begin() + first + count, fl.begin());
    }
    for (uint32_t i = 0; i < count; ++i) out[i] = (fl[i] & BF_AWAKE) ? 1 : 0;
    return B2G_OK;
}

int b2g_set_gravity(void* p, b2g_vec2 g) {
    if (!p) return B2G_ERR_INVALID_ARG;
    W(p)->gravity = g;
    return B2G_OK;
}
int b2g_set_allow_sleeping(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    if (flag) tape_touch(W(p));
    W(p)->allow_sleep = flag != 0;
    return B2G_OK;
}
int b2g_set_part_solve(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    World* w = W(p);
    if (w->part_solve != (flag != 0)) drop_graphs(w);
    w->part_solve = flag != 0;
    return B2G_OK;
}
int b2g_set_warm_starting(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    W(p)->warm = flag != 0;
    return B2G_OK;
}
int b2g_set_continuous_physics(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    World* w = W(p);
    if (flag && (w->filter_fn || w->pre_solve_fn))
        return fail(w, B2G_ERR_UNSUPPORTED, "host contact filters and pre_solve callbacks cannot run inside the continuous pass");
    if (flag && w->auto_grow)
        return fail(w, B2G_ERR_UNSUPPORTED, "automatic capacity growth does not cover the continuous pass");
    w->continuous = flag != 0;
    return B2G_OK;
}
int b2g_set_toi_schedule(void* p, int32_t schedule) {
    if (!p) return B2G_ERR_INVALID_ARG;
    if (schedule < B2G_TOI_SCHEDULE_SIDE_BY_SIDE || schedule > B2G_TOI_SCHEDULE_RESTART_ON_ADVANCE)
        return fail(W(p), B2G_ERR_INVALID_ARG, "unknown time-of-impact schedule");
    W(p)->toi_schedule = schedule;
    return B2G_OK;
}

int b2g_set_auto_clear_forces(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    W(p)->auto_clear = flag != 0;
    return B2G_OK;
}
int b2g_clear_forces(void* p) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (w->device_authoritative) {
        launch_clear_forces(w->d, w->stream);
    } else {
        for (auto& f : w->h_force) f = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    return B2G_OK;
}

int b2g_set_contact_events(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    W(p)->record_events = flag != 0;
    return B2G_OK;
}
int b2g_set_record_pairs(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    W(p)->record_pairs = flag != 0;
    return B2G_OK;
}

int b2g_set_auto_grow(void* p, int32_t flag) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (flag && w->continuous)
        return fail(w, B2G_ERR_UNSUPPORTED, "automatic capacity growth does not cover the continuous pass; turn continuous physics off");
    w->auto_grow = flag != 0;
    return B2G_OK;
}

int b2g_set_contact_filter(void* p, b2g_contact_filter_fn fn, void* user) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (fn && w->continuous)
        return fail(w, B2G_ERR_UNSUPPORTED, "a host contact filter cannot run inside the continuous pass; turn continuous physics off");
    w->filter_fn = fn;
    w->filter_user = user;
    return B2G_OK;
}

int b2g_set_pre_solve(void* p, b2g_pre_solve_fn fn, void* user) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    if (fn && w->continuous)
        return fail(w, B2G_ERR_UNSUPPORTED, "a pre_solve callback cannot run inside the continuous pass; turn continuous physics off");
    w->pre_solve_fn = fn;
    w->pre_solve_user = user;
    return B2G_OK;
}

int b2g_set_barrier_limit(void* p, int64_t cycles) {
    World* w = W(p);
    if (!w || cycles < 0) return B2G_ERR_INVALID_ARG;
    const long long units = cycles == 0 ? 0 : std::max(1LL, std::min((long long)INT32_MAX, (long long)(cycles >> 10)));
    w->barrier_limit_units = (int)units;
    return write_barrier_settings(w);
}

int b2g_set_hierarchy_max_age(void* p, int32_t passes) {
    World* w = W(p);
    if (!w || passes < 0) return B2G_ERR_INVALID_ARG;
    w->hierarchy_max_age = passes;
    return write_barrier_settings(w);
}

int b2g_debug_hold_barriers(void* p, int32_t extra) {
    World* w = W(p);
    if (!w || extra < 0) return B2G_ERR_INVALID_ARG;
    w->barrier_hold = extra;
    return write_barrier_settings(w);
}

int b2g_set_graph_capture(void* p, int32_t flag) {
    if (!p) return B2G_ERR_INVALID_ARG;
    World* w = W(p);
    w->use_graphs = flag != 0;
    if (!w->use_graphs) drop_graphs(w);
    return B2G_OK;
}

int b2g_get_profile(void* p, b2g_profile* out) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    memset(out, 0, sizeof(*out));
    if (!w->timer.valid || w->steps == 0) return B2G_OK;
    float ms[6] = {0};
    for (int i = 1; i < 6; ++i) {
        if (cudaEventElapsedTime(&ms[i], w->timer.e[0], w->timer.e[i]) != cudaSuccess) {
            cudaGetLastError();
            return fail(w, B2G_ERR_CUDA, "profile events could not be timed");
        }
    }
    float toi = 0.0f;
    if (cudaEventElapsedTime(&toi, w->timer.e[0], w->timer.e[8]) != cudaSuccess) {
        cudaGetLastError();
        return fail(w, B2G_ERR_CUDA, "profile events could not be timed");
    }
    out->collide = ms[2] - ms[1];
    out->solve_init = ms[3] - ms[2];
    out->solve_velocity = ms[4] - ms[3];  /* the persistent solver kernel: velocity and position iterations */
    out->solve_position = 0.0f;
    out->broadphase = (toi - ms[4]) + ms[1];
    out->solve = toi - ms[2];
    out->solve_toi = ms[5] - toi;
    out->step = ms[5];
    return B2G_OK;
}

int b2g_get_phase_times(void* p, float* out, int32_t n) {
    World* w = W(p);
    if (!w || !out || n < 7) return B2G_ERR_INVALID_ARG;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    for (int i = 0; i < std::min(n, 10); ++i) out[i] = 0.0f;
    if (!w->timer.valid || w->steps == 0) return B2G_OK;
    if (n >= 10) {
        /* the tree pass in three: keys + sort, hierarchy, traversal (events 4, 9, 10, 7) */
        const int sub[4] = {4, 9, 10, 7};
        for (int i = 0; i < 3; ++i) {
            if (cudaEventElapsedTime(&out[7 + i], w->timer.e[sub[i]], w->timer.e[sub[i + 1]]) != cudaSuccess) {
                cudaGetLastError();
                return fail(w, B2G_ERR_CUDA, "profile events could not be timed");
            }
        }
    }
    /* event order within a step: 0 start, 1 after the initial broadphase, 2 after collide,
     * 6 after islands, 3 after colouring, 4 after the solver, 7 after the tree pass, 5 end */
    const int order[8] = {0, 1, 2, 6, 3, 4, 7, 5};
    float t[8] = {0};
    for (int i = 1; i < 8; ++i) {
        if (cudaEventElapsedTime(&t[i], w->timer.e[order[0]], w->timer.e[order[i]]) != cudaSuccess) {
            cudaGetLastError();
            return fail(w, B2G_ERR_CUDA, "profile events could not be timed");
        }
    }
    for (int i = 0; i < 7; ++i) out[i] = t[i + 1] - t[i];
    return B2G_OK;
}

int b2g_get_step_stats(void* p, b2g_step_stats* out) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int cnt[CNT_SIZE];
    CUDA_OK(w, cudaMemcpy(cnt, w->d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
    out->bp_node_visits = cnt[CNT_BP_VISITS];
    out->bp_leaf_checks = cnt[CNT_BP_CANDIDATES];
    out->new_pairs = cnt[CNT_NEW];
    out->contacts = cnt[CNT_CONTACTS];
    out->constraints = cnt[CNT_CONS];
    out->interior_slots = cnt[CNT_INTERIOR];
    out->parts = cnt[CNT_PARTS];
    out->colours = cnt[CNT_COLOURS];
    out->contact_capacity = w->d.contact_cap;
    out->pair_capacity = w->d.pair_cap;
    out->capacity_grows = w->capacity_grows;
    out->hierarchy_age = cnt[CNT_BP_AGE];
    out->bp_moved_proxies = cnt[CNT_BP_LAST_MOVED];
    out->bp_warp_max_visits = cnt[CNT_BP_WARP_VISITS];
    out->bp_warp_max_checks = cnt[CNT_BP_WARP_CHECKS];
    return B2G_OK;
}

int b2g_get_counts(void* p, b2g_counts* out) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    out->bodies = (int)w->h_flags.size();
    out->fixtures = (int)w->h_fbody.size();
    out->proxies = w->proxies_created;
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int cnt[CNT_SIZE];
    CUDA_OK(w, cudaMemcpy(cnt, w->d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
    out->contacts = cnt[CNT_CONTACTS];
    out->islands_solved = 0;
    out->colours = cnt[CNT_COLOURS];
    out->pairs = cnt[CNT_PAIRS];
    if (cnt[CNT_CONTACTS] > 0) {
        std::vector<uint32_t> fl(cnt[CNT_CONTACTS]);
        CUDA_OK(w, cudaMemcpy(fl.data(), w->d.c.flags, fl.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        int t = 0;
        for (uint32_t f : fl) t += (f & CF_TOUCHING) && !(f & CF_DEAD) ? 1 : 0;
        out->touching_contacts = t;
    }
    out->islands_solved = cnt[CNT_CONS];
    return B2G_OK;
}

/* ---- exact checkpoint: every device buffer of the world and its stepping state ---- */

namespace {

constexpr uint32_t kStateMagic = 0x53473242u;  /* "B2GS" */
constexpr uint32_t kStateVersion = 2;

struct StateHeader {
    uint32_t magic, version;
    int32_t n_bodies, n_fixtures, body_cap, fix_cap, contact_cap, pair_cap, num_worlds, key_bits, morton_world_bits;
    int32_t minsep_buffers, n_alloc;
    uint64_t buffer_bytes;
    float inv_dt0;
    int32_t steps, swaps_parity, new_contacts, warm, continuous, allow_sleep, auto_clear, toi_schedule, asleep_seen,
        part_solve, proxies_created;
    b2g_vec2 gravity;
};

/* the device holds the world (bodies, fixtures) and nothing is in flight */
int state_ready(World* w) {
    if (w->h_flags.empty()) return fail(w, B2G_ERR_INVALID_ARG, "the world has no bodies");
    if (w->tape && w->tape->recording) return fail(w, B2G_ERR_UNSUPPORTED, "a tape is recording");
    int rc = prepare(w);
    if (rc != B2G_OK) return rc;
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    return check_status(w);
}

/* The host-side part of a world's state, after the device buffers: destroyed-object marks, the
 * joint definitions (a mouse joint's target moves), the proxy-id free list and the next fresh node. */
std::vector<unsigned char> host_state(const World* w) {
    std::vector<unsigned char> b;
    auto put = [&b](const void* p, size_t n) {
        const unsigned char* c = (const unsigned char*)p;
        b.insert(b.end(), c, c + n);
    };
    const int32_t nb = (int32_t)w->h_bdead.size(), nf = (int32_t)w->h_fdead.size(), nj = (int32_t)w->joints.size();
    const int32_t nfree = (int32_t)w->free_refids.size();
    put(&nb, sizeof(nb));
    put(w->h_bdead.data(), (size_t)nb);
    put(&nf, sizeof(nf));
    put(w->h_fdead.data(), (size_t)nf);
    put(&nj, sizeof(nj));
    put(w->joints.data(), (size_t)nj * sizeof(b2g_joint_def));
    put(w->h_jdead.data(), (size_t)nj);
    put(w->gear.data(), (size_t)nj * sizeof(GearFrame));
    put(&nfree, sizeof(nfree));
    put(w->free_refids.data(), (size_t)nfree * sizeof(uint32_t));
    put(&w->next_node, sizeof(w->next_node));
    return b;
}

uint64_t state_bytes(const World* w) {
    uint64_t n = sizeof(StateHeader) + w->alloc_bytes.size() * sizeof(uint64_t);
    for (size_t b : w->alloc_bytes) n += b;
    return n + host_state(w).size();
}

/* After a load: every host mirror from the loaded device buffers, and the host part of the state. */
int load_host_state(World* w, const unsigned char* src, const unsigned char* end) {
    auto get = [&src, end](void* p, size_t n) {
        if ((size_t)(end - src) < n) return false;
        memcpy(p, src, n);
        src += n;
        return true;
    };
    int32_t nb = 0, nf = 0, nj = 0, nfree = 0;
    if (!get(&nb, sizeof(nb)) || nb != (int32_t)w->h_flags.size()) return fail(w, B2G_ERR_INVALID_ARG, "state body count");
    if (!get(w->h_bdead.data(), (size_t)nb)) return fail(w, B2G_ERR_INVALID_ARG, "truncated state");
    if (!get(&nf, sizeof(nf)) || nf != (int32_t)w->h_fbody.size()) return fail(w, B2G_ERR_INVALID_ARG, "state fixture count");
    if (!get(w->h_fdead.data(), (size_t)nf)) return fail(w, B2G_ERR_INVALID_ARG, "truncated state");
    if (!get(&nj, sizeof(nj)) || nj != (int32_t)w->joints.size()) return fail(w, B2G_ERR_INVALID_ARG, "state joint count");
    if (!get(w->joints.data(), (size_t)nj * sizeof(b2g_joint_def)) || !get(w->h_jdead.data(), (size_t)nj) ||
        !get(w->gear.data(), (size_t)nj * sizeof(GearFrame)))
        return fail(w, B2G_ERR_INVALID_ARG, "truncated state");
    if (!get(&nfree, sizeof(nfree)) || nfree < 0) return fail(w, B2G_ERR_INVALID_ARG, "truncated state");
    w->free_refids.resize((size_t)nfree);
    if (!get(w->free_refids.data(), (size_t)nfree * sizeof(uint32_t)) || !get(&w->next_node, sizeof(w->next_node)))
        return fail(w, B2G_ERR_INVALID_ARG, "truncated state");
    DevWorld& d = w->d;
#define D(src_, dst, n) CUDA_OK(w, cudaMemcpy((dst).data(), (src_), (size_t)(n) * sizeof((dst)[0]), cudaMemcpyDeviceToHost))
    if (nb > 0) {
        D(d.b_xf, w->h_xf, nb); D(d.b_pos, w->h_pos, nb); D(d.b_pos0, w->h_pos0, nb); D(d.b_vel, w->h_vel, nb);
        D(d.b_force, w->h_force, nb); D(d.b_mass, w->h_mass, nb); D(d.b_damp, w->h_damp, nb); D(d.b_lc, w->h_lc, nb);
        D(d.b_flags, w->h_flags, nb); D(d.b_world, w->h_world, nb);
    }
    if (nf > 0) {
        D(d.f_shape, w->h_shape, nf); D(d.f_body, w->h_fbody, nf); D(d.f_mat, w->h_fmat, nf);
        D(d.f_filter, w->h_filter, nf); D(d.f_group, w->h_group, nf); D(d.f_refid, w->h_refid, nf);
        D(d.f_fat, w->h_fat, nf); D(d.f_moved, w->h_moved, nf);
    }
#undef D
    /* fixture lists, newest first (fixtures are appended in creation order) */
    for (auto& l : w->body_fixtures) l.clear();
    for (int f = nf - 1; f >= 0; --f)
        if (!w->h_fdead[f]) w->body_fixtures[w->h_fbody[f]].push_back(f);
    int live = 0;
    for (int f = 0; f < nf; ++f) live += w->h_refid[f] != 0xffffffffu ? 1 : 0;
    w->proxies_created = live;
    w->kinematic_or_bullet = false;
    for (int b = 0; b < nb; ++b) {
        const uint32_t fl = w->h_flags[b];
        if ((fl & BF_TYPE_MASK) == BODY_KINEMATIC || ((fl & BF_TYPE_MASK) == BODY_DYNAMIC && (fl & BF_BULLET)))
            w->kinematic_or_bullet = true;
    }
    /* the joints' host copies: impulses from the device, then the colouring and tables re-derived (and
     * re-uploaded: the same contents the state holds) */
    if (nj > 0) {
        int rc = download_joint_impulses(w);
        if (rc != B2G_OK) return rc;
        rc = upload_joints(w);
        if (rc != B2G_OK) return rc;
    }
    w->host_dirty = false;
    return B2G_OK;
}

}  // namespace

int b2g_state_size(void* p, uint64_t* bytes) {
    World* w = W(p);
    if (!w || !bytes) return B2G_ERR_INVALID_ARG;
    int rc = state_ready(w);
    if (rc != B2G_OK) return rc;
    *bytes = state_bytes(w);
    return B2G_OK;
}

int b2g_state_save(void* p, void* out, uint64_t bytes) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    int rc = state_ready(w);
    if (rc != B2G_OK) return rc;
    if (bytes < state_bytes(w)) return fail(w, B2G_ERR_INVALID_ARG, "buffer smaller than b2g_state_size");
    StateHeader h{};
    h.magic = kStateMagic;
    h.version = kStateVersion;
    h.n_bodies = w->d.n_bodies;
    h.n_fixtures = w->d.n_fixtures;
    h.body_cap = w->d.body_cap;
    h.fix_cap = w->d.fix_cap;
    h.contact_cap = w->d.contact_cap;
    h.pair_cap = w->d.pair_cap;
    h.num_worlds = w->num_worlds;
    h.key_bits = w->d.key_bits;
    h.morton_world_bits = w->d.morton_world_bits;
    h.minsep_buffers = w->minsep_buffers;
    h.n_alloc = (int32_t)w->allocations.size();
    h.buffer_bytes = state_bytes(w);
    h.inv_dt0 = w->inv_dt0;
    h.steps = w->steps;
    h.swaps_parity = w->swaps & 1;
    h.new_contacts = w->new_contacts;
    h.warm = w->warm;
    h.continuous = w->continuous;
    h.allow_sleep = w->allow_sleep;
    h.auto_clear = w->auto_clear;
    h.toi_schedule = w->toi_schedule;
    h.asleep_seen = w->asleep_seen;
    h.part_solve = w->part_solve;
    h.proxies_created = w->proxies_created;
    h.gravity = w->gravity;
    unsigned char* o = (unsigned char*)out;
    memcpy(o, &h, sizeof(h));
    o += sizeof(h);
    for (size_t b : w->alloc_bytes) {
        const uint64_t v = b;
        memcpy(o, &v, sizeof(v));
        o += sizeof(v);
    }
    for (size_t i = 0; i < w->allocations.size(); ++i) {
        CUDA_OK(w, cudaMemcpy(o, w->allocations[i], w->alloc_bytes[i], cudaMemcpyDeviceToHost));
        o += w->alloc_bytes[i];
    }
    const std::vector<unsigned char> hs = host_state(w);
    memcpy(o, hs.data(), hs.size());
    return B2G_OK;
}

int b2g_state_load(void* p, const void* in, uint64_t bytes) {
    World* w = W(p);
    if (!w || !in) return B2G_ERR_INVALID_ARG;
    if (bytes < sizeof(StateHeader)) return fail(w, B2G_ERR_INVALID_ARG, "not a world state");
    StateHeader h;
    memcpy(&h, in, sizeof(h));
    if (h.magic != kStateMagic || h.version != kStateVersion || h.buffer_bytes != bytes)
        return fail(w, B2G_ERR_INVALID_ARG, "not a world state of this version");
    const unsigned char* end = (const unsigned char*)in + bytes;
    int rc = state_ready(w);
    if (rc != B2G_OK) return rc;
    rc = ensure_minsep_buffers(w, h.minsep_buffers);
    if (rc != B2G_OK) return rc;
    const unsigned char* src = (const unsigned char*)in + sizeof(h);
    bool same = h.n_bodies == w->d.n_bodies && h.n_fixtures == w->d.n_fixtures && h.body_cap == w->d.body_cap &&
                h.fix_cap == w->d.fix_cap && h.contact_cap == w->d.contact_cap && h.pair_cap == w->d.pair_cap &&
                h.num_worlds == w->num_worlds && h.n_alloc == (int32_t)w->allocations.size() &&
                h.minsep_buffers == w->minsep_buffers;
    for (int32_t i = 0; same && i < h.n_alloc; ++i) {
        uint64_t v;
        memcpy(&v, src + (size_t)i * sizeof(v), sizeof(v));
        same = v == w->alloc_bytes[i];
    }
    if (!same)
        return fail(w, B2G_ERR_INVALID_ARG,
                    "the state was saved from a world of another layout (bodies, fixtures, capacities or worlds)");
    src += (size_t)h.n_alloc * sizeof(uint64_t);
    for (size_t i = 0; i < w->allocations.size(); ++i) {
        if ((size_t)(end - src) < w->alloc_bytes[i]) return fail(w, B2G_ERR_INVALID_ARG, "truncated state");
        CUDA_OK(w, cudaMemcpyAsync(w->allocations[i], src, w->alloc_bytes[i], cudaMemcpyHostToDevice, w->stream));
        src += w->alloc_bytes[i];
    }
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    /* the contact table is the buffer that was current when saved */
    if ((w->swaps & 1) != h.swaps_parity) swap_contacts(w);
    w->d.key_bits = h.key_bits;
    w->d.morton_world_bits = h.morton_world_bits;
    w->inv_dt0 = h.inv_dt0;
    w->steps = h.steps;
    w->new_contacts = h.new_contacts != 0;
    w->warm = h.warm != 0;
    w->continuous = h.continuous != 0;
    w->allow_sleep = h.allow_sleep != 0;
    w->auto_clear = h.auto_clear != 0;
    w->toi_schedule = h.toi_schedule;
    w->asleep_seen = h.asleep_seen != 0;
    w->part_solve = h.part_solve != 0;
    w->proxies_created = h.proxies_created;
    w->gravity = h.gravity;
    w->device_authoritative = true;
    rc = load_host_state(w, src, end);
    if (rc != B2G_OK) return rc;
    /* the barrier and hierarchy settings are the world's, not the saved state's */
    return write_barrier_settings(w);
}

int b2g_get_toi_stats(void* p, int32_t* events, int32_t* last_iterations, int32_t* restarts) {
    World* w = W(p);
    if (!w || !events || !last_iterations || !restarts) return B2G_ERR_INVALID_ARG;
    *events = 0;
    *last_iterations = 0;
    *restarts = 0;
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int cnt[CNT_SIZE];
    CUDA_OK(w, cudaMemcpy(cnt, w->d.cnt, sizeof(cnt), cudaMemcpyDeviceToHost));
    *events = cnt[CNT_TOI_EVENTS];
    *last_iterations = cnt[CNT_TOI_ITERS];
    *restarts = cnt[CNT_TOI_ROLLBACKS];
    return B2G_OK;
}

int b2g_get_contacts(void* p, b2g_contact_info* out, int32_t cap, int32_t* n) {
    World* w = W(p);
    if (!w || !n) return B2G_ERR_INVALID_ARG;
    *n = 0;
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    HostContacts h;
    rc = download_contacts(w, h, out != nullptr);
    if (rc != B2G_OK) return rc;
    int live = 0;
    for (int i = 0; i < h.n; ++i) live += (h.flags[i] & CF_DEAD) ? 0 : 1;
    *n = live;
    if (!out || cap < live || live == 0) return B2G_OK;
    int k = 0;
    for (int i = 0; i < h.n; ++i)
        if (!(h.flags[i] & CF_DEAD)) contact_info(h, i, out[k++]);
    return B2G_OK;
}

int b2g_get_events(void* p, b2g_contact_event* out, int32_t cap, int32_t* n) {
    World* w = W(p);
    if (!w || !n) return B2G_ERR_INVALID_ARG;
    *n = 0;
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int nd = 0;
    CUDA_OK(w, cudaMemcpy(&nd, w->d.cnt + CNT_EVENTS, sizeof(int), cudaMemcpyDeviceToHost));
    nd = std::min(nd, w->d.event_cap);
    const int np = (int)w->pending_events.size();
    const int ne = nd + np;
    *n = ne;
    if (!out || cap < ne || ne == 0) return B2G_OK;
    std::vector<int4> ev(ne);
    std::copy(w->pending_events.begin(), w->pending_events.end(), ev.begin());
    if (nd > 0) CUDA_OK(w, cudaMemcpy(ev.data() + np, w->d.events, nd * sizeof(int4), cudaMemcpyDeviceToHost));
    w->pending_events.clear();
    std::sort(ev.begin(), ev.end(), [](const int4& a, const int4& b) {
        if (a.x != b.x) return a.x < b.x;
        if (a.y != b.y) return a.y < b.y;
        return a.z < b.z;
    });
    for (int i = 0; i < ne; ++i) out[i] = b2g_contact_event{ev[i].x, (uint32_t)ev[i].y, (uint32_t)ev[i].z};
    return B2G_OK;
}

int b2g_get_pairs(void* p, uint32_t* out, int32_t cap, int32_t* n) {
    World* w = W(p);
    if (!w || !n) return B2G_ERR_INVALID_ARG;
    *n = 0;
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int np = 0;
    CUDA_OK(w, cudaMemcpy(&np, w->d.cnt + CNT_PAIRS, sizeof(int), cudaMemcpyDeviceToHost));
    np = std::min(np, w->d.pair_cap);
    *n = np;
    if (!out || cap < np || np == 0) return B2G_OK;
    std::vector<uint2> pr(np);
    CUDA_OK(w, cudaMemcpy(pr.data(), w->d.pairs, np * sizeof(uint2), cudaMemcpyDeviceToHost));
    std::sort(pr.begin(), pr.end(), [](const uint2& a, const uint2& b) { return a.x != b.x ? a.x < b.x : a.y < b.y; });
    for (int i = 0; i < np; ++i) {
        out[2 * i] = pr[i].x;
        out[2 * i + 1] = pr[i].y;
    }
    return B2G_OK;
}

int b2g_get_proxy_ids(void* p, int32_t* out, int32_t cap) {
    World* w = W(p);
    if (!w || (!out && cap > 0)) return B2G_ERR_INVALID_ARG;
    const int nf = std::min((int)w->h_refid.size(), (int)cap);
    for (int f = 0; f < nf; ++f) out[f] = w->h_refid[f] == 0xffffffffu ? -1 : (int32_t)w->h_refid[f];
    return B2G_OK;
}

int b2g_get_proxies(void* p, float* aabbs, uint8_t* moved, int32_t cap) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    const int synced = sync_host_edits(w);
    if (synced != B2G_OK) return synced;
    const int nf = std::min((int)w->h_fbody.size(), (int)cap);
    if (w->device_authoritative) {
        int rc = check_status(w);
        if (rc != B2G_OK) return rc;
        if (aabbs) CUDA_OK(w, cudaMemcpy(aabbs, w->d.f_fat, nf * sizeof(float4), cudaMemcpyDeviceToHost));
        if (moved) CUDA_OK(w, cudaMemcpy(moved, w->d.f_moved, nf, cudaMemcpyDeviceToHost));
    } else {
        if (aabbs) memcpy(aabbs, w->h_fat.data(), nf * sizeof(float4));
        if (moved) memcpy(moved, w->h_moved.data(), nf);
    }
    return B2G_OK;
}

int b2g_collide_pairs(const b2g_fixture_def* da, const float* xfa, const b2g_fixture_def* db, const float* xfb,
                      int32_t n, b2g_contact_info* out) {
    if (n < 0 || (n > 0 && (!da || !db || !xfa || !xfb || !out))) return B2G_ERR_INVALID_ARG;
    if (n == 0) return B2G_OK;
    std::vector<ShapeRec> sa(n), sb(n);
    std::vector<float4> xa(n), xb(n);
    std::vector<int> kind(n);
    for (int i = 0; i < n; ++i) {
        build_shape(da[i], sa[i]);
        build_shape(db[i], sb[i]);
        const int ta = da[i].shape_type, tb = db[i].shape_type;
        if (ta == B2G_SHAPE_CIRCLE && tb == B2G_SHAPE_CIRCLE) kind[i] = KIND_CIRCLES;
        else if (ta == B2G_SHAPE_POLYGON && tb == B2G_SHAPE_CIRCLE) kind[i] = KIND_POLYGON_CIRCLE;
        else if (ta == B2G_SHAPE_POLYGON && tb == B2G_SHAPE_POLYGON) kind[i] = KIND_POLYGONS;
        else if (ta == B2G_SHAPE_EDGE && tb == B2G_SHAPE_CIRCLE) kind[i] = KIND_EDGE_CIRCLE;
        else if (ta == B2G_SHAPE_EDGE && tb == B2G_SHAPE_POLYGON) kind[i] = KIND_EDGE_POLYGON;
        else return B2G_ERR_INVALID_ARG;
        const Rot qa = rot(xfa[3 * i + 2]), qb = rot(xfb[3 * i + 2]);
        xa[i] = make_float4(xfa[3 * i], xfa[3 * i + 1], qa.s, qa.c);
        xb[i] = make_float4(xfb[3 * i], xfb[3 * i + 1], qb.s, qb.c);
    }
    ShapeRec *d_sa = nullptr, *d_sb = nullptr;
    float4 *d_xa = nullptr, *d_xb = nullptr, *d_geo = nullptr, *d_pts = nullptr;
    uint4* d_ids = nullptr;
    int* d_kind = nullptr;
    int rc = B2G_OK;
    if (cudaMalloc(&d_sa, n * sizeof(ShapeRec)) != cudaSuccess || cudaMalloc(&d_sb, n * sizeof(ShapeRec)) != cudaSuccess ||
        cudaMalloc(&d_xa, n * sizeof(float4)) != cudaSuccess || cudaMalloc(&d_xb, n * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&d_geo, n * sizeof(float4)) != cudaSuccess || cudaMalloc(&d_pts, n * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&d_ids, n * sizeof(uint4)) != cudaSuccess || cudaMalloc(&d_kind, n * sizeof(int)) != cudaSuccess) {
        rc = B2G_ERR_OUT_OF_MEMORY;
    }
    std::vector<float4> geo(n), pts(n);
    std::vector<uint4> ids(n);
    if (rc == B2G_OK) {
        cudaMemcpy(d_sa, sa.data(), n * sizeof(ShapeRec), cudaMemcpyHostToDevice);
        cudaMemcpy(d_sb, sb.data(), n * sizeof(ShapeRec), cudaMemcpyHostToDevice);
        cudaMemcpy(d_xa, xa.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
        cudaMemcpy(d_xb, xb.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
        cudaMemcpy(d_kind, kind.data(), n * sizeof(int), cudaMemcpyHostToDevice);
        launch_collide_pairs(d_sa, d_xa, d_sb, d_xb, d_kind, n, d_geo, d_pts, d_ids, 0);
        if (cudaMemcpy(geo.data(), d_geo, n * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(pts.data(), d_pts, n * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(ids.data(), d_ids, n * sizeof(uint4), cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = B2G_ERR_CUDA;
    }
    cudaFree(d_sa);
    cudaFree(d_sb);
    cudaFree(d_xa);
    cudaFree(d_xb);
    cudaFree(d_geo);
    cudaFree(d_pts);
    cudaFree(d_ids);
    cudaFree(d_kind);
    if (rc != B2G_OK) return rc;
    for (int i = 0; i < n; ++i) {
        b2g_contact_info& o = out[i];
        memset(&o, 0, sizeof(o));
        o.fixture_a = o.fixture_b = (uint32_t)i;
        o.manifold_type = (int)(ids[i].z & 0xffu);
        o.point_count = (int)((ids[i].z >> 8) & 0xffu);
        o.touching = o.point_count > 0;
        o.local_normal = b2g_vec2{geo[i].x, geo[i].y};
        o.local_point = b2g_vec2{geo[i].z, geo[i].w};
        o.point_local[0] = b2g_vec2{pts[i].x, pts[i].y};
        o.point_local[1] = b2g_vec2{pts[i].z, pts[i].w};
        o.point_id[0] = ids[i].x;
        o.point_id[1] = ids[i].y;
    }
    return B2G_OK;
}

}  // extern "C"

int b2g_time_of_impact(const b2g_fixture_def* da, const b2g_sweep* swa, const b2g_fixture_def* db,
                       const b2g_sweep* swb, const float* t_max, int32_t n, b2g_toi_output* out) {
    if (n < 0 || (n > 0 && (!da || !db || !swa || !swb || !out))) return B2G_ERR_INVALID_ARG;
    if (n == 0) return B2G_OK;
    std::vector<ShapeRec> sa(n), sb(n);
    std::vector<float4> wa(2 * (size_t)n), wb(2 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        for (const b2g_fixture_def* d : {&da[i], &db[i]})
            if (d->shape_type != B2G_SHAPE_CIRCLE && d->shape_type != B2G_SHAPE_POLYGON && d->shape_type != B2G_SHAPE_EDGE)
                return B2G_ERR_INVALID_ARG;
        build_shape(da[i], sa[i]);
        build_shape(db[i], sb[i]);
        const b2g_sweep& a = swa[i];
        const b2g_sweep& b = swb[i];
        wa[2 * i] = make_float4(a.local_center.x, a.local_center.y, a.c0.x, a.c0.y);
        wa[2 * i + 1] = make_float4(a.c.x, a.c.y, a.a0, a.a);
        wb[2 * i] = make_float4(b.local_center.x, b.local_center.y, b.c0.x, b.c0.y);
        wb[2 * i + 1] = make_float4(b.c.x, b.c.y, b.a0, b.a);
    }
    ShapeRec *d_sa = nullptr, *d_sb = nullptr;
    float4 *d_wa = nullptr, *d_wb = nullptr;
    float* d_t = nullptr;
    int2* d_out = nullptr;
    int rc = B2G_OK;
    if (cudaMalloc(&d_sa, n * sizeof(ShapeRec)) != cudaSuccess || cudaMalloc(&d_sb, n * sizeof(ShapeRec)) != cudaSuccess ||
        cudaMalloc(&d_wa, 2 * n * sizeof(float4)) != cudaSuccess || cudaMalloc(&d_wb, 2 * n * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&d_out, n * sizeof(int2)) != cudaSuccess || (t_max && cudaMalloc(&d_t, n * sizeof(float)) != cudaSuccess))
        rc = B2G_ERR_OUT_OF_MEMORY;
    if (rc == B2G_OK) {
        cudaMemcpy(d_sa, sa.data(), n * sizeof(ShapeRec), cudaMemcpyHostToDevice);
        cudaMemcpy(d_sb, sb.data(), n * sizeof(ShapeRec), cudaMemcpyHostToDevice);
        cudaMemcpy(d_wa, wa.data(), 2 * n * sizeof(float4), cudaMemcpyHostToDevice);
        cudaMemcpy(d_wb, wb.data(), 2 * n * sizeof(float4), cudaMemcpyHostToDevice);
        if (t_max) cudaMemcpy(d_t, t_max, n * sizeof(float), cudaMemcpyHostToDevice);
        launch_time_of_impact(d_sa, d_wa, d_sb, d_wb, d_t, n, d_out, 0);
        std::vector<int2> res(n);
        if (cudaMemcpy(res.data(), d_out, n * sizeof(int2), cudaMemcpyDeviceToHost) != cudaSuccess) rc = B2G_ERR_CUDA;
        for (int i = 0; rc == B2G_OK && i < n; ++i) {
            out[i].state = res[i].x;
            memcpy(&out[i].t, &res[i].y, sizeof(float));
        }
    }
    cudaFree(d_sa);
    cudaFree(d_sb);
    cudaFree(d_wa);
    cudaFree(d_wb);
    cudaFree(d_t);
    cudaFree(d_out);
    return rc;
}

/* ---- allocation-free variant of b2g_collide_pairs ----
 * For callers that must not allocate (a frame loop with a fixed time budget, where freeing
 * device memory can wait for the whole device, or a program whose device memory belongs to
 * its own pool allocator). The kernel is k_collide_pairs; its staging buffers are one fixed
 * device array below instead of cudaMalloc'd memory, and host-side staging is a fixed array
 * too, so a call allocates nothing. */
namespace {
constexpr int kNoAllocMax = B2G_NOALLOC_MAX_PAIRS;
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
/* byte offsets of the sections inside the scratch array, each 256-byte aligned */
constexpr size_t kOffShapeA = 0;
constexpr size_t kOffShapeB = align256(kOffShapeA + sizeof(ShapeRec) * kNoAllocMax);
constexpr size_t kOffXfA = align256(kOffShapeB + sizeof(ShapeRec) * kNoAllocMax);
constexpr size_t kOffXfB = align256(kOffXfA + sizeof(float4) * kNoAllocMax);
constexpr size_t kOffKind = align256(kOffXfB + sizeof(float4) * kNoAllocMax);
constexpr size_t kOffGeo = align256(kOffKind + sizeof(int) * kNoAllocMax);
constexpr size_t kOffPts = align256(kOffGeo + sizeof(float4) * kNoAllocMax);
constexpr size_t kOffIds = align256(kOffPts + sizeof(float4) * kNoAllocMax);
constexpr size_t kNoAllocBytes = align256(kOffIds + sizeof(uint4) * kNoAllocMax);
}  // namespace

/* Device scratch of b2g_collide_pairs_noalloc (about 6 MB). Every GPU that loads this library
 * holds it until the process exits. Host code must not use the symbol as a pointer: its
 * device address is looked up per device with cudaGetSymbolAddress. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
alignas(256) unsigned char g_noalloc_host[kNoAllocBytes]; /* host staging, same layout */
std::mutex g_noalloc_lock;
constexpr int kNoAllocDevices = 64;
void* g_noalloc_dev[kNoAllocDevices] = {}; /* device address of the scratch, per device ordinal */
int noalloc_collide(int dev, const b2g_fixture_def* da, const float* xfa, const b2g_fixture_def* db, const float* xfb,
                    int32_t n, b2g_contact_info* out);
}  // namespace

extern "C" {

int b2g_collide_pairs_noalloc(const b2g_fixture_def* da, const float* xfa, const b2g_fixture_def* db,
                              const float* xfb, int32_t n, b2g_contact_info* out) {
    if (n < 0 || (n > 0 && (!da || !db || !xfa || !xfb || !out))) return B2G_ERR_INVALID_ARG;
    if (n > kNoAllocMax) return B2G_ERR_CAPACITY; /* more pairs than the fixed scratch holds */
    if (n == 0) return B2G_OK;
    std::lock_guard<std::mutex> guard(g_noalloc_lock);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocDevices) return B2G_ERR_CUDA;
    /* an error left pending on this thread by an earlier, unrelated call is not this call's */
    (void)cudaGetLastError();
    int rc = noalloc_collide(dev, da, xfa, db, xfb, n, out);
    /* a failed call forgets the device address, so a call after a device reset looks it up again */
    if (rc == B2G_ERR_CUDA) g_noalloc_dev[dev] = nullptr;
    return rc;
}

}  // extern "C"

namespace {

int noalloc_collide(int dev, const b2g_fixture_def* da, const float* xfa, const b2g_fixture_def* db, const float* xfb,
                    int32_t n, b2g_contact_info* out) {
    if (!g_noalloc_dev[dev]) {
        /* set-up on the first call on this device (the device is current here) */
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return B2G_ERR_CUDA;
        g_noalloc_dev[dev] = p;
    }
    unsigned char* d = (unsigned char*)g_noalloc_dev[dev];
    ShapeRec* ha = (ShapeRec*)(g_noalloc_host + kOffShapeA);
    ShapeRec* hb = (ShapeRec*)(g_noalloc_host + kOffShapeB);
    float4* hxa = (float4*)(g_noalloc_host + kOffXfA);
    float4* hxb = (float4*)(g_noalloc_host + kOffXfB);
    int* hkind = (int*)(g_noalloc_host + kOffKind);
    for (int i = 0; i < n; ++i) {
        build_shape(da[i], ha[i]);
        build_shape(db[i], hb[i]);
        const int ta = da[i].shape_type, tb = db[i].shape_type;
        if (ta == B2G_SHAPE_CIRCLE && tb == B2G_SHAPE_CIRCLE) hkind[i] = KIND_CIRCLES;
        else if (ta == B2G_SHAPE_POLYGON && tb == B2G_SHAPE_CIRCLE) hkind[i] = KIND_POLYGON_CIRCLE;
        else if (ta == B2G_SHAPE_POLYGON && tb == B2G_SHAPE_POLYGON) hkind[i] = KIND_POLYGONS;
        else if (ta == B2G_SHAPE_EDGE && tb == B2G_SHAPE_CIRCLE) hkind[i] = KIND_EDGE_CIRCLE;
        else if (ta == B2G_SHAPE_EDGE && tb == B2G_SHAPE_POLYGON) hkind[i] = KIND_EDGE_POLYGON;
        else return B2G_ERR_INVALID_ARG;
        const Rot qa = rot(xfa[3 * i + 2]), qb = rot(xfb[3 * i + 2]);
        hxa[i] = make_float4(xfa[3 * i], xfa[3 * i + 1], qa.s, qa.c);
        hxb[i] = make_float4(xfb[3 * i], xfb[3 * i + 1], qb.s, qb.c);
    }
    /* every element the kernel reads is written by these copies, and it writes every output
     * element it is asked for, so nothing left over from an earlier call is ever read */
    const size_t sizes[5] = {sizeof(ShapeRec), sizeof(ShapeRec), sizeof(float4), sizeof(float4), sizeof(int)};
    const size_t offs[5] = {kOffShapeA, kOffShapeB, kOffXfA, kOffXfB, kOffKind};
    for (int k = 0; k < 5; ++k)
        if (cudaMemcpy(d + offs[k], g_noalloc_host + offs[k], sizes[k] * n, cudaMemcpyHostToDevice) != cudaSuccess)
            return B2G_ERR_CUDA;
    launch_collide_pairs((const ShapeRec*)(d + kOffShapeA), (const float4*)(d + kOffXfA),
                         (const ShapeRec*)(d + kOffShapeB), (const float4*)(d + kOffXfB), (const int*)(d + kOffKind),
                         n, (float4*)(d + kOffGeo), (float4*)(d + kOffPts), (uint4*)(d + kOffIds), 0);
    if (cudaGetLastError() != cudaSuccess) return B2G_ERR_CUDA;
    const size_t osz[3] = {sizeof(float4), sizeof(float4), sizeof(uint4)};
    const size_t ooff[3] = {kOffGeo, kOffPts, kOffIds};
    for (int k = 0; k < 3; ++k)
        if (cudaMemcpy(g_noalloc_host + ooff[k], d + ooff[k], osz[k] * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            return B2G_ERR_CUDA;
    const float4* geo = (const float4*)(g_noalloc_host + kOffGeo);
    const float4* pts = (const float4*)(g_noalloc_host + kOffPts);
    const uint4* ids = (const uint4*)(g_noalloc_host + kOffIds);
    for (int i = 0; i < n; ++i) {
        b2g_contact_info& o = out[i];
        memset(&o, 0, sizeof(o));
        o.fixture_a = o.fixture_b = (uint32_t)i;
        o.manifold_type = (int)(ids[i].z & 0xffu);
        o.point_count = (int)((ids[i].z >> 8) & 0xffu);
        o.touching = o.point_count > 0;
        o.local_normal = b2g_vec2{geo[i].x, geo[i].y};
        o.local_point = b2g_vec2{geo[i].z, geo[i].w};
        o.point_local[0] = b2g_vec2{pts[i].x, pts[i].y};
        o.point_local[1] = b2g_vec2{pts[i].z, pts[i].w};
        o.point_id[0] = ids[i].x;
        o.point_id[1] = ids[i].y;
    }
    return B2G_OK;
}

}  // namespace

extern "C" {

/* B2island::report (private/dynamics/b2_island_private.rs:460-487) of the last step's discrete solve:
 * the constraint slots' fixture pairs, solved point counts and impulses after the velocity iterations
 * (the velocity-constraint arrays keep them until the next step's constraint initialisation) */
int b2g_get_post_solve(void* p, b2g_contact_impulse* out, int32_t cap, int32_t* n) {
    World* w = W(p);
    if (!w || !n || (!out && cap > 0)) return B2G_ERR_INVALID_ARG;
    *n = 0;
    if (!w->allocated || !w->device_authoritative) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int nc = 0;
    CUDA_OK(w, cudaMemcpy(&nc, w->d.cnt + CNT_CONS, sizeof(int), cudaMemcpyDeviceToHost));
    *n = nc;
    if (!out || cap < nc || nc == 0) return B2G_OK;
    std::vector<int2> fx(nc);
    std::vector<int4> idx(nc);
    std::vector<float4> imp(nc);
    CUDA_OK(w, cudaMemcpy(fx.data(), w->d.s_fix, nc * sizeof(int2), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(idx.data(), w->d.vc_idx, nc * sizeof(int4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(imp.data(), w->d.vc_imp, nc * sizeof(float4), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nc; ++i) {
        b2g_contact_impulse& r = out[i];
        memset(&r, 0, sizeof(r));
        r.fixture_a = (uint32_t)fx[i].x;
        r.fixture_b = (uint32_t)fx[i].y;
        r.count = idx[i].z;
        r.normal_impulses[0] = imp[i].x;
        r.tangent_impulses[0] = imp[i].y;
        if (r.count > 1) {
            r.normal_impulses[1] = imp[i].z;
            r.tangent_impulses[1] = imp[i].w;
        }
    }
    return B2G_OK;
}

int b2g_get_solver_order(void* p, uint32_t* out, int32_t cap, int32_t* n) {
    World* w = W(p);
    if (!w || !n) return B2G_ERR_INVALID_ARG;
    *n = 0;
    if (!w->allocated) return B2G_OK;
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    int nc = 0;
    CUDA_OK(w, cudaMemcpy(&nc, w->d.cnt + CNT_CONS, sizeof(int), cudaMemcpyDeviceToHost));
    *n = nc;
    if (!out || cap < nc || nc == 0) return B2G_OK;
    CUDA_OK(w, cudaMemcpy(out, w->d.s_fix, nc * sizeof(int2), cudaMemcpyDeviceToHost));
    return B2G_OK;
}

}  // extern "C"

/* ---- world queries ---- */

extern "C" {

int b2g_ray_cast_closest(void* p, const float* rays, const uint32_t* world_index, int32_t n, b2g_ray_hit* out) {
    World* w = W(p);
    if (!w || n < 0 || (n > 0 && (!rays || !out))) return B2G_ERR_INVALID_ARG;
    if (n == 0) return B2G_OK;
    if (!w->allocated || w->steps == 0) return fail(w, B2G_ERR_INVALID_ARG, "queries use the last step's hierarchy: step once first");
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    float4 *d_rays = nullptr, *d_a = nullptr, *d_b = nullptr;
    uint32_t* d_world = nullptr;
    cudaStream_t s = w->stream;
    cudaError_t e = cudaMalloc((void**)&d_rays, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_a, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_b, n * sizeof(float4));
    if (e == cudaSuccess && world_index) e = cudaMalloc((void**)&d_world, n * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rays, rays, n * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && world_index)
        e = cudaMemcpyAsync(d_world, world_index, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    std::vector<float4> a(n), b(n);
    if (e == cudaSuccess) {
        launch_ray_cast(w->d, d_rays, d_world, n, d_a, d_b, s);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(a.data(), d_a, n * sizeof(float4), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.data(), d_b, n * sizeof(float4), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_rays);
    cudaFree(d_a);
    cudaFree(d_b);
    if (d_world) cudaFree(d_world);
    if (e != cudaSuccess) return fail(w, B2G_ERR_CUDA, cudaGetErrorString(e));
    for (int i = 0; i < n; ++i) {
        int f;
        memcpy(&f, &a[i].x, 4);
        out[i].fixture = f;
        out[i].point = b2g_vec2{a[i].y, a[i].z};
        out[i].normal = b2g_vec2{b[i].x, b[i].y};
        out[i].fraction = b[i].z;
    }
    return check_status(w);
}

int b2g_query_aabb(void* p, const float* boxes, const uint32_t* world_index, int32_t n, uint32_t* out_pairs,
                   int32_t capacity, int32_t* out_count) {
    World* w = W(p);
    if (!w || n < 0 || !out_count || (n > 0 && !boxes) || capacity < 0 || (capacity > 0 && !out_pairs))
        return B2G_ERR_INVALID_ARG;
    *out_count = 0;
    if (n == 0) return B2G_OK;
    if (!w->allocated || w->steps == 0) return fail(w, B2G_ERR_INVALID_ARG, "queries use the last step's hierarchy: step once first");
    int rc = check_status(w);
    if (rc != B2G_OK) return rc;
    const int cap = capacity > 0 ? capacity : 1;
    float4* d_boxes = nullptr;
    uint32_t* d_world = nullptr;
    uint2* d_out = nullptr;
    int* d_count = nullptr;
    cudaStream_t s = w->stream;
    cudaError_t e = cudaMalloc((void**)&d_boxes, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_out, (size_t)cap * sizeof(uint2));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_count, sizeof(int));
    if (e == cudaSuccess && world_index) e = cudaMalloc((void**)&d_world, n * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_boxes, boxes, n * sizeof(float4), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && world_index)
        e = cudaMemcpyAsync(d_world, world_index, n * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_count, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        launch_query_aabb(w->d, d_boxes, d_world, n, d_out, cap, d_count, s);
        e = cudaGetLastError();
    }
    int total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, d_count, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    std::vector<uint2> pairs(std::min(total, cap > 0 ? cap : 0));
    if (e == cudaSuccess && !pairs.empty())
        e = cudaMemcpy(pairs.data(), d_out, pairs.size() * sizeof(uint2), cudaMemcpyDeviceToHost);
    cudaFree(d_boxes);
    cudaFree(d_out);
    cudaFree(d_count);
    if (d_world) cudaFree(d_world);
    if (e != cudaSuccess) return fail(w, B2G_ERR_CUDA, cudaGetErrorString(e));
    *out_count = total;
    if (total > capacity) return fail(w, B2G_ERR_CAPACITY, "more overlaps than capacity; *out_count holds the total");
    std::sort(pairs.begin(), pairs.end(),
              [](const uint2& x, const uint2& y) { return x.x != y.x ? x.x < y.x : x.y < y.y; });
    for (size_t i = 0; i < pairs.size(); ++i) {
        out_pairs[2 * i] = pairs[i].x;
        out_pairs[2 * i + 1] = pairs[i].y;
    }
    return check_status(w);
}

}  // extern "C"

/* ---- launch configuration and the autotuner ---- */

extern "C" {

int b2g_get_launch_config(void* p, b2g_launch_config* out) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    out->coop_blocks_per_sm = w->cfg.coop_per_sm;
    out->collide_block = w->cfg.collide_block;
    out->traverse_block = w->cfg.traverse_block;
    out->tuning_steps = w->tuning_steps;
    out->solver_block = w->cfg.solver_block;
    out->collide_group = w->cfg.collide_group;
    return B2G_OK;
}

int b2g_set_launch_config(void* p, const b2g_launch_config* c) {
    World* w = W(p);
    if (!w || !c) return B2G_ERR_INVALID_ARG;
    auto pow2 = [](int v, int lo, int hi) { return v >= lo && v <= hi && (v & (v - 1)) == 0; };
    const int sb = c->solver_block == 0 ? 256 : c->solver_block;
    if (c->coop_blocks_per_sm < 1 || c->coop_blocks_per_sm > 2 || !pow2(c->collide_block, 32, 256) ||
        !pow2(c->traverse_block, 32, 256) || (sb != 256 && sb != 512) || c->collide_group < 0 || c->collide_group > 32)
        return fail(w, B2G_ERR_INVALID_ARG,
                    "coop_blocks_per_sm in {1, 2}; block sizes powers of two in [32, 256]; solver_block 256 or 512; "
                    "collide_group in [0, 32]");
    w->cfg.coop_per_sm = c->coop_blocks_per_sm;
    w->cfg.collide_block = c->collide_block;
    w->cfg.traverse_block = c->traverse_block;
    w->cfg.solver_block = sb;
    w->cfg.collide_group = c->collide_group;
    w->cfg_set = true;
    apply_launch_config(w);
    drop_graphs(w);
    return B2G_OK;
}

}  // extern "C"

namespace {

/* device milliseconds of `steps` steps (CUDA events around each step, summed) */
int timed_steps(World* w, float dt, int vi, int pi, int steps, double* ms) {
    *ms = 0.0;
    for (int i = 0; i < steps; ++i) {
        int rc = step(w, dt, vi, pi);
        if (rc != B2G_OK) return rc;
        rc = check_status(w);
        if (rc != B2G_OK) return rc;
        float t = 0.0f;
        CUDA_OK(w, cudaEventElapsedTime(&t, w->timer.e[0], w->timer.e[5]));
        *ms += t;
    }
    return B2G_OK;
}

}  // namespace

extern "C" {

/* Coordinate search over the launch configuration on the world's own next steps: for each knob in
 * turn (persistent-kernel blocks per SM, narrowphase block, traversal block, solver block, the
 * narrowphase's polygon pairs per warp batch taken eight lanes to a pair) the candidates take
 * turns over up to four rounds, each turn two untimed steps (the step graph's captures for both
 * contact-buffer parities) and its share of `steps_per_candidate` timed steps; the fastest in
 * total is kept. With the part-local solve the
 * persistent kernels keep one block per SM.
 * The steps are real steps of the world (the configuration never changes results). The choice is
 * applied to the world and remembered for later worlds of the same size bucket in this process. */
int b2g_autotune(void* p, float dt, int32_t vi, int32_t pi, int32_t steps_per_candidate, b2g_launch_config* out) {
    World* w = W(p);
    if (!w || steps_per_candidate < 1 || !(dt > 0.0f)) return B2G_ERR_INVALID_ARG;
    if (w->tape && w->tape->recording) return fail(w, B2G_ERR_INVALID_ARG, "not while a tape is recording");
    if (w->h_flags.empty()) return fail(w, B2G_ERR_INVALID_ARG, "the world has no bodies");
    LaunchCfg best = w->cfg;
    w->cfg_set = true;
    const int coop[] = {1, 2}, collide[] = {64, 128, 256}, traverse[] = {64, 128, 256}, solver[] = {256, 512},
              group[] = {0, 8, 32};
    /* the part-local solve caches a part in its block's shared memory: one block per SM */
    const int ncoop = use_parts(w->d, w->num_sms, w->part_solve) ? 1 : 2;
    /* the world keeps evolving while candidates are timed, so the candidates take turns over
     * several rounds (a step each) instead of running one after another */
    const int rounds = std::max(1, std::min(steps_per_candidate / 2, 4));
    const int per_round = std::max(1, steps_per_candidate / rounds);
    int tuned = 0;
    auto field = [](LaunchCfg& c, int knob) -> int& {
        return knob == 0 ? c.coop_per_sm : knob == 1 ? c.collide_block : knob == 2 ? c.traverse_block
               : knob == 3 ? c.solver_block : c.collide_group;
    };
    for (int knob = 0; knob < 5; ++knob) {
        const int* cand = knob == 0 ? coop : knob == 1 ? collide : knob == 2 ? traverse : knob == 3 ? solver : group;
        /* 512 solver threads only with one block per SM (the registers of two would not fit) */
        const int nc = knob == 0 ? ncoop : knob == 3 ? (best.coop_per_sm == 1 ? 2 : 1) : 3;
        if (nc == 1) {
            field(best, knob) = cand[0];
            continue;
        }
        double total[3] = {0.0, 0.0, 0.0};
        for (int r = 0; r < rounds; ++r) {
            for (int i = 0; i < nc; ++i) {
                LaunchCfg c = best;
                field(c, knob) = cand[i];
                w->cfg = c;
                apply_launch_config(w);
                drop_graphs(w);
                double ms = 0.0;
                /* untimed: the captures of the step graph for both contact-buffer parities */
                int rc = timed_steps(w, dt, vi, pi, 2, &ms);
                if (rc == B2G_OK) rc = timed_steps(w, dt, vi, pi, per_round, &ms);
                tuned += 2 + per_round;
                if (rc != B2G_OK) return rc;
                total[i] += ms;
            }
        }
        int best_i = 0;
        for (int i = 1; i < nc; ++i)
            if (total[i] < total[best_i]) best_i = i;
        field(best, knob) = cand[best_i];
    }
    w->cfg = best;
    w->tuning_steps = tuned;
    apply_launch_config(w);
    drop_graphs(w);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        const int b = size_bucket(w);
        bool found = false;
        for (auto& e : g_tuned)
            if (e.first == b) {
                e.second = best;
                found = true;
            }
        if (!found) g_tuned.emplace_back(b, best);
    }
    return b2g_get_launch_config(p, out);
}

}  // extern "C"

/* ---- differentiable step: tape and backward ---- */

namespace {

template <class T>
int talloc(World* w, std::vector<void*>& mem, size_t& bytes, T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        w->err = std::string("cudaMalloc (tape): ") + cudaGetErrorString(e);
        return B2G_ERR_OUT_OF_MEMORY;
    }
    mem.push_back((void*)*p);
    bytes += n * sizeof(T);
    return B2G_OK;
}

int tape_final_index(const TapeHost* t) { return t->step_cap / t->ckpt_every + 1; }

int tape_status(World* w, TapeHost* t, long long* steps, long long* slots) {
    long long c[TAPE_CNT_SIZE] = {};
    CUDA_OK(w, cudaMemcpyAsync(c, t->d.cnt, sizeof(c), cudaMemcpyDeviceToHost, w->stream));
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    if (steps) *steps = c[TAPE_CNT_STEPS];
    if (slots) *slots = c[TAPE_CNT_SLOTS];
    if (c[TAPE_CNT_STATUS] != 0) {
        t->valid = false;
        return fail(w, B2G_ERR_CAPACITY, "the tape overflowed: raise max_steps / max_slots in b2g_tape_begin");
    }
    return B2G_OK;
}

/* work buffers for segments of ckpt_every steps with up to `slots` constraints */
int tape_work(World* w, TapeHost* t, int slots, int vi, int pi) {
    if (slots < 1) slots = 1;
    if (vi < 1) vi = 1;
    if (pi < 1) pi = 1;
    if (!t->work_mem.empty() && slots <= t->work_slots && vi <= t->work_vi && pi <= t->work_pi) return B2G_OK;
    tape_free_work(t);
    AdjWork& a = t->work;
    a = AdjWork{};
    const size_t nb = (size_t)t->n_bodies, seg = (size_t)t->ckpt_every, ns = (size_t)slots;
    std::vector<void*>& m = t->work_mem;
    size_t& by = t->work_bytes;
    int rc = B2G_OK;
    auto A = [&](auto** ptr, size_t n) {
        if (rc == B2G_OK) rc = talloc(w, m, by, ptr, n);
    };
    A(&a.cur_pos, nb);
    A(&a.cur_vel, nb);
    A(&a.ws_pos, seg * nb);
    A(&a.ws_vel1, seg * nb);
    A(&a.ws_vel2, seg * nb);
    A(&a.vc, ns);
    A(&a.imp, ns);
    A(&a.wv, seg * vi * ns * 3);
    A(&a.ww, seg * ns * 2);
    A(&a.wp, seg * pi * ns * 2);
    A(&a.g_pos, nb);
    A(&a.g_vel, nb);
    A(&a.gvc, ns);
    A(&a.g_imp, ns);
    A(&a.g_end[0], ns);
    A(&a.g_end[1], ns);
    A(&a.cnt, (size_t)CNT_SIZE);
    A(&a.mismatch, (size_t)1);
    if (rc != B2G_OK) {
        tape_free_work(t);
        return rc;
    }
    t->work_slots = slots;
    t->work_vi = vi;
    t->work_pi = pi;
    a.max_slots = slots;
    a.max_vi = vi;
    a.max_pi = pi;
    return B2G_OK;
}

}  // namespace

extern "C" {

int b2g_tape_begin(void* p, int32_t max_steps, int32_t every, int64_t max_slots) {
    World* w = W(p);
    if (!w || max_steps <= 0) return B2G_ERR_INVALID_ARG;
    if (w->h_flags.empty()) return fail(w, B2G_ERR_INVALID_ARG, "the world has no bodies");
    if (w->allow_sleep)
        return fail(w, B2G_ERR_UNSUPPORTED, "the tape needs sleeping off: call b2g_set_allow_sleeping(world, 0)");
    if (!w->joints.empty()) return fail(w, B2G_ERR_UNSUPPORTED, "the tape does not record joints");
    int rc = prepare(w);
    if (rc != B2G_OK) return rc;
    tape_free(w);
    TapeHost* t = new TapeHost;
    t->ckpt_every = every > 0 ? every : 16;
    t->step_cap = max_steps;
    t->slot_cap = max_slots > 0 ? (long long)max_slots : (long long)max_steps * (4LL * w->d.n_fixtures + 1024);
    t->n_bodies = w->d.n_bodies;
    const size_t nck = (size_t)(max_steps / t->ckpt_every + 2) * t->n_bodies;
    TapeDev& d = t->d;
    auto A = [&](auto** ptr, size_t n) {
        if (rc == B2G_OK) rc = talloc(w, t->mem, t->bytes, ptr, n);
    };
    A(&d.slots, (size_t)t->slot_cap);
    A(&d.steps, (size_t)max_steps);
    A(&d.col_off, (size_t)max_steps * (kMaxColours + 1));
    /* the part-local solve has at most one part per SM, each with a row of its colour offsets */
    d.max_parts = std::max(1, std::min(w->num_sms, kMaxParts));
    d.pool_cap = (long long)max_steps * d.max_parts * 20;
    A(&d.part_np, (size_t)max_steps);
    A(&d.part_row, (size_t)max_steps * d.max_parts);
    A(&d.part_pool, (size_t)d.pool_cap);
    A(&d.cmap[0], (size_t)w->d.contact_cap);
    A(&d.cmap[1], (size_t)w->d.contact_cap);
    A(&d.ckpt_pos, nck);
    A(&d.ckpt_vel, nck);
    A(&d.cnt, (size_t)TAPE_CNT_SIZE);
    if (rc != B2G_OK) {
        w->tape = t;
        tape_free(w);
        return rc;
    }
    d.slot_cap = t->slot_cap;
    d.step_cap = max_steps;
    d.ckpt_every = t->ckpt_every;
    d.n_bodies = t->n_bodies;
    cudaMemsetAsync(d.cnt, 0, TAPE_CNT_SIZE * sizeof(long long), w->stream);
    cudaMemsetAsync(d.cmap[0], 0, (size_t)w->d.contact_cap * sizeof(unsigned long long), w->stream);
    cudaMemsetAsync(d.cmap[1], 0, (size_t)w->d.contact_cap * sizeof(unsigned long long), w->stream);
    CUDA_OK(w, cudaGetLastError());
    t->recording = true;
    w->tape = t;
    drop_graphs(w);  /* the step graphs gain the recording kernels */
    return B2G_OK;
}

int b2g_tape_end(void* p) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    TapeHost* t = w->tape;
    if (!t || !t->recording) return fail(w, B2G_ERR_INVALID_ARG, "no tape is recording");
    launch_tape_snapshot(w->d, t->d, tape_final_index(t), w->stream);
    t->recording = false;
    drop_graphs(w);
    long long steps = 0;
    int rc = tape_status(w, t, &steps, nullptr);
    if (rc != B2G_OK) return rc;
    if (steps != t->steps) {
        t->valid = false;
        return fail(w, B2G_ERR_CUDA, "taped step count differs from the steps issued");
    }
    return check_status(w);
}

int b2g_tape_info_get(void* p, b2g_tape_info* out) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    *out = b2g_tape_info{};
    TapeHost* t = w->tape;
    if (!t) return B2G_OK;
    long long steps = 0, slots = 0;
    int rc = tape_status(w, t, &steps, &slots);
    out->recording = t->recording ? 1 : 0;
    out->steps = (int32_t)steps;
    out->slots = slots;
    out->checkpoint_interval = t->ckpt_every;
    out->valid = (t->valid && rc == B2G_OK) ? 1 : 0;
    out->device_bytes = (int64_t)(t->bytes + t->work_bytes);
    out->replay_mismatches = t->mismatches;
    return B2G_OK;
}

int b2g_tape_get_step(void* p, int32_t step, b2g_tape_step* out_step, int32_t* out_col, b2g_tape_slot* out_slots,
                      int32_t cap) {
    World* w = W(p);
    if (!w) return B2G_ERR_INVALID_ARG;
    TapeHost* t = w->tape;
    if (!t) return fail(w, B2G_ERR_INVALID_ARG, "no tape");
    long long steps = 0;
    int rc = tape_status(w, t, &steps, nullptr);
    if (rc != B2G_OK) return rc;
    if (step < 0 || step >= steps) return fail(w, B2G_ERR_INVALID_ARG, "step out of range");
    TapeStep st;
    CUDA_OK(w, cudaMemcpy(&st, t->d.steps + step, sizeof(st), cudaMemcpyDeviceToHost));
    /* The solve order as one list of colour groups (slots of a group are independent): each
     * part's interior colours, then the boundary colours. */
    std::vector<int> groups;
    int np = 0;
    CUDA_OK(w, cudaMemcpy(&np, t->d.part_np + step, sizeof(int), cudaMemcpyDeviceToHost));
    if (np > 0) {
        std::vector<int> rows((size_t)np);
        CUDA_OK(w, cudaMemcpy(rows.data(), t->d.part_row + (size_t)step * t->d.max_parts, np * sizeof(int),
                              cudaMemcpyDeviceToHost));
        int last_n = 0;
        CUDA_OK(w, cudaMemcpy(&last_n, t->d.part_pool + rows[np - 1], sizeof(int), cudaMemcpyDeviceToHost));
        const int beg = rows[0], end = rows[np - 1] + last_n + 2;
        std::vector<int> seg((size_t)(end - beg));
        CUDA_OK(w, cudaMemcpy(seg.data(), t->d.part_pool + beg, seg.size() * sizeof(int), cudaMemcpyDeviceToHost));
        for (int q = 0; q < np; ++q) {
            const int* row = seg.data() + (rows[q] - beg);
            for (int c = 0; c < row[0]; ++c) groups.push_back(row[1 + c]);
        }
    }
    std::vector<int> co((size_t)st.ncol + 1);
    CUDA_OK(w, cudaMemcpy(co.data(), t->d.col_off + (size_t)step * (kMaxColours + 1), co.size() * sizeof(int),
                          cudaMemcpyDeviceToHost));
    for (int c = 0; c < st.ncol; ++c) groups.push_back(co[c]);
    const int ngroups = (int)groups.size();
    groups.push_back(st.nslots);
    st.ncol = ngroups;
    if (out_step) memcpy(out_step, &st, sizeof(st));
    if (out_col) memcpy(out_col, groups.data(), groups.size() * sizeof(int));
    if (out_slots) {
        if (cap < st.nslots) return fail(w, B2G_ERR_CAPACITY, "slot buffer too small");
        if (st.nslots > 0)
            CUDA_OK(w, cudaMemcpy(out_slots, t->d.slots + st.slot_off, (size_t)st.nslots * sizeof(TapeSlot),
                                  cudaMemcpyDeviceToHost));
    }
    return B2G_OK;
}

int b2g_tape_get_checkpoint(void* p, int32_t index, float* out, uint32_t count) {
    World* w = W(p);
    if (!w || !out) return B2G_ERR_INVALID_ARG;
    TapeHost* t = w->tape;
    if (!t) return fail(w, B2G_ERR_INVALID_ARG, "no tape");
    if (count > (uint32_t)t->n_bodies) return fail(w, B2G_ERR_INVALID_ARG, "more bodies than the tape holds");
    if (index == -1) {
        if (t->recording) return fail(w, B2G_ERR_INVALID_ARG, "the final state exists after b2g_tape_end");
        index = tape_final_index(t);
    } else if (index < 0 || index > (t->steps - 1) / t->ckpt_every) {
        return fail(w, B2G_ERR_INVALID_ARG, "checkpoint index out of range");
    }
    std::vector<float4> pos(count), vel(count);
    const size_t o = (size_t)index * t->n_bodies;
    CUDA_OK(w, cudaStreamSynchronize(w->stream));
    CUDA_OK(w, cudaMemcpy(pos.data(), t->d.ckpt_pos + o, count * sizeof(float4), cudaMemcpyDeviceToHost));
    CUDA_OK(w, cudaMemcpy(vel.data(), t->d.ckpt_vel + o, count * sizeof(float4), cudaMemcpyDeviceToHost));
    for (uint32_t b = 0; b < count; ++b) {
        memcpy(out + 8 * (size_t)b, &pos[b], sizeof(float4));
        memcpy(out + 8 * (size_t)b + 4, &vel[b], sizeof(float4));
    }
    return B2G_OK;
}

/* Reverse pass: segments of ckpt_every steps from the last to the first; each replays its
 * steps from the segment's checkpoint, then runs the adjoint backwards through them. */
int b2g_backward(void* p, const b2g_body_state* d_final, b2g_body_state* d_initial) {
    World* w = W(p);
    if (!w || !d_final || !d_initial) return B2G_ERR_INVALID_ARG;
    TapeHost* t = w->tape;
    if (!t) return fail(w, B2G_ERR_INVALID_ARG, "no tape: call b2g_tape_begin, step, b2g_tape_end");
    if (t->recording) return fail(w, B2G_ERR_INVALID_ARG, "call b2g_tape_end before b2g_backward");
    if (!t->valid)
        return fail(w, B2G_ERR_INVALID_ARG,
                    "the tape is invalid: bodies were edited or created, or a dt = 0 step ran, while recording");
    long long nsteps = 0;
    int rc = tape_status(w, t, &nsteps, nullptr);
    if (rc != B2G_OK) return rc;
    const int T = (int)nsteps;
    const int nb = t->n_bodies;
    std::vector<TapeStep> st(std::max(T, 1));
    if (T > 0) CUDA_OK(w, cudaMemcpy(st.data(), t->d.steps, T * sizeof(TapeStep), cudaMemcpyDeviceToHost));
    int max_slots = 1, max_vi = 1, max_pi = 1;
    for (int i = 0; i < T; ++i) {
        max_slots = std::max(max_slots, st[i].nslots);
        max_vi = std::max(max_vi, st[i].vi);
        max_pi = std::max(max_pi, st[i].pi);
    }
    rc = tape_work(w, t, max_slots, max_vi, max_pi);
    if (rc != B2G_OK) return rc;
    AdjWork a = t->work;
    a.t = t->d;
    a.b_mass = w->d.b_mass;
    a.b_damp = w->d.b_damp;
    a.b_flags = w->d.b_flags;
    a.b_lc = w->d.b_lc;
    a.nb = nb;
    /* dL/d(final solver state): the origin p = c - R(a) lc moves with c and a */
    std::vector<float4> fpos(nb), gpos(nb), gvel(nb);
    const size_t fo = (size_t)tape_final_index(t) * nb;
    CUDA_OK(w, cudaMemcpy(fpos.data(), t->d.ckpt_pos + fo, nb * sizeof(float4), cudaMemcpyDeviceToHost));
    for (int b = 0; b < nb; ++b) {
        const b2g_body_state& g = d_final[b];
        const double an = fpos[b].z, sn = std::sin(an), cs = std::cos(an);
        const double lx = w->h_lc[b].x, ly = w->h_lc[b].y;
        const double drx = -sn * lx - cs * ly, dry = cs * lx - sn * ly;
        const double gcx = (double)g.position.x + g.world_center.x, gcy = (double)g.position.y + g.world_center.y;
        const double ga = (double)g.angle - ((double)g.position.x * drx + (double)g.position.y * dry);
        gpos[b] = make_float4((float)gcx, (float)gcy, (float)ga, 0.0f);
        gvel[b] = make_float4(g.linear_velocity.x, g.linear_velocity.y, g.angular_velocity, 0.0f);
    }
    cudaStream_t s = w->stream;
    CUDA_OK(w, cudaMemcpyAsync(a.g_pos, gpos.data(), nb * sizeof(float4), cudaMemcpyHostToDevice, s));
    CUDA_OK(w, cudaMemcpyAsync(a.g_vel, gvel.data(), nb * sizeof(float4), cudaMemcpyHostToDevice, s));
    CUDA_OK(w, cudaMemsetAsync(a.g_end[0], 0, (size_t)a.max_slots * sizeof(float4), s));
    CUDA_OK(w, cudaMemsetAsync(a.g_end[1], 0, (size_t)a.max_slots * sizeof(float4), s));
    CUDA_OK(w, cudaMemsetAsync(a.cnt, 0, CNT_SIZE * sizeof(int), s));
    CUDA_OK(w, cudaMemsetAsync(a.mismatch, 0, sizeof(unsigned), s));
    const int every = t->ckpt_every;
    const int nseg = (T + every - 1) / every;
    for (int g = nseg - 1; g >= 0; --g) {
        a.t0 = g * every;
        a.t1 = std::min(T, a.t0 + every);
        const size_t eo = (size_t)(a.t1 == T ? tape_final_index(t) : a.t1 / every) * nb;
        a.end_pos = t->d.ckpt_pos + eo;
        a.end_vel = t->d.ckpt_vel + eo;
        const int e = launch_adjoint_segment(a, s, w->num_sms);
        if (e != 0) return fail(w, B2G_ERR_CUDA, cudaGetErrorString((cudaError_t)e));
    }
    int dcnt[CNT_SIZE] = {};
    unsigned mism = 0;
    CUDA_OK(w, cudaMemcpyAsync(gpos.data(), a.g_pos, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_OK(w, cudaMemcpyAsync(gvel.data(), a.g_vel, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_OK(w, cudaMemcpyAsync(fpos.data(), t->d.ckpt_pos, nb * sizeof(float4), cudaMemcpyDeviceToHost, s));
    CUDA_OK(w, cudaMemcpyAsync(dcnt, a.cnt, sizeof(dcnt), cudaMemcpyDeviceToHost, s));
    CUDA_OK(w, cudaMemcpyAsync(&mism, a.mismatch, sizeof(mism), cudaMemcpyDeviceToHost, s));
    CUDA_OK(w, cudaStreamSynchronize(s));
    if (dcnt[CNT_STATUS] & ST_BARRIER_TIMEOUT)
        return fail(w, B2G_ERR_TIMEOUT, "a grid barrier of the backward pass timed out");
    t->mismatches = mism;
    /* dL/d(initial origin, angle): c0 = p0 + R(a0) lc */
    for (int b = 0; b < nb; ++b) {
        const double an = fpos[b].z, sn = std::sin(an), cs = std::cos(an);
        const double lx = w->h_lc[b].x, ly = w->h_lc[b].y;
        const double drx = -sn * lx - cs * ly, dry = cs * lx - sn * ly;
        b2g_body_state& o = d_initial[b];
        o.position = b2g_vec2{gpos[b].x, gpos[b].y};
        o.angle = (float)((double)gpos[b].z + (double)gpos[b].x * drx + (double)gpos[b].y * dry);
        o.linear_velocity = b2g_vec2{gvel[b].x, gvel[b].y};
        o.angular_velocity = gvel[b].z;
        o.world_center = b2g_vec2{gpos[b].x, gpos[b].y};
    }
    return B2G_OK;
}

}  // extern "C"
