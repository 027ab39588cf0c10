/*
 * b2g_contact.cuh — B2contact::update on the device, shared by the narrowphase pass
 * (k_collide.cu) and the continuous-physics pass (k_continuous.cu).
 *
 * Reference: b2_contact_update, src/private/dynamics/b2_contact.rs:103-218; set_awake,
 * src/b2_body.rs:783-801.
 */
#ifndef B2G_CONTACT_CUH
#define B2G_CONTACT_CUH

#include "b2g_internal.h"

namespace b2g {
namespace {

/* set_awake(true): a static body is left alone; any other is flagged awake with its sleep time
 * reset (the reference resets it whether or not the body slept) */
__device__ __forceinline__ void wake_body(const DevWorld& w, int b) {
    const uint32_t f = w.b_flags[b];
    if ((f & BF_TYPE_MASK) == BODY_STATIC) return;
    if (!(f & BF_AWAKE)) atomicOr(&w.b_flags[b], BF_AWAKE);
    w.b_vel[b].w = 0.0f;  /* sleep_time = 0 */
}

/* set_awake(true) recorded for the collide pass of a world whose bodies may sleep: the reference's
 * collide sees, at each contact of its list, the bodies woken by the contacts before it, so a wake
 * is noted with the waking contact's place in the (key-sorted) table and applied when the pass ends */
__device__ __forceinline__ void wake_body_at(const DevWorld& w, int b, int at) {
    if ((w.b_flags[b] & BF_TYPE_MASK) == BODY_STATIC) return;
    atomicMin(&w.b_wake[b], at);
}

__device__ __forceinline__ void push_event(const DevWorld& w, int kind, int fa, int fb) {
    int slot = atomicAdd(&w.cnt[CNT_EVENTS], 1);
    if (slot < w.event_cap) w.events[slot] = make_int4(kind, fa, fb, 0);
    else atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_EVENT_OVERFLOW);
}

__device__ __forceinline__ Xf load_xf(const DevWorld& w, int b) {
    float4 x = w.b_xf[b];
    Xf r;
    r.p = mk(x.x, x.y);
    r.q.s = x.z;
    r.q.c = x.w;
    return r;
}

/* fixture f's rows of the structure-of-arrays shape tables (h: its header, f_hdr[f]) */
__device__ __forceinline__ ShapeRows shape_rows(const DevWorld& w, int f, float4 h) {
    ShapeRows r;
    r.vn = w.f_vn + (size_t)f * kMaxPolygonVertices;
    r.centroid = mk(h.x, h.y);
    r.radius = h.z;
    r.meta = __float_as_int(h.w);
    return r;
}
__device__ __forceinline__ ShapeRows shape_rows(const DevWorld& w, int f) { return shape_rows(w, f, w.f_hdr[f]); }

/* the manifold a routine starts from: no points, zero geometry and ids */
__device__ __forceinline__ void manifold_init(Manifold& m) {
    m.type = MANIFOLD_CIRCLES;
    m.count = 0;
    m.ln = mk(0.0f, 0.0f);
    m.lp = mk(0.0f, 0.0f);
    m.p[0] = m.p[1] = mk(0.0f, 0.0f);
    m.id[0] = m.id[1] = 0u;
}

/* The part of B2contact::update (private/dynamics/b2_contact.rs:103-218) after the manifold m of
 * contact i has been evaluated (flags: its current flags; fx, bd: its fixtures and bodies; ids,
 * oldimp: its manifold ids word and impulses): re-enable it, carry impulses from old points with the
 * same feature id, update the touching flag, wake both bodies when it changes (at once, or noted at
 * table place wake_at >= 0: wake_body_at) and record begin/end events. set_flags are or-ed into the
 * stored flags. The ids and impulses are stored only where they changed (a contact that stays apart
 * keeps both). Returns whether the contact touches. */
__device__ __forceinline__ bool contact_finish(const DevWorld& w, bool record_events, int i, uint32_t flags, int2 fx,
                                               int2 bd, uint4 ids, float4 oldimp, const Manifold& m, int wake_at,
                                               uint32_t set_flags) {
    const bool was_touching = (flags & CF_TOUCHING) != 0;
    const int old_count = (int)((ids.z >> 8) & 0xffu);
    flags |= CF_ENABLED | set_flags;
    float ni[2] = {0.0f, 0.0f}, ti[2] = {0.0f, 0.0f};
    for (int p = 0; p < m.count; ++p) {
        if (old_count > 0 && ids.x == m.id[p]) {
            ni[p] = oldimp.x;
            ti[p] = oldimp.y;
        } else if (old_count > 1 && ids.y == m.id[p]) {
            ni[p] = oldimp.z;
            ti[p] = oldimp.w;
        }
    }
    const bool touching = m.count > 0;
    w.c.mgeo[i] = make_float4(m.ln.x, m.ln.y, m.lp.x, m.lp.y);
    w.c.mpts[i] = make_float4(m.p[0].x, m.p[0].y, m.p[1].x, m.p[1].y);
    const float4 imp = make_float4(ni[0], ti[0], ni[1], ti[1]);
    if (__float_as_uint(imp.x) != __float_as_uint(oldimp.x) || __float_as_uint(imp.y) != __float_as_uint(oldimp.y) ||
        __float_as_uint(imp.z) != __float_as_uint(oldimp.z) || __float_as_uint(imp.w) != __float_as_uint(oldimp.w))
        w.c.mimp[i] = imp;
    const uint4 nids = make_uint4(m.id[0], m.id[1], (uint32_t)m.type | ((uint32_t)m.count << 8), ids.w);
    if (nids.x != ids.x || nids.y != ids.y || nids.z != ids.z) w.c.mids[i] = nids;
    if (touching != was_touching) {
        if (wake_at < 0) {
            wake_body(w, bd.x);
            wake_body(w, bd.y);
        } else {
            wake_body_at(w, bd.x, wake_at);
            wake_body_at(w, bd.y, wake_at);
        }
    }
    w.c.flags[i] = touching ? (flags | CF_TOUCHING) : (flags & ~CF_TOUCHING);
    if (record_events) {
        if (!was_touching && touching) push_event(w, 0, fx.x, fx.y);
        if (was_touching && !touching) push_event(w, 1, fx.x, fx.y);
    }
    return touching;
}

/* B2contact::update of contact i, one thread: the manifold evaluated by the routine of the
 * contact's kind on the bodies' transforms, then contact_finish. A sensor keeps no points (sensor
 * overlap tests, GJK, are outside the GPU path: sensors never touch). Returns whether the contact
 * touches. */
__device__ __forceinline__ bool contact_update(const DevWorld& w, bool record_events, int i, uint32_t flags, int2 fx,
                                               int2 bd, uint4 ids, int wake_at = -1, uint32_t set_flags = 0u) {
    if (flags & CF_SENSOR) {
        const bool was_touching = (flags & CF_TOUCHING) != 0;
        w.c.mids[i] = make_uint4(ids.x, ids.y, ids.z & 0xffu, ids.w);
        w.c.flags[i] = (flags | CF_ENABLED | set_flags) & ~CF_TOUCHING;
        if (record_events && was_touching) push_event(w, 1, fx.x, fx.y);
        return false;
    }
    const int kind = (int)((flags >> CF_KIND_SHIFT) & 7u);
    Manifold m;
    manifold_init(m);
    evaluate(kind, m, shape_rows(w, fx.x), load_xf(w, bd.x), shape_rows(w, fx.y), load_xf(w, bd.y));
    return contact_finish(w, record_events, i, flags, fx, bd, ids, w.c.mimp[i], m, wake_at, set_flags);
}

/* register table of b2_contact_registers.rs:67-103: +1 keep order, -1 swap, 0 no contact */
__device__ __forceinline__ int register_kind(int ta, int tb) {
    const int table[9] = {+1, -1, -1, +1, 0, +1, +1, -1, +1};
    return table[ta * 3 + tb];
}
__device__ __forceinline__ int contact_kind(int ta, int tb) {
    if (ta == SHAPE_CIRCLE) return KIND_CIRCLES;
    if (ta == SHAPE_POLYGON) return tb == SHAPE_CIRCLE ? KIND_POLYGON_CIRCLE : KIND_POLYGONS;
    return tb == SHAPE_CIRCLE ? KIND_EDGE_CIRCLE : KIND_EDGE_POLYGON;
}

/* the joint part of B2body::should_collide (private/dynamics/b2_body.rs:399-413): no joint between
 * the two bodies keeps them from colliding */
__device__ __forceinline__ bool joint_allows(const DevWorld& w, int a, int b) {
    for (int e = w.b_jnt_off[a]; e < w.b_jnt_off[a + 1]; ++e) {
        const int j = w.b_jnt[e];
        const int2 jb = w.j_body[j];
        const int other = jb.x == a ? jb.y : jb.x;
        if (other == b && !(__float_as_uint(w.j_par[j].y) & JF_COLLIDE)) return false;
    }
    return true;
}

/* b2_contact_manager_add_pair's rejections after the existing-contact check
 * (private/dynamics/b2_contact_manager.rs:178-302): same body, no dynamic body, a joint that keeps
 * the bodies apart, the default filter (private/dynamics/b2_world_callbacks.rs:6-18; skipped when the
 * host's contact filter replaces it and filters the new pairs itself), no manifold routine for the
 * two shape types (b2_contact_registers.rs:67-103). f is the fixture with the smaller proxy id. On
 * acceptance (fa, fb) is the contact's fixture pair, fixture A the one of the primary shape type. */
/* the default contact filter, should_collide of private/dynamics/b2_world_callbacks.rs:6-18, on the
 * fixtures' current filter data (f_filter = category | mask << 16, f_group = group (int16) | sensor << 16) */
__device__ __forceinline__ bool filter_allows(const DevWorld& w, int fa, int fb) {
    const uint32_t xa = w.f_filter[fa], xb = w.f_filter[fb];
    const int grp_a = (int)(int16_t)(w.f_group[fa] & 0xffffu);
    const int grp_b = (int)(int16_t)(w.f_group[fb] & 0xffffu);
    if (grp_a == grp_b && grp_a != 0) return grp_a > 0;
    return ((xa >> 16) & (xb & 0xffffu)) != 0u && ((xa & 0xffffu) & (xb >> 16)) != 0u;
}

/* self.should_collide(other), B2body::should_collide (private/dynamics/b2_body.rs:391-416): one body
 * dynamic, no joint of self's keeping it from other */
__device__ __forceinline__ bool bodies_collide(const DevWorld& w, int self, int other) {
    const uint32_t fs = w.b_flags[self], fo = w.b_flags[other];
    if ((fs & BF_TYPE_MASK) != BODY_DYNAMIC && (fo & BF_TYPE_MASK) != BODY_DYNAMIC) return false;
    return joint_allows(w, self, other);
}

__device__ __forceinline__ bool pair_accept(const DevWorld& w, int f, int g, int& fa, int& fb, bool default_filter = true) {
    fa = f;
    fb = g;
    const int ba = w.f_body[fa], bb = w.f_body[fb];
    if (ba == bb) return false;
    if (!bodies_collide(w, bb, ba)) return false;
    if (default_filter && !filter_allows(w, fa, fb)) return false;
    const int reg = register_kind(shape_type(w.f_shape[fa]), shape_type(w.f_shape[fb]));
    if (reg == 0) return false;
    if (reg < 0) {
        fa = g;
        fb = f;
    }
    return true;
}

/* b2_contact_create + B2contact::new (private/dynamics/b2_contact.rs:11-60) into slot pos of d:
 * enabled, not touching, an empty manifold, the mixing laws of src/b2_contact.rs:29-46 */
__device__ __forceinline__ void init_contact(const DevWorld& w, const Contacts& d, int pos, unsigned long long key,
                                             int2 fx) {
    const float4 ma = w.f_mat[fx.x], mb = w.f_mat[fx.y];
    const int kind = contact_kind(shape_type(w.f_shape[fx.x]), shape_type(w.f_shape[fx.y]));
    const bool sensor = ((w.f_group[fx.x] | w.f_group[fx.y]) & 0x10000u) != 0u;
    d.key[pos] = key;
    d.fix[pos] = fx;
    d.body[pos] = make_int2(w.f_body[fx.x], w.f_body[fx.y]);
    d.flags[pos] = CF_ENABLED | (sensor ? CF_SENSOR : 0u) | ((uint32_t)kind << CF_KIND_SHIFT);
    const float friction = fsqrt(ma.x * mb.x);
    const float restitution = ma.y > mb.y ? ma.y : mb.y;
    const float threshold = ma.z < mb.z ? ma.z : mb.z;
    d.mat[pos] = make_float4(friction, restitution, threshold, 0.0f);
    d.mgeo[pos] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d.mpts[pos] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d.mimp[pos] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    d.mids[pos] = make_uint4(0u, 0u, 0u, 0u);
}

__device__ __forceinline__ void copy_contact(const Contacts& s, int i, const Contacts& d, int o) {
    d.key[o] = s.key[i];
    d.fix[o] = s.fix[i];
    d.body[o] = s.body[i];
    d.flags[o] = s.flags[i];
    d.mat[o] = s.mat[i];
    d.mgeo[o] = s.mgeo[i];
    d.mpts[o] = s.mpts[i];
    d.mimp[o] = s.mimp[i];
    d.mids[o] = s.mids[i];
}

}  // namespace
}  // namespace b2g
#endif
