/*
 * k_collide.cu — the narrowphase pass of a step (B2contactManager::collide).
 *
 * Reference: b2_contact_manager_collide, src/private/dynamics/b2_contact_manager.rs:83-171,
 * and b2_contact_update, src/private/dynamics/b2_contact.rs:103-218.
 *
 * Each warp takes batches of 32 consecutive contacts of the (key-sorted) contact table, one lane per
 * contact for the bookkeeping:
 *   - skip when neither body is awake and non-static. The reference's loop sees, at each contact
 *     of its list, the bodies woken by the updates before it; where bodies may sleep, a wake is
 *     noted with the waking contact's table place, a contact counts a body woken at an earlier
 *     place as awake, and the contacts a wake makes active are collided in further rounds until
 *     none is left (the table's key order standing for the list order); the wakes are applied
 *     after the pass;
 *   - if the two fat AABBs stopped overlapping, flag the contact dead (the next merge
 *     drops it), emit an end event if it was touching, and wake both bodies if its
 *     manifold had points (B2contact::destroy);
 *   - otherwise evaluate the manifold with the routine of the contact's kind, carry
 *     normal/tangent impulses from old points with the same feature id, update the
 *     touching flag, wake both bodies when it changes, and emit begin/end events.
 * Then the batch's manifolds: one lane per pair, or, for a batch with at most cfg_collide_group
 * polygon pairs, those pairs four at a time, eight lanes to a pair (collide_polygons_group: lane k
 * holds row k of both polygons; the default, 0, keeps one lane per pair, which measured at least as
 * fast on GB300). Shapes are read from the structure-of-arrays rows (f_vn, f_hdr): a polygon's used
 * rows are one contiguous 16·V-byte read.
 * Algorithmic bytes per evaluated contact: ~116 B of contact/manifold state + the two shapes' rows
 * (16 B header + 16 B per vertex row) + two body transforms.
 */
#include "b2g_contact.cuh"
#include "b2g_sync.cuh"

namespace b2g {

namespace {

/* Body b counts as active for contact i (table place i): awake and not static. With deferred
 * wakes (the world's bodies may sleep), "awake" is awake when the pass began, or woken by the
 * update of a contact earlier in the table than i. */
__device__ __forceinline__ bool active_for(const DevWorld& w, int b, uint32_t f, int i, bool deferred) {
    if ((f & BF_TYPE_MASK) == BODY_STATIC) return false;
    if (f & BF_AWAKE) return true;
    return deferred && ((volatile int*)w.b_wake)[b] < i;
}

enum { HEAD_SKIPPED = 0, HEAD_DONE = 1, HEAD_EVALUATE = 2 };

/* a contact whose manifold is to be evaluated: its flags, fixtures, bodies and manifold ids */
struct Head {
    uint32_t flags;
    int2 fx, bd;
    uint4 ids;
};

/* b2_contact_manager_collide for contact i up to the manifold's evaluation: HEAD_SKIPPED if it was
 * skipped as inactive, HEAD_DONE if nothing is left to do (dead, destroyed now, or a sensor, whose
 * update needs no shapes), HEAD_EVALUATE with h filled if its manifold is to be evaluated */
__device__ __forceinline__ int collide_head(const DevWorld& w, const StepParams& sp, int i, bool deferred, Head& h) {
    /* the contact's own fields go out together, then its bodies' flags and its fixtures' fat AABBs
     * together: two rounds of loads before any decision */
    uint32_t flags = w.c.flags[i];
    const int2 fx = w.c.fix[i];
    const int2 bd = w.c.body[i];
    const uint4 ids = w.c.mids[i];
    if (flags & CF_DEAD) return HEAD_DONE;
    const uint32_t fa_flags = w.b_flags[bd.x];
    const uint32_t fb_flags = w.b_flags[bd.y];
    const float4 A = w.f_fat[fx.x];
    const float4 B = w.f_fat[fx.y];
    bool destroy = false;
    if (flags & CF_FILTER) {
        /* flagged for filtering (a joint made or destroyed, new filter data): should these bodies and
         * fixtures collide? CF_REJECT: the host's contact filter said no before the step */
        const bool allowed = sp.custom_filter ? !(flags & CF_REJECT) : filter_allows(w, fx.x, fx.y);
        if (!bodies_collide(w, bd.y, bd.x) || !allowed) destroy = true;
        else w.c.flags[i] = flags = flags & ~(CF_FILTER | CF_REJECT);
    }
    if (!destroy && !active_for(w, bd.x, fa_flags, i, deferred) && !active_for(w, bd.y, fb_flags, i, deferred)) {
        if (sp.pre_solve && (flags & CF_UPDATED)) w.c.flags[i] = flags & ~CF_UPDATED;
        return HEAD_SKIPPED;
    }
    const bool was_touching = (flags & CF_TOUCHING) != 0;
    const int old_count = (int)((ids.z >> 8) & 0xffu);
    if (destroy || !overlap4(A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w)) {
        /* destroyed after the pass (the reference collects them and destroys them after its loop) */
        if (sp.record_events && was_touching) push_event(w, 1, fx.x, fx.y);
        if (old_count > 0 && !(flags & CF_SENSOR)) {
            if (deferred) {
                if ((fa_flags & BF_TYPE_MASK) != BODY_STATIC) w.b_dwake[bd.x] = 1;
                if ((fb_flags & BF_TYPE_MASK) != BODY_STATIC) w.b_dwake[bd.y] = 1;
            } else {
                wake_body(w, bd.x);
                wake_body(w, bd.y);
            }
        }
        w.c.flags[i] = (flags | CF_DEAD) & ~CF_TOUCHING;
        return HEAD_DONE;
    }
    if (flags & CF_SENSOR) {
        contact_update(w, sp.record_events != 0, i, flags, fx, bd, ids, deferred ? i : -1,
                       sp.pre_solve ? CF_UPDATED : 0u);
        return HEAD_DONE;
    }
    h.flags = flags;
    h.fx = fx;
    h.bd = bd;
    h.ids = ids;
    return HEAD_EVALUATE;
}

/* The manifolds of one batch: every lane of the warp calls this together; a lane whose state is
 * HEAD_EVALUATE has contact i (described by h) evaluated and finished. When the batch holds at most
 * cfg_collide_group polygon pairs, they go four at a time through collide_polygons_group, each
 * finished by its segment's first lane; otherwise every lane evaluates its own pair. */
__device__ __forceinline__ void collide_batch(const DevWorld& w, const StepParams& sp, int i, int state, const Head& h,
                                              bool deferred) {
    const int lane = threadIdx.x & 31;
    const bool rec = sp.record_events != 0;
    const uint32_t set_flags = sp.pre_solve ? CF_UPDATED : 0u;
    const int kind = state == HEAD_EVALUATE ? (int)((h.flags >> CF_KIND_SHIFT) & 7u) : -1;
    const unsigned polygons = __ballot_sync(kFullWarp, kind == KIND_POLYGONS);
    const bool segments = __popc(polygons) <= w.cfg_collide_group;
    if (kind >= 0 && (kind != KIND_POLYGONS || !segments)) {
        Manifold m;
        manifold_init(m);
        evaluate(kind, m, shape_rows(w, h.fx.x), load_xf(w, h.bd.x), shape_rows(w, h.fx.y), load_xf(w, h.bd.y));
        contact_finish(w, rec, i, h.flags, h.fx, h.bd, h.ids, w.c.mimp[i], m, deferred ? i : -1, set_flags);
    }
    unsigned todo = segments ? polygons : 0u;
    const int seg = lane >> 3, row = lane & 7;
    while (todo) {
        const int src = seg_source(todo, seg);
        todo = seg_rest(todo);
        const int from = src >= 0 ? src : lane;
        const int ci = __shfl_sync(kFullWarp, i, from);
        const int2 fx = make_int2(__shfl_sync(kFullWarp, h.fx.x, from), __shfl_sync(kFullWarp, h.fx.y, from));
        const int2 bd = make_int2(__shfl_sync(kFullWarp, h.bd.x, from), __shfl_sync(kFullWarp, h.bd.y, from));
        float4 la = make_float4(0.0f, 0.0f, 0.0f, 0.0f), lb = la, ha = la, hb = la;
        Xf xa, xb;
        xa.p = xb.p = mk(0.0f, 0.0f);
        xa.q.s = xb.q.s = 0.0f;
        xa.q.c = xb.q.c = 1.0f;
        if (src >= 0) {
            ha = w.f_hdr[fx.x];
            hb = w.f_hdr[fx.y];
            la = w.f_vn[(size_t)fx.x * kMaxPolygonVertices + row];
            lb = w.f_vn[(size_t)fx.y * kMaxPolygonVertices + row];
            xa = load_xf(w, bd.x);
            xb = load_xf(w, bd.y);
        }
        Manifold m;
        manifold_init(m);
        collide_polygons_group(m, row, la, (__float_as_int(ha.w) >> 8) & 0xff, ha.z, xa, lb,
                               (__float_as_int(hb.w) >> 8) & 0xff, hb.z, xb);
        const uint32_t cflags = __shfl_sync(kFullWarp, h.flags, from);
        const uint4 ids = make_uint4(__shfl_sync(kFullWarp, h.ids.x, from), __shfl_sync(kFullWarp, h.ids.y, from),
                                     __shfl_sync(kFullWarp, h.ids.z, from), __shfl_sync(kFullWarp, h.ids.w, from));
        if (src >= 0 && row == 0)
            contact_finish(w, rec, ci, cflags, fx, bd, ids, w.c.mimp[ci], m, deferred ? ci : -1, set_flags);
    }
}

/* all lanes of the warp leave together when the world has been aborted */
__device__ __forceinline__ bool warp_aborted(const DevWorld& w) {
    return __any_sync(kFullWarp, world_aborted(w.cnt));
}

}  // namespace

__global__ void __launch_bounds__(256, 4) k_collide(DevWorld w, StepParams sp, int deferred) {
    if (warp_aborted(w)) return;
    const int n = w.cnt[CNT_CONTACTS];
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const int i = base + lane;
        Head h;
        const int state = i < n ? collide_head(w, sp, i, deferred != 0, h) : HEAD_SKIPPED;
        if (deferred && i < n) w.c_done[i] = state != HEAD_SKIPPED ? 1 : 0;
        collide_batch(w, sp, i, state, h, deferred != 0);
    }
}

/* The contacts skipped as inactive whose body a contact earlier in the table woke: collided in
 * rounds until a round finds none (a chain of wakes along the table's order). */
__global__ void __launch_bounds__(256) k_collide_cascade(DevWorld w, StepParams sp) {
    if (warp_aborted(w)) return;
    grid_barrier_start();
    const int n = w.cnt[CNT_CONTACTS];
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    volatile int* vcnt = w.cnt;
    int round = 0;
    for (; round < n + 1; ++round) {
        if (gtid == 0) vcnt[CNT_CASCADE + (round + 1) % 3] = 0;
        int mine = 0;
        for (int base = gtid - lane; base < n; base += gridDim.x * blockDim.x) {
            const int i = base + lane;
            bool want = i < n && !w.c_done[i];
            if (want) {
                const int2 bd = w.c.body[i];
                const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
                want = active_for(w, bd.x, fa, i, true) || active_for(w, bd.y, fb, i, true);
            }
            Head h;
            const int state = want ? collide_head(w, sp, i, true, h) : HEAD_SKIPPED;
            collide_batch(w, sp, i, state, h, true);
            if (want) {
                w.c_done[i] = 1;
                ++mine;
            }
        }
        if (mine) atomicAdd(&w.cnt[CNT_CASCADE + round % 3], mine);
        if (!grid_barrier(w)) return;
        if (vcnt[CNT_CASCADE + round % 3] == 0) break;
    }
    if (gtid == 0) vcnt[CNT_CASCADE_ROUNDS] = round;
}

/* apply the pass's wakes (set_awake(true): awake, sleep time 0) and clear the records */
__global__ void k_collide_wake(DevWorld w) {
    B2G_RETURN_IF_ABORTED(w);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.n_bodies; b += gridDim.x * blockDim.x) {
        if (w.b_wake[b] != kNoWake || w.b_dwake[b]) {
            const uint32_t f = w.b_flags[b];
            if ((f & BF_TYPE_MASK) != BODY_STATIC) {
                w.b_flags[b] = f | BF_AWAKE;
                w.b_vel[b].w = 0.0f;
            }
            w.b_wake[b] = kNoWake;
            w.b_dwake[b] = 0;
        }
    }
}

/* B2world::create_joint (private/dynamics/b2_world.rs:258-271): the contacts between two bodies
 * joined without collide_connected are flagged for filtering at the next collide */
__global__ void k_flag_joint_contacts(DevWorld w) {
    B2G_RETURN_IF_ABORTED(w);
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int2 bd = w.c.body[i];
        if (!joint_allows(w, bd.y, bd.x)) w.c.flags[i] |= CF_FILTER;
    }
}

/* Contact edits of a host call between steps, one thread per contact of the table:
 *  - fix_mark bit 0 (a destroyed fixture: B2body::destroy_fixture, B2world::destroy_body): the
 *    contact is destroyed as B2contactManager::destroy does (private/dynamics/b2_contact_manager.rs:24-78
 *    with b2_contact_destroy, private/dynamics/b2_contact.rs:33-46): an end event if it touches, both
 *    bodies woken if its manifold has points and neither fixture is a sensor; it is then dead (collide
 *    skips it and the next merge drops it);
 *  - fix_mark bit 1 (B2fixture::refilter, private/dynamics/b2_fixture.rs:181-211) and the body pairs
 *    of destroyed joints without collide_connected (B2world::destroy_joint,
 *    private/dynamics/b2_world.rs:326-340): the contact is flagged for filtering at the next collide. */
__global__ void k_edit_contacts(DevWorld w, const uint8_t* fix_mark, const int2* body_pairs, int n_pairs,
                                int record_events) {
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t flags = w.c.flags[i];
        if (flags & CF_DEAD) continue;
        const int2 fx = w.c.fix[i];
        const uint8_t m = fix_mark[fx.x] | fix_mark[fx.y];
        if (m & 1u) {
            if (record_events && (flags & CF_TOUCHING)) push_event(w, 1, fx.x, fx.y);
            const int old_count = (int)((w.c.mids[i].z >> 8) & 0xffu);
            if (old_count > 0 && !(flags & CF_SENSOR)) {
                const int2 bd = w.c.body[i];
                wake_body(w, bd.x);
                wake_body(w, bd.y);
            }
            w.c.flags[i] = (flags | CF_DEAD) & ~CF_TOUCHING;
            continue;
        }
        bool flag = (m & 2u) != 0;
        if (!flag && n_pairs > 0) {
            const int2 bd = w.c.body[i];
            for (int k = 0; k < n_pairs && !flag; ++k) {
                const int2 p = body_pairs[k];
                flag = (p.x == bd.x && p.y == bd.y) || (p.x == bd.y && p.y == bd.x);
            }
        }
        if (flag) w.c.flags[i] = flags | CF_FILTER;
    }
}

void launch_edit_contacts(const DevWorld& w, const uint8_t* fix_mark, const int2* body_pairs, int n_pairs,
                          bool record_events, cudaStream_t s) {
    k_edit_contacts<<<grid_for(w.contact_cap, 256, w.num_sms * 8), 256, 0, s>>>(w, fix_mark, body_pairs, n_pairs,
                                                                                record_events ? 1 : 0);
    B2G_LAUNCHED(1);
}

void launch_flag_joint_contacts(const DevWorld& w, cudaStream_t s, int num_sms) {
    k_flag_joint_contacts<<<grid_for(w.contact_cap, 256, num_sms * 8), 256, 0, s>>>(w);
    B2G_LAUNCHED(1);
}

/* The narrowphase's structure-of-arrays copy of fixtures [0, n)'s shape records: row k of fixture f
 * (f_vn[f * 8 + k]) = (v[k], n[k]) for the rows its shape uses (a polygon's vertex count, a circle's
 * centre, an edge's four vertices), zeros past them; f_hdr[f] = (centroid, radius, meta bits). */
__global__ void k_shape_rows(DevWorld w, int n) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        const ShapeRec& s = w.f_shape[f];
        const int type = shape_type(s);
        const int rows = type == SHAPE_POLYGON ? shape_count(s) : type == SHAPE_EDGE ? 4 : 1;
        float4* vn = w.f_vn + (size_t)f * kMaxPolygonVertices;
#pragma unroll
        for (int k = 0; k < kMaxPolygonVertices; ++k)
            vn[k] = k < rows ? make_float4(s.v[k].x, s.v[k].y, s.n[k].x, s.n[k].y) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        w.f_hdr[f] = make_float4(s.centroid.x, s.centroid.y, s.radius, __int_as_float(s.meta));
    }
}

void launch_shape_rows(const DevWorld& w, int n_fixtures, cudaStream_t s) {
    if (n_fixtures <= 0) return;
    k_shape_rows<<<grid_for(n_fixtures, 256, w.num_sms * 8), 256, 0, s>>>(w, n_fixtures);
    B2G_LAUNCHED(1);
}

void launch_collide(const DevWorld& w, const StepParams& sp, cudaStream_t s, bool may_sleep, int num_sms) {
    const int block = w.cfg_collide_block;
    k_collide<<<grid_for(w.contact_cap, block, w.num_sms * 2048 / block), block, 0, s>>>(w, sp, may_sleep ? 1 : 0);
    B2G_LAUNCHED(1);
    if (!may_sleep) return;
    DevWorld wc = w;
    StepParams p = sp;
    void* args[] = {&wc, &p};
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    cudaMemsetAsync(w.cnt + CNT_CASCADE, 0, 3 * sizeof(int), s);
    cudaLaunchCooperativeKernel((const void*)k_collide_cascade, dim3(num_sms), dim3(256), args, 0, s);
    k_collide_wake<<<grid_for(w.n_bodies, 256, num_sms * 8), 256, 0, s>>>(w);
    B2G_LAUNCHED(2);
}

/* Stand-alone manifolds of independent shape pairs (the public b2_collide_* functions,
 * src/b2_collision.rs:259-315). xf = (x, y, sin, cos) per shape. Batches of 32 pairs per warp as in
 * k_collide: a batch with at most kPairsCollideGroup polygon pairs takes them four at a time through
 * collide_polygons_group, the rest (and a batch with more) one lane each. Shape pairs of mixed kinds
 * use both forms, so the routine's known answers pin the segment form a world's launch configuration
 * can choose as well as the one-lane form. */
constexpr int kPairsCollideGroup = 8;

__global__ void k_collide_pairs(const ShapeRec* a, const float4* xa, const ShapeRec* b, const float4* xb,
                                const int* kind, int n, float4* geo, float4* pts, uint4* ids) {
    const int lane = threadIdx.x & 31;
    const int seg = lane >> 3, row = lane & 7;
    auto load = [](const float4* x, int i) {
        const float4 v = x[i];
        Xf t;
        t.p = mk(v.x, v.y);
        t.q.s = v.z;
        t.q.c = v.w;
        return t;
    };
    auto store = [&](int i, const Manifold& m) {
        geo[i] = make_float4(m.ln.x, m.ln.y, m.lp.x, m.lp.y);
        pts[i] = make_float4(m.p[0].x, m.p[0].y, m.p[1].x, m.p[1].y);
        ids[i] = make_uint4(m.id[0], m.id[1], (uint32_t)m.type | ((uint32_t)m.count << 8), 0u);
    };
    for (int base = blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += gridDim.x * blockDim.x) {
        const int i = base + lane;
        const int k = i < n ? kind[i] : -1;
        const unsigned polygons = __ballot_sync(kFullWarp, i < n && k == KIND_POLYGONS);
        const bool segments = __popc(polygons) <= kPairsCollideGroup;
        if (i < n && (k != KIND_POLYGONS || !segments)) {
            Manifold m;
            m.type = MANIFOLD_CIRCLES;
            m.count = 0;
            m.ln = m.lp = mk(0.0f, 0.0f);
            m.p[0] = m.p[1] = mk(0.0f, 0.0f);
            m.id[0] = m.id[1] = 0u;
            const ShapeRec sa = a[i];
            const ShapeRec sb = b[i];
            evaluate(k, m, sa, load(xa, i), sb, load(xb, i));
            store(i, m);
        }
        unsigned todo = segments ? polygons : 0u;
        while (todo) {
            const int src = seg_source(todo, seg);
            todo = seg_rest(todo);
            const int ci = __shfl_sync(kFullWarp, i, src >= 0 ? src : lane);
            float4 la = make_float4(0.0f, 0.0f, 0.0f, 0.0f), lb = la;
            int na = 0, nb = 0;
            float ra = 0.0f, rb = 0.0f;
            Xf A, B;
            A.p = B.p = mk(0.0f, 0.0f);
            A.q.s = B.q.s = 0.0f;
            A.q.c = B.q.c = 1.0f;
            if (src >= 0) {
                const ShapeRec& sa = a[ci];
                const ShapeRec& sb = b[ci];
                la = make_float4(sa.v[row].x, sa.v[row].y, sa.n[row].x, sa.n[row].y);
                lb = make_float4(sb.v[row].x, sb.v[row].y, sb.n[row].x, sb.n[row].y);
                na = shape_count(sa);
                nb = shape_count(sb);
                ra = sa.radius;
                rb = sb.radius;
                A = load(xa, ci);
                B = load(xb, ci);
            }
            Manifold m;
            m.type = MANIFOLD_CIRCLES;
            m.count = 0;
            m.ln = m.lp = mk(0.0f, 0.0f);
            m.p[0] = m.p[1] = mk(0.0f, 0.0f);
            m.id[0] = m.id[1] = 0u;
            collide_polygons_group(m, row, la, na, ra, A, lb, nb, rb, B);
            if (src >= 0 && row == 0) store(ci, m);
        }
    }
}

void launch_collide_pairs(const ShapeRec* a, const float4* xa, const ShapeRec* b, const float4* xb, const int* kind,
                          int n, float4* geo, float4* pts, uint4* ids, cudaStream_t s) {
    k_collide_pairs<<<grid_for(n, 128, current_sm_count() * 16), 128, 0, s>>>(a, xa, b, xb, kind, n, geo, pts, ids); B2G_LAUNCHED(1);
}

}  // namespace b2g
