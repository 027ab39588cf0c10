/*
 * k_collide.cu — the narrowphase pass of a step (B2contactManager::collide).
 *
 * Reference: b2_contact_manager_collide, src/private/dynamics/b2_contact_manager.rs:83-171,
 * and b2_contact_update, src/private/dynamics/b2_contact.rs:103-218.
 *
 * One thread per contact of the (key-sorted) contact table:
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
 * Algorithmic bytes per evaluated contact: ~116 B of contact/manifold state + two
 * 144-byte shape records + two body transforms.
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

/* b2_contact_manager_collide for contact i; false if it was skipped as inactive */
__device__ __forceinline__ bool collide_contact(const DevWorld& w, const StepParams& sp, int i, bool deferred) {
    uint32_t flags = w.c.flags[i];
    if (flags & CF_DEAD) return true;
    const int2 fx = w.c.fix[i];
    const int2 bd = w.c.body[i];
    const uint32_t fa_flags = w.b_flags[bd.x];
    const uint32_t fb_flags = w.b_flags[bd.y];
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
        return false;
    }
    const float4 A = w.f_fat[fx.x];
    const float4 B = w.f_fat[fx.y];
    const bool was_touching = (flags & CF_TOUCHING) != 0;
    const uint4 ids = w.c.mids[i];
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
        return true;
    }
    contact_update(w, sp.record_events != 0, i, flags, fx, bd, ids, deferred ? i : -1);
    if (sp.pre_solve) w.c.flags[i] |= CF_UPDATED;
    return true;
}

}  // namespace

__global__ void __launch_bounds__(256) k_collide(DevWorld w, StepParams sp, int deferred) {
    B2G_RETURN_IF_ABORTED(w);
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool done = collide_contact(w, sp, i, deferred != 0);
        if (deferred) w.c_done[i] = done ? 1 : 0;
    }
}

/* The contacts skipped as inactive whose body a contact earlier in the table woke: collided in
 * rounds until a round finds none (a chain of wakes along the table's order). */
__global__ void __launch_bounds__(256) k_collide_cascade(DevWorld w, StepParams sp) {
    B2G_RETURN_IF_ABORTED(w);
    grid_barrier_start();
    const int n = w.cnt[CNT_CONTACTS];
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    volatile int* vcnt = w.cnt;
    int round = 0;
    for (; round < n + 1; ++round) {
        if (gtid == 0) vcnt[CNT_CASCADE + (round + 1) % 3] = 0;
        int mine = 0;
        for (int i = gtid; i < n; i += gridDim.x * blockDim.x) {
            if (w.c_done[i]) continue;
            const int2 bd = w.c.body[i];
            const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
            if (!active_for(w, bd.x, fa, i, true) && !active_for(w, bd.y, fb, i, true)) continue;
            collide_contact(w, sp, i, true);
            w.c_done[i] = 1;
            ++mine;
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
 * src/b2_collision.rs:259-315). xf = (x, y, sin, cos) per shape. */
__global__ void k_collide_pairs(const ShapeRec* a, const float4* xa, const ShapeRec* b, const float4* xb,
                                const int* kind, int n, float4* geo, float4* pts, uint4* ids) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Xf A, B;
        const float4 x0 = xa[i], x1 = xb[i];
        A.p = mk(x0.x, x0.y);
        A.q.s = x0.z;
        A.q.c = x0.w;
        B.p = mk(x1.x, x1.y);
        B.q.s = x1.z;
        B.q.c = x1.w;
        Manifold m;
        m.type = MANIFOLD_CIRCLES;
        m.count = 0;
        m.ln = m.lp = mk(0.0f, 0.0f);
        m.p[0] = m.p[1] = mk(0.0f, 0.0f);
        m.id[0] = m.id[1] = 0u;
        const ShapeRec sa = a[i];
        const ShapeRec sb = b[i];
        evaluate(kind[i], m, sa, A, sb, B);
        geo[i] = make_float4(m.ln.x, m.ln.y, m.lp.x, m.lp.y);
        pts[i] = make_float4(m.p[0].x, m.p[0].y, m.p[1].x, m.p[1].y);
        ids[i] = make_uint4(m.id[0], m.id[1], (uint32_t)m.type | ((uint32_t)m.count << 8), 0u);
    }
}

void launch_collide_pairs(const ShapeRec* a, const float4* xa, const ShapeRec* b, const float4* xb, const int* kind,
                          int n, float4* geo, float4* pts, uint4* ids, cudaStream_t s) {
    k_collide_pairs<<<grid_for(n, 128, current_sm_count() * 16), 128, 0, s>>>(a, xa, b, xb, kind, n, geo, pts, ids); B2G_LAUNCHED(1);
}

}  // namespace b2g
