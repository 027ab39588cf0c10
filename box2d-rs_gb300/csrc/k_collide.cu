/*
 * k_collide.cu — the narrowphase pass of a step (B2contactManager::collide).
 *
 * Reference: b2_contact_manager_collide, src/private/dynamics/b2_contact_manager.rs:83-171,
 * and b2_contact_update, src/private/dynamics/b2_contact.rs:103-218.
 *
 * One thread per contact of the (key-sorted) contact table:
 *   - skip when neither body is awake and non-static;
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

namespace b2g {

__global__ void __launch_bounds__(256) k_collide(DevWorld w, StepParams sp) {
    const int n = w.cnt[CNT_CONTACTS];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t flags = w.c.flags[i];
        if (flags & CF_DEAD) continue;
        const int2 fx = w.c.fix[i];
        const int2 bd = w.c.body[i];
        const uint32_t fa_flags = w.b_flags[bd.x];
        const uint32_t fb_flags = w.b_flags[bd.y];
        const bool activeA = (fa_flags & BF_AWAKE) && (fa_flags & BF_TYPE_MASK) != BODY_STATIC;
        const bool activeB = (fb_flags & BF_AWAKE) && (fb_flags & BF_TYPE_MASK) != BODY_STATIC;
        if (!activeA && !activeB) continue;
        const float4 A = w.f_fat[fx.x];
        const float4 B = w.f_fat[fx.y];
        const bool was_touching = (flags & CF_TOUCHING) != 0;
        const uint4 ids = w.c.mids[i];
        const int old_count = (int)((ids.z >> 8) & 0xffu);
        if (!overlap4(A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w)) {
            if (sp.record_events && was_touching) push_event(w, 1, fx.x, fx.y);
            if (old_count > 0 && !(flags & CF_SENSOR)) {
                wake_body(w, bd.x);
                wake_body(w, bd.y);
            }
            w.c.flags[i] = (flags | CF_DEAD) & ~CF_TOUCHING;
            continue;
        }
        contact_update(w, sp.record_events != 0, i, flags, fx, bd, ids);
    }
}

void launch_collide(const DevWorld& w, const StepParams& sp, cudaStream_t s) {
    const int block = w.cfg_collide_block;
    k_collide<<<grid_for(w.contact_cap, block, 152 * 2048 / block), block, 0, s>>>(w, sp); B2G_LAUNCHED(1);
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
    k_collide_pairs<<<grid_for(n, 128, 152 * 16), 128, 0, s>>>(a, xa, b, xb, kind, n, geo, pts, ids); B2G_LAUNCHED(1);
}

}  // namespace b2g
