/*
 * k_continuous.cu — continuous physics of a step: the time-of-impact pass (B2world::solve_toi).
 *
 * Reference: B2world::solve_toi (private/dynamics/b2_world.rs:534-901), B2island::solve_toi
 * (private/dynamics/b2_island_private.rs:330-458), solve_toi_position_constraints
 * (private/dynamics/b2_contact_solver_private.rs:733-823), B2body::advance (src/b2_body.rs:979-986)
 * and B2Sweep::advance (src/b2_math.rs:773-779).
 *
 * The reference repeats until no contact has a time of impact at or below 1 - 10 eps: compute (or
 * reuse) the time of impact of every contact with a bullet, static or kinematic body, take the
 * earliest, move its two bodies there, solve the small island of that contact and of the bodies'
 * contacts with static, kinematic or bullet partners over the rest of the step, re-synchronise the
 * moved proxies and add the new pairs they overlap.
 *
 * Events side by side. A "simple" body is a non-bullet dynamic body that touches no kinematic or
 * bullet body; its events are with static bodies, and its island holds only itself and static
 * bodies, which an event never changes (advancing a static sweep leaves it where it is). Events of
 * different simple bodies therefore commute, and the earliest event of every simple body that comes
 * before the world's earliest other event is solved in the same iteration; every other event is
 * solved alone, in the reference's order. The only order-dependent effects left are:
 *  - a body whose sweep two events of one iteration want advanced to different alphas (a kinematic
 *    or bullet body newly reached by two simple bodies): detected, and the pass restarts from a
 *    snapshot taken before its first event, solving every event alone;
 *  - pairs of two simple bodies found with proxies moved in another order: a pair whose fat AABBs
 *    overlap at the end of the pass is found either way; a pair found only in between never gets a
 *    manifold and the next collide removes it, so it changes no body.
 * A static body's alpha0 is not kept: the reference advances a body to its static partner's alpha0
 * only when that is ahead of the body's, which its order of events never makes happen (a body's
 * times of impact are recomputed right after the body's own event).
 *
 * One persistent cooperative launch (one block per SM) runs the loop; an iteration is:
 *   1 each eligible contact with a stale time of impact computes it (one thread per contact);
 *     candidates at or below 1 - 10 eps lower their body's and world's minima (atomicMin on bits)
 *   2 pending sweep advances are committed; ties among equal times go to the smallest contact key
 *     (the reference takes the first of its contact list; the oracle's ordering hook does the same)
 *   3 events are chosen: the earliest candidate of each simple body that precedes the world's
 *     earliest other candidate, else that one alone
 *   4 one thread per event: advance the two bodies, update the contact; a contact that does not
 *     touch is disabled and the sweeps restored
 *   5 the other contacts of each event's dynamic bodies whose partner is static, kinematic or a
 *     bullet are gathered per event (the reference walks the bodies' contact lists)
 *   6 one warp per event (one lane; islands are small): in key order, tentatively advance each
 *     partner and update the contact, keeping it if it touches; B2island::solve_toi in shared
 *     memory (up to 20 position iterations moving only the event's two bodies, the leap of faith,
 *     velocity iterations without warm starting, integration over (1 - alpha) dt); proxy
 *     synchronisation, with the moved proxies' LBVH leaves updated in place and their ancestors'
 *     boxes grown to cover them
 *   7 pairs of the moved proxies on the LBVH (skip itself, skip a moved partner with a larger proxy
 *     id); new contacts are appended to the table
 * After the loop the appended contacts are merged into the key-sorted table.
 */
#include <climits>

#include "b2g_contact.cuh"
#include "b2g_solver_math.cuh"
#include "b2g_sync.cuh"
#include "b2g_toi.cuh"

namespace b2g {
namespace {

constexpr int kTBlock = 256;
constexpr int kIslWarps = 4;               /* warps of a block that solve islands (shared scratch each) */
constexpr int kMaxSubSteps = 8;            /* B2_MAX_SUB_STEPS, src/b2_common.rs:51 */
constexpr int kToiPositionIterations = 20; /* private/dynamics/b2_world.rs:856 */
constexpr float kToiBaumgarte = 0.75f;     /* B2_TOI_BAUMGARTE, src/b2_common.rs:80 */
constexpr int kIslBodies = 64;             /* the TOI island's body capacity, 2 x B2_MAX_TOICONTACTS */
constexpr int kIslContacts = kToiCand + 1;
constexpr int kMaxIters = 1 << 16;         /* iterations of one pass */
constexpr int kStack = 64;
constexpr uint32_t kNoAlpha = 0xffffffffu;
/* 1 - 10 eps: the largest alpha that is still an event (private/dynamics/b2_world.rs:697) */
constexpr float kEventMax = 1.0f - 10.0f * kEpsilon;

__device__ __forceinline__ bool dynamic_body(uint32_t f) { return (f & BF_TYPE_MASK) == BODY_DYNAMIC; }
__device__ __forceinline__ bool static_body(uint32_t f) { return (f & BF_TYPE_MASK) == BODY_STATIC; }

__device__ __forceinline__ void toi_overflow(const DevWorld& w) {
    atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_TOI_OVERFLOW);
}

__device__ __forceinline__ Sweep load_sweep(const DevWorld& w, int b) {
    const float2 lc = w.b_lc[b];
    const float4 p = w.b_pos[b], p0 = w.b_pos0[b];
    Sweep s;
    s.lc = mk(lc.x, lc.y);
    s.c0 = mk(p0.x, p0.y);
    s.a0 = p0.z;
    s.c = mk(p.x, p.y);
    s.a = p.z;
    s.alpha0 = w.b_alpha0[b];
    return s;
}

__device__ __forceinline__ void store_sweep(const DevWorld& w, int b, const Sweep& s) {
    float4 p = w.b_pos[b], p0 = w.b_pos0[b];
    p.x = s.c.x;
    p.y = s.c.y;
    p.z = s.a;
    p0.x = s.c0.x;
    p0.y = s.c0.y;
    p0.z = s.a0;
    w.b_pos[b] = p;
    w.b_pos0[b] = p0;
    w.b_alpha0[b] = s.alpha0;
}

/* B2Sweep::advance, src/b2_math.rs:773-779 */
__device__ __forceinline__ void sweep_advance(Sweep& s, float alpha) {
    const float beta = fdiv(alpha - s.alpha0, 1.0f - s.alpha0);
    s.c0 = add(s.c0, scale(beta, sub(s.c, s.c0)));
    s.a0 += beta * (s.a - s.a0);
    s.alpha0 = alpha;
}

/* B2body::synchronize_transform, src/b2_body.rs:974-977 */
__device__ __forceinline__ void sync_transform(const DevWorld& w, int b, V2 c, float a, V2 lc) {
    const Rot q = rot(a);
    const V2 p = sub(c, mul(q, lc));
    w.b_xf[b] = make_float4(p.x, p.y, q.s, q.c);
}

/* B2body::advance, src/b2_body.rs:979-986 (a static body does not move: left alone) */
__device__ __forceinline__ void body_advance(const DevWorld& w, int b, float alpha) {
    if (static_body(w.b_flags[b])) return;
    Sweep s = load_sweep(w, b);
    sweep_advance(s, alpha);
    s.c = s.c0;
    s.a = s.a0;
    store_sweep(w, b, s);
    sync_transform(w, b, s.c, s.a, s.lc);
}

/* a body's sweep put back (with its transform) */
__device__ __forceinline__ void restore_body(const DevWorld& w, int b, const Sweep& s) {
    if (static_body(w.b_flags[b])) return;
    store_sweep(w, b, s);
    sync_transform(w, b, s.c, s.a, s.lc);
}

/* ask for the body's sweep to be advanced to alpha in phase 2 (each body listed once); two
 * different alphas for one body in an iteration of side-by-side events are a conflict (and any
 * advance is one under B2G_TOI_SCHEDULE_RESTART_ON_ADVANCE) */
__device__ __forceinline__ void request_advance(const DevWorld& w, const StepParams& sp, int b, float alpha,
                                                bool batched) {
    const uint32_t t = __float_as_uint(alpha);
    const uint32_t prev = atomicMax(&w.b_sync[b], t);
    if (prev == 0u) {
        const int slot = atomicAdd(&w.cnt[CNT_TOI_SYNC], 1);
        if (slot < w.body_cap) w.t_sync[slot] = b;
    }
    if (batched && ((prev != 0u && prev != t) || sp.toi_schedule == B2G_TOI_SCHEDULE_RESTART_ON_ADVANCE))
        atomicExch(&w.cnt[CNT_TOI_CONFLICT], 1);
}

/* contacts appended by the pass so far (slots [n_tab, n_tab + this) of the table hold them) */
__device__ __forceinline__ int appended(const DevWorld& w, int n_tab) {
    const int n = min(((volatile int*)w.cnt)[CNT_TOI_NEW], kToiNewCap);
    return min(n, w.contact_cap - n_tab);
}

__device__ __forceinline__ int lower_bound_key(const unsigned long long* a, int n, unsigned long long key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* the table slot of the live contact with this key: binary search in the sorted table, then the
 * contacts appended by the pass; -1 if none */
__device__ int find_contact(const DevWorld& w, int n_tab, int n_all, unsigned long long key) {
    const int lo = lower_bound_key(w.c.key, n_tab, key);
    if (lo < n_tab && w.c.key[lo] == key) return lo;
    for (int i = n_tab; i < n_all; ++i)
        if (w.c.key[i] == key) return i;
    return -1;
}

/* the reference's static conditions for a time of impact: no sensor, and a bullet or a
 * non-dynamic body on one side (private/dynamics/b2_world.rs:594-621) */
__device__ __forceinline__ uint8_t toi_eligible(const DevWorld& w, int i) {
    if (w.c.flags[i] & CF_SENSOR) return 0;
    const int2 bd = w.c.body[i];
    const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
    const bool collideA = (fa & BF_BULLET) || !dynamic_body(fa);
    const bool collideB = (fb & BF_BULLET) || !dynamic_body(fb);
    return (collideA || collideB) ? 1 : 0;
}

/* a contact with a kinematic or bullet body marks its dynamic bodies: their events go one at a time */
__device__ __forceinline__ void mark_complex(const DevWorld& w, int i, int epoch) {
    const int2 bd = w.c.body[i];
    const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
    const bool xa = (fa & BF_TYPE_MASK) == BODY_KINEMATIC || (dynamic_body(fa) && (fa & BF_BULLET));
    const bool xb = (fb & BF_TYPE_MASK) == BODY_KINEMATIC || (dynamic_body(fb) && (fb & BF_BULLET));
    if (xb && dynamic_body(fa)) w.b_cx[bd.x] = epoch;
    if (xa && dynamic_body(fb)) w.b_cx[bd.y] = epoch;
}

__device__ __forceinline__ bool box_overlap(const float4 a, const float4 b) {
    /* b2_test_overlap, src/b2_collision.rs:355-368 (closed boxes) */
    if (b.x - a.z > 0.0f || b.y - a.w > 0.0f) return false;
    if (a.x - b.z > 0.0f || a.y - b.w > 0.0f) return false;
    return true;
}

__device__ __forceinline__ void atomic_min_float(float* p, float v) {
    int old = __float_as_int(*(volatile float*)p);
    while (v < __int_as_float(old)) {
        const int prev = atomicCAS((int*)p, old, __float_as_int(v));
        if (prev == old) break;
        old = prev;
    }
}

__device__ __forceinline__ void atomic_max_float(float* p, float v) {
    int old = __float_as_int(*(volatile float*)p);
    while (v > __int_as_float(old)) {
        const int prev = atomicCAS((int*)p, old, __float_as_int(v));
        if (prev == old) break;
        old = prev;
    }
}

/* The proxy f got a new fat AABB: its LBVH leaf (and its parent's record of it) take the new box
 * exactly, and every ancestor's record of the subtree grows to cover it, so a walk of the
 * hierarchy (here and in the world queries) sees the proxy where it is. */
__device__ void tree_move(const DevWorld& w, int f, float4 box, bool exact_only) {
    const int n = w.n_fixtures;
    const int l = w.f_leaf[f];
    w.bp_leaf[l] = box;
    if (n < 2) return;
    int child = ~l;
    int node = w.bp_parent[n - 1 + l];
    bool leaf_slot = true;
    for (int guard = 0; guard < 128; ++guard) {
        const int2 ch = w.bp_node_child[node];
        float4* slot = ch.x == child ? &w.bp_node_b0[node] : &w.bp_node_b1[node];
        if (leaf_slot) {
            *slot = box;
            leaf_slot = false;
            if (exact_only) return;
        } else {
            atomic_min_float(&slot->x, box.x);
            atomic_min_float(&slot->y, box.y);
            atomic_max_float(&slot->z, box.z);
            atomic_max_float(&slot->w, box.w);
        }
        if (node == 0) return;
        child = node;
        node = w.bp_parent[node];
    }
}

/* update_pairs' callback and add_pair for query proxy q and partner p (q moved in this
 * iteration); a new contact goes to table slot n_tab + CNT_TOI_NEW */
__device__ void toi_pair(const DevWorld& w, int q, int p, int n_tab, int n_all, int epoch) {
    if (p == q) return;
    const uint32_t rq = w.f_refid[q], rp = w.f_refid[p];
    if (w.f_moved[p] && rp > rq) return;  /* p's own query reports the pair */
    const uint32_t lo = rq < rp ? rq : rp, hi = rq < rp ? rp : rq;
    const unsigned long long key = ((unsigned long long)lo << w.key_bits) | hi;
    if (find_contact(w, n_tab, n_all, key) >= 0) return;
    int fa, fb;
    if (!pair_accept(w, rq < rp ? q : p, rq < rp ? p : q, fa, fb)) return;
    const int slot = atomicAdd(&w.cnt[CNT_TOI_NEW], 1);
    const int pos = n_tab + slot;
    if (slot >= kToiNewCap || pos >= w.contact_cap) {
        toi_overflow(w);
        return;
    }
    init_contact(w, w.c, pos, key, make_int2(fa, fb));
    w.t_elig[pos] = toi_eligible(w, pos);
    w.t_count[pos] = 0;
    w.t_when[pos] = -1;
    mark_complex(w, pos, epoch);
}

/* What B2contactSolver::new reads for island contact ci, with the island's local body indices,
 * positions (c, a) and velocities; qA, qB = rot(a) of the two bodies */
__device__ __forceinline__ ConstraintIn island_constraint(const DevWorld& w, int ci, int ia, int ib, float4 pa,
                                                          float4 pb, float4 va, float4 vb, Rot qA, Rot qB) {
    const int2 fx = w.c.fix[ci];
    const int2 bd = w.c.body[ci];
    const uint4 ids = w.c.mids[ci];
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    ConstraintIn in;
    in.mat = w.c.mat[ci];
    in.geo = w.c.mgeo[ci];
    in.pts = w.c.mpts[ci];
    in.imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  /* sub-steps do not warm start */
    in.mtype = (int)(ids.z & 0xffu);
    in.count = (int)((ids.z >> 8) & 0xffu);
    in.ia = ia;
    in.ib = ib;
    in.flags = 3;
    in.mA = massA.y;
    in.iA = massA.w;
    in.mB = massB.y;
    in.iB = massB.w;
    in.rA = w.f_shape[fx.x].radius;
    in.rB = w.f_shape[fx.y].radius;
    in.lcA = w.b_lc[bd.x];
    in.lcB = w.b_lc[bd.y];
    in.cA = mk(pa.x, pa.y);
    in.cB = mk(pb.x, pb.y);
    in.vA = mk(va.x, va.y);
    in.vB = mk(vb.x, vb.y);
    in.wA = va.z;
    in.wB = vb.z;
    in.qA = qA;
    in.qB = qB;
    return in;
}

struct IslandScratch {
    int body[kIslBodies];
    int con[kIslContacts];
    int cand[kToiCand];
    unsigned long long cand_key[kToiCand];
    float4 pos[kIslBodies];
    float4 vel[kIslBodies];
    PosSlot ps[kIslContacts];
    VelSlot vs[kIslContacts];
};

/* Phase 6 for solid event e (one thread): build the island, B2island::solve_toi, synchronise the
 * dynamic bodies' proxies (b2_world.rs:741-893). */
__device__ void event_island(const DevWorld& w, const StepParams& sp, IslandScratch& S, int e, int iter) {
    const int ev = w.ev_contact[e];
    const int2 ab = w.c.body[ev];
    const int A = ab.x, B = ab.y;
    const float alpha = w.ev_alpha[e];
    const bool rec = sp.record_events != 0;
    int nb = 2, nc = 1;
    S.body[0] = A;
    S.body[1] = B;
    S.con[0] = ev;
    /* the other contacts of the event's dynamic bodies, in key order */
    const int* cand = w.ev_cand + (size_t)e * (kToiCand + 1);
    const int ncand = min(cand[0], kToiCand);
    for (int k = 0; k < ncand; ++k) {
        const int j = cand[1 + k];
        const unsigned long long key = w.c.key[j];
        int at = k;
        while (at > 0 && S.cand_key[at - 1] > key) {
            S.cand_key[at] = S.cand_key[at - 1];
            S.cand[at] = S.cand[at - 1];
            --at;
        }
        S.cand_key[at] = key;
        S.cand[at] = j;
    }
    auto local = [&](int b) {
        for (int k = 0; k < nb; ++k)
            if (S.body[k] == b) return k;
        return -1;
    };
    for (int k = 0; k < ncand; ++k) {
        const int j = S.cand[k];
        const int2 bd = w.c.body[j];
        const bool viaA = (bd.x == A || bd.x == B) && dynamic_body(w.b_flags[bd.x]);
        const int other = viaA ? bd.y : bd.x;
        const bool in_island = local(other) >= 0;
        const Sweep backup = load_sweep(w, other);
        if (!in_island) body_advance(w, other, alpha);
        const bool touching = contact_update(w, rec, j, w.c.flags[j], w.c.fix[j], bd, w.c.mids[j]);
        if (!touching) {
            restore_body(w, other, backup);
            continue;
        }
        if (nc < kIslContacts) S.con[nc++] = j;
        else toi_overflow(w);
        if (in_island) continue;
        wake_body(w, other);
        if (nb < kIslBodies) S.body[nb++] = other;
        else toi_overflow(w);
    }

    /* B2island::solve_toi, b2_island_private.rs:330-458 */
    for (int k = 0; k < nb; ++k) {
        S.pos[k] = w.b_pos[S.body[k]];
        S.vel[k] = w.b_vel[S.body[k]];
    }
    /* B2contactSolver::new: the position constraints (their velocity part is made again below) */
    for (int q = 0; q < nc; ++q) {
        const int ci = S.con[q];
        const int2 bd = w.c.body[ci];
        const int ia = max(local(bd.x), 0), ib = max(local(bd.y), 0);
        const float4 xa = w.b_xf[bd.x], xb = w.b_xf[bd.y];
        Rot qa, qb;
        qa.s = xa.z;
        qa.c = xa.w;
        qb.s = xb.z;
        qb.c = xb.w;
        VelSlot vs;
        make_constraint(island_constraint(w, ci, ia, ib, S.pos[ia], S.pos[ib], S.vel[ia], S.vel[ib], qa, qb), vs,
                        S.ps[q]);
    }
    /* solve_toi_position_constraints: only the event's bodies (island indices 0 and 1) move */
    for (int it = 0; it < kToiPositionIterations; ++it) {
        float min_sep = 0.0f;
        for (int q = 0; q < nc; ++q) {
            PosSlot sl = S.ps[q];
            const int ia = sl.idx.x, ib = sl.idx.y;
            if (!(ia == 0 || ia == 1)) {
                sl.inv.x = 0.0f;
                sl.inv.z = 0.0f;
            }
            if (!(ib == 0 || ib == 1)) {
                sl.inv.y = 0.0f;
                sl.inv.w = 0.0f;
            }
            float4 pa = S.pos[ia], pb = S.pos[ib];
            const float ms = solve_position_math(sl, pa, pb, kToiBaumgarte);
            S.pos[ia] = pa;
            S.pos[ib] = pb;
            min_sep = fminr(min_sep, ms);
        }
        if (min_sep >= -1.5f * kLinearSlop) break;
    }
    /* leap of faith to the new safe state */
    for (int k = 0; k < 2; ++k) {
        if (static_body(w.b_flags[S.body[k]])) continue;
        float4 p0 = w.b_pos0[S.body[k]];
        p0.x = S.pos[k].x;
        p0.y = S.pos[k].y;
        p0.z = S.pos[k].z;
        w.b_pos0[S.body[k]] = p0;
    }
    /* initialize_velocity_constraints on the corrected positions, then the velocity iterations */
    for (int q = 0; q < nc; ++q) {
        const int ci = S.con[q];
        const int ia = S.ps[q].idx.x, ib = S.ps[q].idx.y;
        PosSlot ps;
        make_constraint(island_constraint(w, ci, ia, ib, S.pos[ia], S.pos[ib], S.vel[ia], S.vel[ib], rot(S.pos[ia].z),
                                          rot(S.pos[ib].z)),
                        S.vs[q], ps);
    }
    for (int it = 0; it < sp.vi; ++it) {
        for (int q = 0; q < nc; ++q) {
            const VelSlot sl = S.vs[q];
            const int ia = sl.idx.x, ib = sl.idx.y;
            float4 imp = sl.imp;
            float4 va = S.vel[ia], vb = S.vel[ib];
            solve_velocity_math(sl, imp, va, vb);
            S.vs[q].imp = imp;
            S.vel[ia] = va;
            S.vel[ib] = vb;
        }
    }
    /* integrate positions over the rest of the step and synchronise the bodies (a static body's
     * position is unchanged by it: left alone) */
    const float h = (1.0f - alpha) * sp.dt;
    for (int k = 0; k < nb; ++k) {
        const int b = S.body[k];
        if (static_body(w.b_flags[b])) continue;
        float4 p = S.pos[k];
        const float4 v = S.vel[k];
        V2 vv = mk(v.x, v.y);
        float wv = v.z;
        const V2 translation = scale(h, vv);
        if (dot(translation, translation) > kMaxTranslationSquared) {
            const float ratio = fdiv(kMaxTranslation, length(translation));
            vv.x *= ratio;
            vv.y *= ratio;
        }
        const float rotation = h * wv;
        if (rotation * rotation > kMaxRotationSquared) {
            const float ratio = fdiv(kMaxRotation, fabsr(rotation));
            wv *= ratio;
        }
        p.x += h * vv.x;
        p.y += h * vv.y;
        p.z += h * wv;
        const float4 old = w.b_pos[b];
        w.b_pos[b] = make_float4(p.x, p.y, p.z, old.w);
        w.b_vel[b] = make_float4(vv.x, vv.y, wv, w.b_vel[b].w);
        const float2 lc = w.b_lc[b];
        sync_transform(w, b, mk(p.x, p.y), p.z, mk(lc.x, lc.y));
    }
    /* synchronize_fixtures of the dynamic bodies; their contacts' times of impact go stale */
    for (int k = 0; k < nb; ++k) {
        const int b = S.body[k];
        const uint32_t fl = w.b_flags[b];
        if (!dynamic_body(fl)) continue;
        w.b_inval[b] = iter;
        const float4 x2 = w.b_xf[b];
        Xf xf2;
        xf2.p = mk(x2.x, x2.y);
        xf2.q.s = x2.z;
        xf2.q.c = x2.w;
        Xf xf1 = xf2;
        if (fl & BF_AWAKE) {
            const float4 p0 = w.b_pos0[b];
            const float2 lc = w.b_lc[b];
            xf1.q = rot(p0.z);
            xf1.p = sub(mk(p0.x, p0.y), mul(xf1.q, mk(lc.x, lc.y)));
        }
        for (int e2 = w.b_fix_off[b]; e2 < w.b_fix_off[b + 1]; ++e2) {
            const int f = w.b_fix[e2];
            if (!sync_fixture(w, f, xf1, xf2)) continue;
            tree_move(w, f, w.f_fat[f], false);
            const int slot = atomicAdd(&w.cnt[CNT_TOI_MOVED], 1);
            if (slot < w.fix_cap) w.t_moved[slot] = f;
        }
    }
    atomicAdd(&w.cnt[CNT_TOI_EVENTS], 1);
}

/* B2world::solve_toi with a complete step: alpha0 = 0, no body in an island; bodies touching a
 * kinematic or bullet body are marked; proxies find their LBVH leaves */
__device__ void pass_init(const DevWorld& w, int n_tab, int epoch, int gtid, int gstride) {
    for (int b = gtid; b < w.n_bodies; b += gstride) {
        w.b_alpha0[b] = 0.0f;
        w.b_stamp[b] = -1;
        w.b_inval[b] = -1;
        w.b_sync[b] = 0u;
        w.b_best[b] = kNoAlpha;
        w.b_bkey[b] = ~0ull;
    }
    for (int wd = gtid; wd < w.num_worlds; wd += gstride) {
        w.tw_alpha[wd] = kNoAlpha;
        w.tw_key[wd] = ~0ull;
        w.tw_salpha[wd] = kNoAlpha;
        w.tw_skey[wd] = ~0ull;
    }
    for (int i = gtid; i < n_tab; i += gstride) mark_complex(w, i, epoch);
    for (int l = gtid; l < w.n_fixtures; l += gstride) w.f_leaf[w.bp_val[l]] = l;
}

/* (alpha bits, key) pairs in time order */
__device__ __forceinline__ bool earlier(uint32_t a, unsigned long long ka, uint32_t b, unsigned long long kb) {
    return a < b || (a == b && ka < kb);
}

__global__ void __launch_bounds__(kTBlock) k_continuous(DevWorld w, StepParams sp) {
    B2G_RETURN_IF_ABORTED(w);
    extern __shared__ __align__(16) unsigned char smem[];
    IslandScratch* scratch = reinterpret_cast<IslandScratch*>(smem);
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int n_tab = w.cnt[CNT_CONTACTS];
    const bool rec = sp.record_events != 0;
    volatile int* vcnt = w.cnt;
    int epoch = w.cnt[CNT_TOI_PASSES] * 2 + 1;  /* odd, never 0 (the marks' initial value) */
    bool batched = sp.toi_schedule != B2G_TOI_SCHEDULE_ONE_AT_A_TIME;
    bool snapshot = false;  /* the pass's snapshot was taken (uniform across blocks) */

    pass_init(w, n_tab, epoch, gtid, gstride);
    if (!grid_barrier(w)) return;

    int iter = 0;
    for (; iter < kMaxIters; ++iter) {
        const int n_all = n_tab + appended(w, n_tab);
        /* 1: times of impact (private/dynamics/b2_world.rs:564-693) */
        for (int i = gtid; i < n_all; i += gstride) {
            if (iter == 0 && i < n_tab) {
                /* contacts of the table start the pass with no time of impact and no events */
                const uint8_t e = toi_eligible(w, i);
                w.t_elig[i] = e;
                w.t_count[i] = 0;
                w.t_when[i] = -1;
                if (!e) continue;
            } else if (!w.t_elig[i]) {
                continue;
            }
            if (!(w.c.flags[i] & CF_ENABLED)) continue;
            if (w.t_count[i] > kMaxSubSteps) continue;
            const int2 bd = w.c.body[i];
            const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
            float alpha;
            const int when = w.t_when[i];
            if (when >= 0 && when > w.b_inval[bd.x] && when > w.b_inval[bd.y]) {
                alpha = w.t_toi[i];
            } else {
                const bool activeA = (fa & BF_AWAKE) && !static_body(fa);
                const bool activeB = (fb & BF_AWAKE) && !static_body(fb);
                if (!activeA && !activeB) continue;
                Sweep sa = load_sweep(w, bd.x), sb = load_sweep(w, bd.y);
                float alpha0;
                if (static_body(fa)) {
                    alpha0 = sb.alpha0;
                } else if (static_body(fb)) {
                    alpha0 = sa.alpha0;
                } else {
                    alpha0 = sa.alpha0;
                    if (sa.alpha0 < sb.alpha0) {
                        alpha0 = sb.alpha0;
                        sweep_advance(sa, alpha0);
                        request_advance(w, sp, bd.x, alpha0, batched);
                    } else if (sb.alpha0 < sa.alpha0) {
                        alpha0 = sa.alpha0;
                        sweep_advance(sb, alpha0);
                        request_advance(w, sp, bd.y, alpha0, batched);
                    }
                }
                const int2 fx = w.c.fix[i];
                DistProxy pa, pb;
                make_proxy(w.f_shape[fx.x], pa);
                make_proxy(w.f_shape[fx.y], pb);
                int state;
                float beta;
                time_of_impact(pa, sa, pb, sb, 1.0f, state, beta);
                alpha = state == B2G_TOI_TOUCHING ? fminr(alpha0 + (1.0f - alpha0) * beta, 1.0f) : 1.0f;
                w.t_toi[i] = alpha;
                w.t_when[i] = iter;
            }
            if (alpha <= kEventMax) {
                const uint32_t abits = __float_as_uint(alpha);
                const int wd = (int)w.b_world[bd.x];
                int x = -1;
                if (batched) {
                    if (static_body(fa) && dynamic_body(fb) && !(fb & BF_BULLET) && w.b_cx[bd.y] != epoch) x = bd.y;
                    else if (static_body(fb) && dynamic_body(fa) && !(fa & BF_BULLET) && w.b_cx[bd.x] != epoch)
                        x = bd.x;
                }
                if (x >= 0) {
                    atomicMin(&w.b_best[x], abits);
                    atomicMin(&w.tw_salpha[wd], abits);
                } else {
                    atomicMin(&w.tw_alpha[wd], abits);
                }
                const int slot = atomicAdd(&w.cnt[CNT_TOI_HITS], 1);
                if (slot < w.contact_cap) {
                    w.t_hits[slot] = i;
                    w.t_hitx[slot] = x;
                }
            }
        }
        if (!grid_barrier(w)) return;
        const int hits = min(vcnt[CNT_TOI_HITS], w.contact_cap);
        if (hits == 0) break;

        if (batched && vcnt[CNT_TOI_CONFLICT] && !snapshot) {
            /* a conflict where none can arise: report it rather than restart from nothing */
            if (gtid == 0) toi_overflow(w);
            batched = false;
        }
        if (batched && vcnt[CNT_TOI_CONFLICT]) {
            /* two side-by-side events asked one body for different alphas: back to the snapshot,
             * then every event alone */
            for (int b = gtid; b < w.n_bodies; b += gstride) {
                w.b_xf[b] = w.s_xf[b];
                w.b_pos[b] = w.s_pos[b];
                w.b_pos0[b] = w.s_pos0[b];
                w.b_vel[b] = w.s_vel[b];
                w.b_flags[b] = w.s_flags[b];
            }
            for (int f = gtid; f < w.n_fixtures; f += gstride) {
                w.f_fat[f] = w.s_fat[f];
                w.f_moved[f] = 0;
            }
            for (int l = gtid; l < w.n_fixtures; l += gstride) tree_move(w, (int)w.bp_val[l], w.s_fat[w.bp_val[l]], true);
            for (int i = gtid; i < n_tab; i += gstride) {
                w.c.flags[i] = w.c_alt.flags[i];
                w.c.mgeo[i] = w.c_alt.mgeo[i];
                w.c.mpts[i] = w.c_alt.mpts[i];
                w.c.mimp[i] = w.c_alt.mimp[i];
                w.c.mids[i] = w.c_alt.mids[i];
            }
            if (!grid_barrier(w)) return;
            if (gtid == 0) {
                vcnt[CNT_EVENTS] = vcnt[CNT_TOI_SNAP_EV];
                vcnt[CNT_TOI_EVENTS] = vcnt[CNT_TOI_SNAP_TE];
                for (int c = CNT_TOI_NEW; c < CNT_TOI_SNAP_EV; ++c) vcnt[c] = 0;
                vcnt[CNT_TOI_ROLLBACKS] += 1;
            }
            batched = false;
            epoch += 1;
            pass_init(w, n_tab, epoch, gtid, gstride);
            if (!grid_barrier(w)) return;
            iter = -1;
            continue;
        }
        if (iter == 0 && batched && (sp.toi_may_conflict || sp.toi_schedule == B2G_TOI_SCHEDULE_RESTART_ON_ADVANCE)) {
            /* the snapshot a conflict goes back to (nothing has moved yet). Without kinematic and
             * bullet bodies every event is with a static body and no sweep is ever advanced for a
             * time of impact, so no conflict can arise and none is kept. */
            for (int b = gtid; b < w.n_bodies; b += gstride) {
                w.s_xf[b] = w.b_xf[b];
                w.s_pos[b] = w.b_pos[b];
                w.s_pos0[b] = w.b_pos0[b];
                w.s_vel[b] = w.b_vel[b];
                w.s_flags[b] = w.b_flags[b];
            }
            for (int f = gtid; f < w.n_fixtures; f += gstride) w.s_fat[f] = w.f_fat[f];
            for (int i = gtid; i < n_tab; i += gstride) {
                w.c_alt.flags[i] = w.c.flags[i];
                w.c_alt.mgeo[i] = w.c.mgeo[i];
                w.c_alt.mpts[i] = w.c.mpts[i];
                w.c_alt.mimp[i] = w.c.mimp[i];
                w.c_alt.mids[i] = w.c.mids[i];
            }
            if (gtid == 0) {
                vcnt[CNT_TOI_SNAP_EV] = vcnt[CNT_EVENTS];
                vcnt[CNT_TOI_SNAP_TE] = vcnt[CNT_TOI_EVENTS];
            }
            snapshot = true;
        }

        /* 2: commit the sweep advances; ties of the minima go to the smallest key */
        const int nsync = min(vcnt[CNT_TOI_SYNC], w.body_cap);
        for (int j = gtid; j < nsync; j += gstride) {
            const int b = w.t_sync[j];
            Sweep s = load_sweep(w, b);
            sweep_advance(s, __uint_as_float(w.b_sync[b]));
            store_sweep(w, b, s);
            w.b_sync[b] = 0u;
        }
        for (int j = gtid; j < hits; j += gstride) {
            const int i = w.t_hits[j];
            const int x = w.t_hitx[j];
            const uint32_t abits = __float_as_uint(w.t_toi[i]);
            const unsigned long long key = w.c.key[i];
            const int wd = (int)w.b_world[w.c.body[i].x];
            if (x >= 0) {
                if (abits == w.b_best[x]) atomicMin(&w.b_bkey[x], key);
                if (abits == w.tw_salpha[wd]) atomicMin(&w.tw_skey[wd], key);
            } else if (abits == w.tw_alpha[wd]) {
                atomicMin(&w.tw_key[wd], key);
            }
        }
        const int nmoved_prev = min(vcnt[CNT_TOI_MOVED], w.fix_cap);
        for (int j = gtid; j < nmoved_prev; j += gstride) w.f_moved[w.t_moved[j]] = 0;
        if (!grid_barrier(w)) return;

        /* 3: the events of this iteration */
        if (gtid == 0) {
            vcnt[CNT_TOI_SYNC] = 0;
            vcnt[CNT_TOI_MOVED] = 0;
        }
        for (int j = gtid; j < hits; j += gstride) {
            const int i = w.t_hits[j];
            const int x = w.t_hitx[j];
            const uint32_t abits = __float_as_uint(w.t_toi[i]);
            const unsigned long long key = w.c.key[i];
            const int wd = (int)w.b_world[w.c.body[i].x];
            const uint32_t ca = w.tw_alpha[wd];
            const unsigned long long ck = w.tw_key[wd];
            const bool simple_first = earlier(w.tw_salpha[wd], w.tw_skey[wd], ca, ck);
            bool take = false;
            if (x >= 0) {
                if (key == w.b_bkey[x]) {
                    take = simple_first && earlier(abits, key, ca, ck);
                    w.b_best[x] = kNoAlpha;
                    w.b_bkey[x] = ~0ull;
                }
            } else {
                take = !simple_first && abits == ca && key == ck;
            }
            if (take) {
                const int e = atomicAdd(&w.cnt[CNT_TOI_NEV], 1);
                if (e < kToiEvCap) {
                    w.ev_contact[e] = i;
                    w.ev_alpha[e] = __uint_as_float(abits);
                }
            }
        }
        if (!grid_barrier(w)) return;

        /* 4: advance each event's bodies and update its contact (b2_world.rs:695-739) */
        if (gtid == 0) vcnt[CNT_TOI_HITS] = 0;
        for (int wd = gtid; wd < w.num_worlds; wd += gstride) {
            w.tw_alpha[wd] = kNoAlpha;
            w.tw_key[wd] = ~0ull;
            w.tw_salpha[wd] = kNoAlpha;
            w.tw_skey[wd] = ~0ull;
        }
        const int nev = min(vcnt[CNT_TOI_NEV], kToiEvCap);
        for (int e = gtid; e < nev; e += gstride) {
            const int i = w.ev_contact[e];
            const float alpha = w.ev_alpha[e];
            const int2 bd = w.c.body[i];
            const Sweep s1 = load_sweep(w, bd.x), s2 = load_sweep(w, bd.y);
            body_advance(w, bd.x, alpha);
            body_advance(w, bd.y, alpha);
            const bool touching = contact_update(w, rec, i, w.c.flags[i], w.c.fix[i], bd, w.c.mids[i]);
            w.t_when[i] = -1;
            w.t_count[i] += 1;
            w.ev_cand[(size_t)e * (kToiCand + 1)] = 0;
            if (!touching) {
                w.c.flags[i] &= ~CF_ENABLED;
                restore_body(w, bd.x, s1);
                restore_body(w, bd.y, s2);
                w.ev_solid[e] = -1;
                continue;
            }
            wake_body(w, bd.x);
            wake_body(w, bd.y);
            if (dynamic_body(w.b_flags[bd.x])) {
                w.b_stamp[bd.x] = iter;
                w.b_event[bd.x] = e;
            }
            if (dynamic_body(w.b_flags[bd.y])) {
                w.b_stamp[bd.y] = iter;
                w.b_event[bd.y] = e;
            }
            w.ev_solid[e] = iter;
        }
        if (!grid_barrier(w)) return;

        /* 5: the event bodies' other contacts with static, kinematic or bullet partners */
        for (int i = gtid; i < n_all; i += gstride) {
            const int2 bd = w.c.body[i];
            const bool sx = w.b_stamp[bd.x] == iter, sy = w.b_stamp[bd.y] == iter;
            if (!sx && !sy) continue;
            const int body = sx ? bd.x : bd.y;
            const int e = w.b_event[body];
            if (w.ev_contact[e] == i) continue;
            const uint32_t fx = w.b_flags[bd.x], fy = w.b_flags[bd.y];
            const uint32_t fbody = sx ? fx : fy, fother = sx ? fy : fx;
            if (dynamic_body(fother) && !(fbody & BF_BULLET) && !(fother & BF_BULLET)) continue;
            if (w.c.flags[i] & CF_SENSOR) continue;
            int* cand = w.ev_cand + (size_t)e * (kToiCand + 1);
            const int slot = atomicAdd(cand, 1);
            if (slot < kToiCand) cand[1 + slot] = i;
            else toi_overflow(w);
        }
        if (!grid_barrier(w)) return;

        /* 6: the islands, one lane per event */
        if (lane == 0 && warp < kIslWarps) {
            for (int e = blockIdx.x * kIslWarps + warp; e < nev; e += gridDim.x * kIslWarps)
                if (w.ev_solid[e] == iter) event_island(w, sp, scratch[warp], e, iter);
        }
        if (!grid_barrier(w)) return;

        /* 7: find_new_contacts for the proxies this iteration moved */
        if (gtid == 0) vcnt[CNT_TOI_NEV] = 0;
        const int nm = min(vcnt[CNT_TOI_MOVED], w.fix_cap);
        for (int qi = gtid; qi < nm; qi += gstride) {
            const int q = w.t_moved[qi];
            const uint32_t wd = w.b_world[w.f_body[q]];
            const float4 box = w.f_fat[q];
            for (int h = 0; h < 2; ++h) {
                const int root = w.bp_world_root[wd + (h ? (uint32_t)w.num_worlds : 0u)];
                if (root == INT_MIN) continue;
                if (root < 0) {
                    if (box_overlap(w.bp_leaf[~root], box)) toi_pair(w, q, (int)w.bp_val[~root], n_tab, n_all, epoch);
                    continue;
                }
                int stack[kStack];
                int top = 0;
                stack[top++] = root;
                while (top > 0) {
                    const int node = stack[--top];
                    const int2 ch = w.bp_node_child[node];
                    const float4 bx[2] = {w.bp_node_b0[node], w.bp_node_b1[node]};
                    const int kids[2] = {ch.x, ch.y};
                    for (int c = 0; c < 2; ++c) {
                        if (!box_overlap(bx[c], box)) continue;
                        if (kids[c] < 0) toi_pair(w, q, (int)w.bp_val[~kids[c]], n_tab, n_all, epoch);
                        else if (top < kStack) stack[top++] = kids[c];
                        else atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_STACK_OVERFLOW);
                    }
                }
            }
        }
        if (!grid_barrier(w)) return;
    }
    if (iter == kMaxIters) toi_overflow(w);

    /* the pass is over: clear its moved flags, merge its new contacts into the sorted table */
    if (gtid == 0) {
        vcnt[CNT_TOI_ITERS] = iter;
        vcnt[CNT_TOI_PASSES] += 1;
    }
    {
        const int nm = min(vcnt[CNT_TOI_MOVED], w.fix_cap);
        for (int j = gtid; j < nm; j += gstride) w.f_moved[w.t_moved[j]] = 0;
    }
    const int na = appended(w, n_tab);
    if (na == 0) return;
    for (int j = gtid; j < na; j += gstride) {
        const unsigned long long key = w.c.key[n_tab + j];
        int rank = 0;
        for (int k = 0; k < na; ++k) rank += w.c.key[n_tab + k] < key ? 1 : 0;
        w.t_nkey[rank] = key;
        w.t_nslot[rank] = n_tab + j;
    }
    if (!grid_barrier(w)) return;
    const int lo = lower_bound_key(w.c.key, n_tab, w.t_nkey[0]);
    for (int i = lo + gtid; i < n_tab; i += gstride)
        copy_contact(w.c, i, w.c_alt, i + lower_bound_key(w.t_nkey, na, w.c.key[i]));
    for (int r = gtid; r < na; r += gstride)
        copy_contact(w.c, w.t_nslot[r], w.c_alt, r + lower_bound_key(w.c.key, n_tab, w.t_nkey[r]));
    if (!grid_barrier(w)) return;
    for (int k = lo + gtid; k < n_tab + na; k += gstride) copy_contact(w.c_alt, k, w.c, k);
    if (gtid == 0) vcnt[CNT_CONTACTS] = n_tab + na;
}

}  // namespace

int launch_continuous(const DevWorld& w, const StepParams& sp, cudaStream_t s, int num_sms) {
    static bool configured = false;
    const int smem = kIslWarps * (int)sizeof(IslandScratch);
    if (!configured) {
        cudaFuncSetAttribute((const void*)k_continuous, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        configured = true;
    }
    DevWorld wc = w;
    StepParams p = sp;
    void* args[] = {&wc, &p};
    cudaMemsetAsync(w.cnt + CNT_TOI_FIRST, 0, (CNT_TOI_LAST - CNT_TOI_FIRST) * sizeof(int), s);
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    B2G_LAUNCHED(1);
    return (int)cudaLaunchCooperativeKernel((const void*)k_continuous, dim3(num_sms), dim3(kTBlock), args, smem, s);
}

}  // namespace b2g
