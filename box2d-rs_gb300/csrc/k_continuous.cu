/*
 * k_continuous.cu — continuous physics of a step: the time-of-impact pass (B2world::solve_toi).
 *
 * Reference: B2world::solve_toi (private/dynamics/b2_world.rs:534-901), B2island::solve_toi
 * (private/dynamics/b2_island_private.rs:330-458), solve_toi_position_constraints
 * (private/dynamics/b2_contact_solver_private.rs:733-823), B2body::advance (src/b2_body.rs:979-986)
 * and B2Sweep::advance (src/b2_math.rs:773-779).
 *
 * The reference repeats until no contact has a time of impact below 1 - 10 eps: compute (or
 * reuse) the time of impact of every contact with a bullet, static or kinematic body, take the
 * smallest, move its two bodies there, solve the small island of that contact and of the bodies'
 * contacts with static, kinematic or bullet partners over the rest of the step, re-synchronise the
 * moved proxies and add the new pairs they overlap. Events are sequential within a world and
 * independent across worlds, so one iteration here is one event in every world that has one.
 * One persistent cooperative launch (one block per SM) runs the loop in six grid-wide phases per
 * iteration, separated by the bounded grid barrier:
 *   1 each eligible contact with a stale time of impact computes it (one thread per contact);
 *     the two sweeps are first put on the same alpha0 (locally; the advance is committed in
 *     phase 2). Event candidates lower their world's minimum alpha (atomicMin on the bits).
 *   2 pending sweep advances are committed; candidates equal to their world's minimum lower the
 *     world's minimum contact key: among equal times of impact the event is the contact with the
 *     smallest key (the reference takes the first in its contact list; the oracle's ordering hook
 *     takes the smallest key too).
 *   3 one thread per world with an event: advance the two bodies, update the contact; a contact
 *     that does not touch is disabled and the sweeps are restored.
 *   4 the other contacts of the event's dynamic bodies whose partner is static, kinematic or a
 *     bullet are gathered per world (the reference walks the bodies' contact lists).
 *   5 one block per world (one thread, islands are small): in key order, tentatively advance each
 *     partner and update the contact, keeping it if it touches; then B2island::solve_toi in shared
 *     memory (up to 20 position iterations that move only the event's two bodies, the leap of faith,
 *     velocity constraints without warm starting, integration over (1 - alpha) dt), proxy
 *     synchronisation and invalidation of the displaced bodies' times of impact.
 *   6 pairs of the moved proxies (the reference's rule: skip itself, skip a moved partner with a
 *     larger proxy id): the step's LBVH finds partners whose leaves are current; proxies moved
 *     earlier in the pass (stale leaves) are tested from a list. New contacts are appended to the
 *     contact table.
 * After the loop the appended contacts are merged into the key-sorted table.
 *
 * Sweep advances. When a contact's two sweeps start at different alpha0 the reference advances
 * the earlier one before computing the time of impact. Every time of impact recomputed in an
 * iteration belongs to a contact of a body displaced by the previous iteration's island (alpha0 =
 * that event's alpha, the largest so far) or created by it, so all advances of one iteration go to
 * the same alpha and one advance per body gives the reference's bits in any order. (A body woken
 * out of sleep by a contact update, with sleeping on, is the exception: its contacts may ask for
 * different alphas; the largest is taken.)
 */
#include <climits>

#include "b2g_contact.cuh"
#include "b2g_solver_math.cuh"
#include "b2g_sync.cuh"
#include "b2g_toi.cuh"

namespace b2g {
namespace {

constexpr int kTBlock = 256;
constexpr int kMaxSubSteps = 8;            /* B2_MAX_SUB_STEPS, src/b2_common.rs:51 */
constexpr int kToiPositionIterations = 20; /* private/dynamics/b2_world.rs:856 */
constexpr float kToiBaumgarte = 0.75f;     /* B2_TOI_BAUMGARTE, src/b2_common.rs:80 */
constexpr int kIslBodies = 64;             /* the TOI island's body capacity, 2 x B2_MAX_TOICONTACTS */
constexpr int kIslContacts = kToiCand + 1;
constexpr int kMaxIters = 1 << 16;       /* iterations of one pass (events per world) */
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

/* B2body::advance, src/b2_body.rs:979-986 */
__device__ __forceinline__ void body_advance(const DevWorld& w, int b, float alpha) {
    Sweep s = load_sweep(w, b);
    sweep_advance(s, alpha);
    s.c = s.c0;
    s.a = s.a0;
    store_sweep(w, b, s);
    sync_transform(w, b, s.c, s.a, s.lc);
}

/* a body's sweep put back (with its transform) */
__device__ __forceinline__ void restore_body(const DevWorld& w, int b, const Sweep& s) {
    store_sweep(w, b, s);
    sync_transform(w, b, s.c, s.a, s.lc);
}

/* ask for the body's sweep to be advanced to alpha in phase 2 (each body listed once) */
__device__ __forceinline__ void request_advance(const DevWorld& w, int b, float alpha) {
    const uint32_t prev = atomicMax(&w.b_sync[b], __float_as_uint(alpha));
    if (prev == 0u) {
        const int slot = atomicAdd(&w.cnt[CNT_TOI_SYNC], 1);
        if (slot < w.body_cap) w.t_sync[slot] = b;
    }
}

/* contacts appended by the pass so far (slots [n_tab, n_tab + this) of the table hold them) */
__device__ __forceinline__ int appended(const DevWorld& w, int n_tab) {
    const int n = min(((volatile int*)w.cnt)[CNT_TOI_NEW], kToiNewCap);
    return min(n, w.contact_cap - n_tab);
}

/* the table slot of the live contact with this key: binary search in the sorted table, then the
 * contacts appended by the pass; -1 if none */
__device__ int find_contact(const DevWorld& w, int n_tab, int n_all, unsigned long long key) {
    int lo = 0, hi = n_tab;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (w.c.key[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    if (lo < n_tab && w.c.key[lo] == key) return lo;
    for (int i = n_tab; i < n_all; ++i)
        if (w.c.key[i] == key) return i;
    return -1;
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

__device__ __forceinline__ bool box_overlap(const float4 a, const float4 b) {
    /* b2_test_overlap, src/b2_collision.rs:355-368 (closed boxes) */
    if (b.x - a.z > 0.0f || b.y - a.w > 0.0f) return false;
    if (a.x - b.z > 0.0f || a.y - b.w > 0.0f) return false;
    return true;
}

/* update_pairs' callback and add_pair for query proxy q and partner p (q moved in this
 * iteration); a new contact goes to table slot n_tab + CNT_TOI_NEW */
__device__ void toi_pair(const DevWorld& w, int q, int p, int n_tab, int n_all) {
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
    w.t_stamp[pos] = -1;
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

/* Phase 5 for world wd's solid event (one thread): build the island, B2island::solve_toi,
 * synchronise the dynamic bodies' proxies. */
__device__ void event_island(const DevWorld& w, const StepParams& sp, IslandScratch& S, int wd, int iter) {
    const int4 ev = w.tw_event[wd];
    const int A = ev.y, B = ev.z;
    const float alpha = w.tw_ealpha[wd];
    const bool rec = sp.record_events != 0;
    int nb = 2, nc = 1;
    S.body[0] = A;
    S.body[1] = B;
    S.con[0] = ev.x;
    /* the other contacts of the event's dynamic bodies, in key order */
    const int* cand = w.tw_cand + (size_t)wd * (kToiCand + 1);
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
    for (int k = 0; k < ncand; ++k) {
        const int j = S.cand[k];
        const int2 bd = w.c.body[j];
        const bool viaA = (bd.x == A || bd.x == B) && dynamic_body(w.b_flags[bd.x]);
        const int other = viaA ? bd.y : bd.x;
        const bool in_island = w.b_stamp[other] == iter;
        const Sweep backup = load_sweep(w, other);
        if (!in_island) body_advance(w, other, alpha);
        const bool touching = contact_update(w, rec, j, w.c.flags[j], w.c.fix[j], bd, w.c.mids[j]);
        if (!touching) {
            restore_body(w, other, backup);
            continue;
        }
        w.t_stamp[j] = iter;
        if (nc < kIslContacts) S.con[nc++] = j;
        else toi_overflow(w);
        if (in_island) continue;
        w.b_stamp[other] = iter;
        wake_body(w, other);
        if (nb < kIslBodies) S.body[nb++] = other;
        else toi_overflow(w);
    }

    /* B2island::solve_toi, b2_island_private.rs:330-458 */
    for (int k = 0; k < nb; ++k) {
        S.pos[k] = w.b_pos[S.body[k]];
        S.vel[k] = w.b_vel[S.body[k]];
    }
    auto local = [&](int b) {
        for (int k = 0; k < nb; ++k)
            if (S.body[k] == b) return k;
        return 0;
    };
    /* B2contactSolver::new: the position constraints (their velocity part is made again below) */
    for (int q = 0; q < nc; ++q) {
        const int ci = S.con[q];
        const int2 bd = w.c.body[ci];
        const int ia = local(bd.x), ib = local(bd.y);
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
    /* integrate positions over the rest of the step and synchronise the bodies */
    const float h = (1.0f - alpha) * sp.dt;
    for (int k = 0; k < nb; ++k) {
        const int b = S.body[k];
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
        for (int e = w.b_fix_off[b]; e < w.b_fix_off[b + 1]; ++e) {
            const int f = w.b_fix[e];
            if (!sync_fixture(w, f, xf1, xf2)) continue;
            const int slot = atomicAdd(&w.cnt[CNT_TOI_MOVED], 1);
            if (slot < kToiMovedCap) w.t_moved[slot] = f;
            else toi_overflow(w);
            if (!w.f_pmoved[f]) {
                w.f_pmoved[f] = 1;
                const int ps = atomicAdd(&w.cnt[CNT_TOI_PMOVED], 1);
                if (ps < kToiPassMovedCap) w.t_pmoved[ps] = f;
                else toi_overflow(w);
            }
        }
    }
    atomicAdd(&w.cnt[CNT_TOI_EVENTS], 1);
}

__global__ void __launch_bounds__(kTBlock) k_continuous(DevWorld w, StepParams sp) {
    __shared__ IslandScratch S;
    grid_barrier_start();
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = gridDim.x * blockDim.x;
    const int n_tab = w.cnt[CNT_CONTACTS];
    const bool rec = sp.record_events != 0;
    volatile int* vcnt = w.cnt;

    /* B2world::solve_toi with a complete step: alpha0 = 0, no body in an island */
    for (int b = gtid; b < w.n_bodies; b += gstride) {
        w.b_alpha0[b] = 0.0f;
        w.b_stamp[b] = -1;
        w.b_inval[b] = -1;
        w.b_sync[b] = 0u;
    }
    for (int wd = gtid; wd < w.num_worlds; wd += gstride) {
        w.tw_alpha[wd] = kNoAlpha;
        w.tw_key[wd] = ~0ull;
        w.tw_event[wd] = make_int4(-1, -1, -1, -1);
    }
    if (!grid_barrier(w)) return;

    int iter = 0;
    for (; iter < kMaxIters; ++iter) {
        const int n_all = n_tab + appended(w, n_tab);
        /* phase 1: times of impact (private/dynamics/b2_world.rs:564-693) */
        for (int i = gtid; i < n_all; i += gstride) {
            if (iter == 0 && i < n_tab) {
                /* contacts of the table start the pass with no time of impact and no events */
                const uint8_t e = toi_eligible(w, i);
                w.t_elig[i] = e;
                w.t_count[i] = 0;
                w.t_when[i] = -1;
                w.t_stamp[i] = -1;
                if (!e) continue;
            } else if (!w.t_elig[i]) {
                continue;
            }
            if (!(w.c.flags[i] & CF_ENABLED)) continue;
            if (w.t_count[i] > kMaxSubSteps) continue;
            const int2 bd = w.c.body[i];
            float alpha;
            const int when = w.t_when[i];
            if (when >= 0 && when > w.b_inval[bd.x] && when > w.b_inval[bd.y]) {
                alpha = w.t_toi[i];
            } else {
                const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
                const bool activeA = (fa & BF_AWAKE) && !static_body(fa);
                const bool activeB = (fb & BF_AWAKE) && !static_body(fb);
                if (!activeA && !activeB) continue;
                Sweep sa = load_sweep(w, bd.x), sb = load_sweep(w, bd.y);
                float alpha0 = sa.alpha0;
                if (sa.alpha0 < sb.alpha0) {
                    alpha0 = sb.alpha0;
                    sweep_advance(sa, alpha0);
                    request_advance(w, bd.x, alpha0);
                } else if (sb.alpha0 < sa.alpha0) {
                    alpha0 = sa.alpha0;
                    sweep_advance(sb, alpha0);
                    request_advance(w, bd.y, alpha0);
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
                atomicMin(&w.tw_alpha[w.b_world[bd.x]], __float_as_uint(alpha));
                const int slot = atomicAdd(&w.cnt[CNT_TOI_HITS], 1);
                if (slot < w.contact_cap) w.t_hits[slot] = i;
            }
        }
        if (!grid_barrier(w)) return;
        const int hits = min(vcnt[CNT_TOI_HITS], w.contact_cap);
        if (hits == 0) break;

        /* phase 2: commit the sweep advances; the event of each world is its smallest key among
         * the contacts with the smallest alpha */
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
            const int wd = (int)w.b_world[w.c.body[i].x];
            if (__float_as_uint(w.t_toi[i]) == w.tw_alpha[wd]) atomicMin(&w.tw_key[wd], w.c.key[i]);
        }
        const int nmoved_prev = min(vcnt[CNT_TOI_MOVED], kToiMovedCap);
        for (int j = gtid; j < nmoved_prev; j += gstride) w.f_moved[w.t_moved[j]] = 0;
        if (!grid_barrier(w)) return;

        /* phase 3: advance the event's bodies and update its contact (b2_world.rs:695-739) */
        if (gtid == 0) {
            vcnt[CNT_TOI_HITS] = 0;
            vcnt[CNT_TOI_SYNC] = 0;
            vcnt[CNT_TOI_MOVED] = 0;
        }
        for (int wd = gtid; wd < w.num_worlds; wd += gstride) {
            const uint32_t ab = w.tw_alpha[wd];
            if (ab == kNoAlpha) continue;
            const unsigned long long key = w.tw_key[wd];
            w.tw_alpha[wd] = kNoAlpha;
            w.tw_key[wd] = ~0ull;
            const float alpha = __uint_as_float(ab);
            const int i = find_contact(w, n_tab, n_all, key);
            if (i < 0) {
                toi_overflow(w);
                continue;
            }
            const int2 bd = w.c.body[i];
            const Sweep s1 = load_sweep(w, bd.x), s2 = load_sweep(w, bd.y);
            body_advance(w, bd.x, alpha);
            body_advance(w, bd.y, alpha);
            const bool touching = contact_update(w, rec, i, w.c.flags[i], w.c.fix[i], bd, w.c.mids[i]);
            w.t_when[i] = -1;
            w.t_count[i] += 1;
            if (!touching) {
                w.c.flags[i] &= ~CF_ENABLED;
                restore_body(w, bd.x, s1);
                restore_body(w, bd.y, s2);
                w.tw_event[wd] = make_int4(i, bd.x, bd.y, -1);
                continue;
            }
            wake_body(w, bd.x);
            wake_body(w, bd.y);
            w.b_stamp[bd.x] = iter;
            w.b_stamp[bd.y] = iter;
            w.t_stamp[i] = iter;
            w.tw_event[wd] = make_int4(i, bd.x, bd.y, iter);
            w.tw_ealpha[wd] = alpha;
            w.tw_cand[(size_t)wd * (kToiCand + 1)] = 0;
        }
        if (!grid_barrier(w)) return;

        /* phase 4: the event bodies' other contacts with static, kinematic or bullet partners */
        for (int i = gtid; i < n_all; i += gstride) {
            const int2 bd = w.c.body[i];
            const bool sx = w.b_stamp[bd.x] == iter, sy = w.b_stamp[bd.y] == iter;
            if (!sx && !sy) continue;
            if (w.t_stamp[i] == iter) continue;
            const uint32_t fx = w.b_flags[bd.x], fy = w.b_flags[bd.y];
            const bool viaA = sx && dynamic_body(fx), viaB = sy && dynamic_body(fy);
            if (!viaA && !viaB) continue;
            const uint32_t fbody = viaA ? fx : fy, fother = viaA ? fy : fx;
            if (dynamic_body(fother) && !(fbody & BF_BULLET) && !(fother & BF_BULLET)) continue;
            if (w.c.flags[i] & CF_SENSOR) continue;
            int* cand = w.tw_cand + (size_t)w.b_world[bd.x] * (kToiCand + 1);
            const int slot = atomicAdd(cand, 1);
            if (slot < kToiCand) cand[1 + slot] = i;
            else toi_overflow(w);
        }
        if (!grid_barrier(w)) return;

        /* phase 5: the islands (b2_world.rs:741-893) */
        if (threadIdx.x == 0) {
            for (int wd = blockIdx.x; wd < w.num_worlds; wd += gridDim.x)
                if (w.tw_event[wd].w == iter) event_island(w, sp, S, wd, iter);
        }
        if (!grid_barrier(w)) return;

        /* phase 6: find_new_contacts for the proxies this iteration moved */
        const int nm = min(vcnt[CNT_TOI_MOVED], kToiMovedCap);
        const int npm = min(vcnt[CNT_TOI_PMOVED], kToiPassMovedCap);
        const long long items = (long long)nm * (1 + npm);
        for (long long it = gtid; it < items; it += gstride) {
            const int qi = (int)(it % nm);
            const int q = w.t_moved[qi];
            const uint32_t wd = w.b_world[w.f_body[q]];
            const float4 box = w.f_fat[q];
            if (it < nm) {
                /* the step's hierarchy: leaves of proxies not moved in this pass are current */
                for (int h = 0; h < 2; ++h) {
                    const int root = w.bp_world_root[wd + (h ? (uint32_t)w.num_worlds : 0u)];
                    if (root == INT_MIN) continue;
                    if (root < 0) {
                        const int p = (int)w.bp_val[~root];
                        if (!w.f_pmoved[p] && box_overlap(w.bp_leaf[~root], box)) toi_pair(w, q, p, n_tab, n_all);
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
                            if (kids[c] < 0) {
                                const int p = (int)w.bp_val[~kids[c]];
                                if (!w.f_pmoved[p]) toi_pair(w, q, p, n_tab, n_all);
                            } else if (top < kStack) {
                                stack[top++] = kids[c];
                            } else {
                                atomicOr((unsigned*)&w.cnt[CNT_STATUS], ST_STACK_OVERFLOW);
                            }
                        }
                    }
                }
            } else {
                /* proxies moved earlier in the pass, with their current fat AABBs */
                const int p = w.t_pmoved[(int)(it / nm) - 1];
                if (w.b_world[w.f_body[p]] != wd) continue;
                if (box_overlap(w.f_fat[p], box)) toi_pair(w, q, p, n_tab, n_all);
            }
        }
        if (!grid_barrier(w)) return;
    }
    if (iter == kMaxIters) toi_overflow(w);

    /* the pass is over: clear its moved flags, merge its new contacts into the sorted table */
    if (gtid == 0) vcnt[CNT_TOI_ITERS] = iter;
    {
        const int nm = min(vcnt[CNT_TOI_MOVED], kToiMovedCap);
        for (int j = gtid; j < nm; j += gstride) w.f_moved[w.t_moved[j]] = 0;
        const int npm = min(vcnt[CNT_TOI_PMOVED], kToiPassMovedCap);
        for (int j = gtid; j < npm; j += gstride) w.f_pmoved[w.t_pmoved[j]] = 0;
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
    DevWorld wc = w;
    StepParams p = sp;
    void* args[] = {&wc, &p};
    cudaMemsetAsync(w.cnt + CNT_TOI_FIRST, 0, (CNT_TOI_LAST - CNT_TOI_FIRST) * sizeof(int), s);
    cudaMemsetAsync(w.cnt + CNT_BARRIER, 0, sizeof(int), s);
    B2G_LAUNCHED(1);
    return (int)cudaLaunchCooperativeKernel((const void*)k_continuous, dim3(num_sms), dim3(kTBlock), args, 0, s);
}

}  // namespace b2g
