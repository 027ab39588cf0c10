/*
 * b2g_solver_math.cuh — per-constraint arithmetic of B2contactSolver and the fixture
 * synchronisation, shared by the step's solver (k_solver.cu) and the continuous-physics pass
 * (k_continuous.cu).
 *
 * Reference: B2contactSolver::new + initialize_velocity_constraints, warm_start,
 * solve_velocity_constraints, solve_position_constraints and solve_toi_position_constraints
 * (src/private/dynamics/b2_contact_solver_private.rs:20-823); b2_world_manifold_initialize
 * (private/collision/b2_collision.rs:7-68); b2_fixture_synchronize
 * (private/dynamics/b2_fixture.rs:147-173) with B2dynamicTree::move_proxy
 * (private/collision/b2_dynamic_tree.rs:109-168). Each routine is the reference's sequence of
 * IEEE f32 operations (built without fused multiply-add).
 */
#ifndef B2G_SOLVER_MATH_CUH
#define B2G_SOLVER_MATH_CUH

#include "b2g_internal.h"

namespace b2g {
namespace {

/* One constraint slot's velocity data (vc_* arrays); idx = (body code A, body code B, point count,
 * flags). A body code is the body index in the global arrays, or in the part-local solve the
 * body's place in the block's shared-memory cache (>= 0) or -(index + 1) for a body read from
 * global memory. */
struct VelSlot {
    int4 idx;
    float4 inv, nf, imp, r0, r1, m0, m1, k;
};

/* One constraint slot's position data (pc_* arrays), idx as in VelSlot */
struct PosSlot {
    int4 idx;
    float4 lp, geo, lc, inv, meta;
    int island;
    int pad[3];        /* pad[0]: cached early-exit flag of the island (part-local solve) */
};

/* What B2contactSolver::new and initialize_velocity_constraints read for one contact: its
 * material and manifold, the warm-start impulses already scaled by dt_ratio (zero without warm
 * starting), the bodies' masses, local centres, positions (c, a), velocities and rotations
 * (rot(a)), the shapes' radii; ia, ib and flags go to the slot's index word as given. */
struct ConstraintIn {
    float4 mat, geo, pts, imp;
    int mtype, count, ia, ib, flags;
    float mA, iA, mB, iB, rA, rB;
    float2 lcA, lcB;
    V2 cA, cB, vA, vB;
    float wA, wB;
    Rot qA, qB;
};

/* B2contactSolver::new + initialize_velocity_constraints for one contact */
__device__ __forceinline__ void make_constraint(const ConstraintIn& in, VelSlot& vs, PosSlot& ps) {
    const float4 mat = in.mat, geo = in.geo, pts = in.pts;
    const int mtype = in.mtype, count = in.count;
    const float mA = in.mA, iA = in.iA, mB = in.mB, iB = in.iB;
    const float rA = in.rA, rB = in.rB;
    const float2 lcA = in.lcA, lcB = in.lcB;
    const V2 cA = in.cA, cB = in.cB, vA = in.vA, vB = in.vB;
    const float wA = in.wA, wB = in.wB;
    Xf xfA, xfB;
    xfA.q = in.qA;
    xfB.q = in.qB;
    xfA.p = sub(cA, mul(xfA.q, mk(lcA.x, lcA.y)));
    xfB.p = sub(cB, mul(xfB.q, mk(lcB.x, lcB.y)));
    /* b2_world_manifold_initialize, private/collision/b2_collision.rs:7-68 */
    V2 normal = mk(1.0f, 0.0f);
    V2 wp[2] = {mk(0.0f, 0.0f), mk(0.0f, 0.0f)};
    const V2 ln = mk(geo.x, geo.y), lpt = mk(geo.z, geo.w);
    const V2 lp[2] = {mk(pts.x, pts.y), mk(pts.z, pts.w)};
    if (mtype == MANIFOLD_CIRCLES) {
        V2 pa = mul(xfA, lpt);
        V2 pb = mul(xfB, lp[0]);
        if (dist_sq(pa, pb) > kEpsilon * kEpsilon) {
            normal = sub(pb, pa);
            normalize(normal);
        }
        V2 ca = add(pa, scale(rA, normal));
        V2 cb = sub(pb, scale(rB, normal));
        wp[0] = scale(0.5f, add(ca, cb));
    } else if (mtype == MANIFOLD_FACE_A) {
        normal = mul(xfA.q, ln);
        V2 plane = mul(xfA, lpt);
        for (int j = 0; j < count; ++j) {
            V2 clip = mul(xfB, lp[j]);
            V2 ca = add(clip, scale(rA - dot(sub(clip, plane), normal), normal));
            V2 cb = sub(clip, scale(rB, normal));
            wp[j] = scale(0.5f, add(ca, cb));
        }
    } else {
        normal = mul(xfB.q, ln);
        V2 plane = mul(xfB, lpt);
        for (int j = 0; j < count; ++j) {
            V2 clip = mul(xfA, lp[j]);
            V2 cb = add(clip, scale(rB - dot(sub(clip, plane), normal), normal));
            V2 ca = sub(clip, scale(rA, normal));
            wp[j] = scale(0.5f, add(ca, cb));
        }
        normal = neg(normal);
    }
    V2 ra[2], rb[2];
    float nm[2] = {0.0f, 0.0f}, tm[2] = {0.0f, 0.0f}, bias[2] = {0.0f, 0.0f};
    const V2 tangent = cross_vs(normal, 1.0f);
    for (int j = 0; j < 2; ++j) {
        ra[j] = mk(0.0f, 0.0f);
        rb[j] = mk(0.0f, 0.0f);
    }
    for (int j = 0; j < count; ++j) {
        ra[j] = sub(wp[j], cA);
        rb[j] = sub(wp[j], cB);
        float rnA = cross(ra[j], normal);
        float rnB = cross(rb[j], normal);
        float kNormal = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        nm[j] = kNormal > 0.0f ? fdiv(1.0f, kNormal) : 0.0f;
        float rtA = cross(ra[j], tangent);
        float rtB = cross(rb[j], tangent);
        float kTangent = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
        tm[j] = kTangent > 0.0f ? fdiv(1.0f, kTangent) : 0.0f;
        float vRel = dot(normal, sub(sub(add(vB, cross_sv(wB, rb[j])), vA), cross_sv(wA, ra[j])));
        if (vRel < -mat.z) bias[j] = -mat.y * vRel;
    }
    int vcount = count;
    float k11 = 0.0f, k12 = 0.0f, k22 = 0.0f, na = 0.0f, nb = 0.0f, nd = 0.0f;
    if (count == 2) {
        float rn1A = cross(ra[0], normal);
        float rn1B = cross(rb[0], normal);
        float rn2A = cross(ra[1], normal);
        float rn2B = cross(rb[1], normal);
        k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
        k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
        k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
        const float kMaxConditionNumber = 1000.0f;
        if (k11 * k11 < kMaxConditionNumber * (k11 * k22 - k12 * k12)) {
            /* B2Mat22::get_inverse of [[k11, k12], [k12, k22]] */
            float det = k11 * k22 - k12 * k12;
            if (det != 0.0f) det = fdiv(1.0f, det);
            na = det * k22;      /* ex.x */
            /* ex.y = -det * k12 equals ey.x (K is symmetric) */
            nb = -det * k12;     /* ey.x */
            nd = det * k11;      /* ey.y */
        } else {
            vcount = 1;
            k11 = k12 = k22 = 0.0f;
        }
    }
    vs.idx = make_int4(in.ia, in.ib, vcount, in.flags);
    vs.inv = make_float4(mA, mB, iA, iB);
    vs.nf = make_float4(normal.x, normal.y, mat.x, mat.w);
    vs.r0 = make_float4(ra[0].x, ra[0].y, rb[0].x, rb[0].y);
    vs.r1 = make_float4(ra[1].x, ra[1].y, rb[1].x, rb[1].y);
    /* the inverse's off-diagonal (nb == nc) and ey.y ride in the spare lanes */
    vs.m0 = make_float4(nm[0], tm[0], bias[0], nb);
    vs.m1 = make_float4(nm[1], tm[1], bias[1], nd);
    vs.imp = in.imp;
    /* K = [[k11, k12], [k12, k22]] and its inverse ([[na, nb], [nc, nd]], nb == nc) */
    vs.k = make_float4(k11, k12, k22, na);
    ps.idx = vs.idx;
    ps.lp = make_float4(lp[0].x, lp[0].y, lp[1].x, lp[1].y);
    ps.geo = make_float4(ln.x, ln.y, lpt.x, lpt.y);
    ps.lc = make_float4(lcA.x, lcA.y, lcB.x, lcB.y);
    ps.inv = make_float4(mA, mB, iA, iB);
    ps.meta = make_float4(rA, rB, __int_as_float(mtype), __int_as_float(count));
    ps.island = 0;
    ps.pad[0] = ps.pad[1] = ps.pad[2] = 0;
}

/* warm_start for one slot on the bodies' velocities (v, w, sleep time) va, vb */
__device__ __forceinline__ void warm_math(const VelSlot& sl, float4& va, float4& vb) {
    const int4 idx = sl.idx;
    const float4 inv = sl.inv;
    const float4 nf = sl.nf;
    const float4 imp = sl.imp;
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const V2 normal = mk(nf.x, nf.y);
    const V2 tangent = cross_vs(normal, 1.0f);
    const float4 r[2] = {sl.r0, sl.r1};
    const float ni[2] = {imp.x, imp.z}, ti[2] = {imp.y, imp.w};
    for (int j = 0; j < idx.z; ++j) {
        const V2 rA = mk(r[j].x, r[j].y), rB = mk(r[j].z, r[j].w);
        const V2 P = add(scale(ni[j], normal), scale(ti[j], tangent));
        wA -= inv.z * cross(rA, P);
        vA = sub(vA, scale(inv.x, P));
        wB += inv.w * cross(rB, P);
        vB = add(vB, scale(inv.y, P));
    }
    va = make_float4(vA.x, vA.y, wA, va.w);
    vb = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_velocity_constraints for one slot: updates its impulses imp and the velocities va, vb */
__device__ __forceinline__ void solve_velocity_math(const VelSlot& sl, float4& imp, float4& va, float4& vb) {
    const int4 idx = sl.idx;
    const float4 inv = sl.inv;
    const float4 nf = sl.nf;
    const float4 r0 = sl.r0, r1 = sl.r1;
    const float4 m0 = sl.m0, m1 = sl.m1;
    const float mA = inv.x, mB = inv.y, iA = inv.z, iB = inv.w;
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const V2 normal = mk(nf.x, nf.y);
    const V2 tangent = cross_vs(normal, 1.0f);
    const float friction = nf.z;
    const V2 rA0 = mk(r0.x, r0.y), rB0 = mk(r0.z, r0.w), rA1 = mk(r1.x, r1.y), rB1 = mk(r1.z, r1.w);
    /* friction first (b2_contact_solver_private.rs:295-323) */
    {
        V2 dv = sub(sub(add(vB, cross_sv(wB, rB0)), vA), cross_sv(wA, rA0));
        float vt = dot(dv, tangent) - nf.w;
        float lambda = m0.y * (-vt);
        float maxFriction = friction * imp.x;
        float newImpulse = fclampr(imp.y + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - imp.y;
        imp.y = newImpulse;
        V2 P = scale(lambda, tangent);
        vA = sub(vA, scale(mA, P));
        wA -= iA * cross(rA0, P);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB0, P);
    }
    if (idx.z == 2) {
        V2 dv = sub(sub(add(vB, cross_sv(wB, rB1)), vA), cross_sv(wA, rA1));
        float vt = dot(dv, tangent) - nf.w;
        float lambda = m1.y * (-vt);
        float maxFriction = friction * imp.z;
        float newImpulse = fclampr(imp.w + lambda, -maxFriction, maxFriction);
        lambda = newImpulse - imp.w;
        imp.w = newImpulse;
        V2 P = scale(lambda, tangent);
        vA = sub(vA, scale(mA, P));
        wA -= iA * cross(rA1, P);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB1, P);
    }
    if (idx.z == 1) {
        V2 dv = sub(sub(add(vB, cross_sv(wB, rB0)), vA), cross_sv(wA, rA0));
        float vn = dot(dv, normal);
        float lambda = -m0.x * (vn - m0.z);
        float newImpulse = fmaxr(imp.x + lambda, 0.0f);
        lambda = newImpulse - imp.x;
        imp.x = newImpulse;
        V2 P = scale(lambda, normal);
        vA = sub(vA, scale(mA, P));
        wA -= iA * cross(rA0, P);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB0, P);
    } else {
        /* 2-point block LCP, b2_contact_solver_private.rs:380-575 */
        const float4 K = sl.k;
        const float k11 = K.x, k12 = K.y, k22 = K.z;
        const float na = K.w, nbc = m0.w, nd = m1.w;
        const V2 a = mk(imp.x, imp.z);
        V2 dv1 = sub(sub(add(vB, cross_sv(wB, rB0)), vA), cross_sv(wA, rA0));
        V2 dv2 = sub(sub(add(vB, cross_sv(wB, rB1)), vA), cross_sv(wA, rA1));
        float vn1 = dot(dv1, normal);
        float vn2 = dot(dv2, normal);
        V2 b = mk(vn1 - m0.z, vn2 - m1.z);
        /* b -= K * a */
        b = sub(b, mk(k11 * a.x + k12 * a.y, k12 * a.x + k22 * a.y));
        V2 x;
        bool solved = false;
        /* case 1: x = -inv(K) b */
        x = neg(mk(na * b.x + nbc * b.y, nbc * b.x + nd * b.y));
        if (x.x >= 0.0f && x.y >= 0.0f) solved = true;
        if (!solved) {
            x.x = -m0.x * b.x;
            x.y = 0.0f;
            vn2 = k12 * x.x + b.y;
            if (x.x >= 0.0f && vn2 >= 0.0f) solved = true;
        }
        if (!solved) {
            x.x = 0.0f;
            x.y = -m1.x * b.y;
            vn1 = k12 * x.y + b.x;
            if (x.y >= 0.0f && vn1 >= 0.0f) solved = true;
        }
        if (!solved) {
            x.x = 0.0f;
            x.y = 0.0f;
            vn1 = b.x;
            vn2 = b.y;
            if (vn1 >= 0.0f && vn2 >= 0.0f) solved = true;
        }
        if (solved) {
            V2 d = sub(x, a);
            V2 P1 = scale(d.x, normal);
            V2 P2 = scale(d.y, normal);
            vA = sub(vA, scale(mA, add(P1, P2)));
            wA -= iA * (cross(rA0, P1) + cross(rA1, P2));
            vB = add(vB, scale(mB, add(P1, P2)));
            wB += iB * (cross(rB0, P1) + cross(rB1, P2));
            imp.x = x.x;
            imp.z = x.y;
        }
    }
    va = make_float4(vA.x, vA.y, wA, va.w);
    vb = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_position_constraints for one slot on the bodies' (c, a) pa, pb; returns this slot's min
 * separation (<= 0). baumgarte: kBaumgarte, or kToiBaumgarte for the time-of-impact solve
 * (solve_toi_position_constraints, b2_contact_solver_private.rs:733-823, which also zeroes the
 * masses of bodies other than the event's two in the slot it passes) */
__device__ __forceinline__ float solve_position_math(const PosSlot& sl, float4& pa, float4& pb,
                                                     float baumgarte = kBaumgarte) {
    const float4 lp = sl.lp, geo = sl.geo, lc = sl.lc, inv = sl.inv, meta = sl.meta;
    const float mA = inv.x, mB = inv.y, iA = inv.z, iB = inv.w;
    const V2 lcA = mk(lc.x, lc.y), lcB = mk(lc.z, lc.w);
    const int mtype = __float_as_int(meta.z);
    const int count = __float_as_int(meta.w);
    const float rA = meta.x, rB = meta.y;
    const V2 ln = mk(geo.x, geo.y), lpt = mk(geo.z, geo.w);
    const V2 lps[2] = {mk(lp.x, lp.y), mk(lp.z, lp.w)};
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    float minSep = 0.0f;
    for (int j = 0; j < count; ++j) {
        Xf xfA, xfB;
        xfA.q = rot(aA);
        xfB.q = rot(aB);
        xfA.p = sub(cA, mul(xfA.q, lcA));
        xfB.p = sub(cB, mul(xfB.q, lcB));
        V2 normal, point;
        float separation;
        if (mtype == MANIFOLD_CIRCLES) {
            V2 pA = mul(xfA, lpt);
            V2 pB = mul(xfB, lps[0]);
            normal = sub(pB, pA);
            normalize(normal);
            point = scale(0.5f, add(pA, pB));
            separation = dot(sub(pB, pA), normal) - rA - rB;
        } else if (mtype == MANIFOLD_FACE_A) {
            normal = mul(xfA.q, ln);
            V2 plane = mul(xfA, lpt);
            V2 clip = mul(xfB, lps[j]);
            separation = dot(sub(clip, plane), normal) - rA - rB;
            point = clip;
        } else {
            normal = mul(xfB.q, ln);
            V2 plane = mul(xfB, lpt);
            V2 clip = mul(xfA, lps[j]);
            separation = dot(sub(clip, plane), normal) - rA - rB;
            point = clip;
            normal = neg(normal);
        }
        V2 ra = sub(point, cA);
        V2 rb = sub(point, cB);
        minSep = fminr(minSep, separation);
        float C = fclampr(baumgarte * (separation + kLinearSlop), -kMaxLinearCorrection, 0.0f);
        float rnA = cross(ra, normal);
        float rnB = cross(rb, normal);
        float K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        float impulse = K > 0.0f ? fdiv(-C, K) : 0.0f;
        V2 P = scale(impulse, normal);
        cA = sub(cA, scale(mA, P));
        aA -= iA * cross(ra, P);
        cB = add(cB, scale(mB, P));
        aB += iB * cross(rb, P);
    }
    pa = make_float4(cA.x, cA.y, aA, pa.w);
    pb = make_float4(cB.x, cB.y, aB, pb.w);
    return minSep;
}


/* B2dynamicTree::move_proxy, private/collision/b2_dynamic_tree.rs:109-168 (fat AABB rule only);
 * returns whether the proxy moved (got a new fat AABB and the moved flag) */
__device__ __forceinline__ bool move_proxy(const DevWorld& w, int f, const AABB& aabb, V2 disp) {
    const V2 r = mk(kAabbExtension, kAabbExtension);
    AABB fat;
    fat.lo = sub(aabb.lo, r);
    fat.hi = add(aabb.hi, r);
    const V2 d = scale(kAabbMultiplier, disp);
    if (d.x < 0.0f) fat.lo.x += d.x; else fat.hi.x += d.x;
    if (d.y < 0.0f) fat.lo.y += d.y; else fat.hi.y += d.y;
    const float4 t = w.f_fat[f];
    AABB tree;
    tree.lo = mk(t.x, t.y);
    tree.hi = mk(t.z, t.w);
    if (contains(tree, aabb)) {
        AABB huge;
        huge.lo = sub(fat.lo, scale(4.0f, r));
        huge.hi = add(fat.hi, scale(4.0f, r));
        if (contains(huge, tree)) return false;
    }
    w.f_fat[f] = make_float4(fat.lo.x, fat.lo.y, fat.hi.x, fat.hi.y);
    w.f_moved[f] = 1;
    return true;
}

/* b2_fixture_synchronize, private/dynamics/b2_fixture.rs:147-173 (for each of the fixture's proxies:
 * none for a destroyed fixture or one on a disabled body); returns whether the proxy moved */
__device__ __forceinline__ bool sync_fixture(const DevWorld& w, int f, const Xf& xf1, const Xf& xf2) {
    if (w.f_refid[f] == 0xffffffffu) return false;
    const ShapeRec s = w.f_shape[f];
    AABB a1, a2;
    shape_aabb(s, xf1, a1);
    shape_aabb(s, xf2, a2);
    const AABB swept = combine(a1, a2);
    const V2 disp = sub(center(a2), center(a1));
    return move_proxy(w, f, swept, disp);
}

}  // namespace
}  // namespace b2g
#endif
