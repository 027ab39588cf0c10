/*
 * b2g_joint.cuh — the joints on the device: revolute, prismatic, wheel, pulley, distance, weld,
 * friction, motor, mouse and gear, each a restatement of its reference file's
 * init_velocity_constraints / solve_velocity_constraints / solve_position_constraints in the same
 * sequence of IEEE f32 operations (built without fused multiply-add). The revolute joint (B2revoluteJoint,
 * private/dynamics/joints/b2_revolute_joint.rs:21-287): init_velocity_constraints (anchors,
 * effective masses, warm start), solve_velocity_constraints (motor, lower and upper limits, the
 * point constraint) and solve_position_constraints (angular limit, then the point), each the
 * reference's sequence of IEEE f32 operations (built without fused multiply-add).
 *
 * Joint j's definition: j_body (A, B), j_anchor (local anchor A, local anchor B), j_lim
 * (reference angle, lower, upper, motor speed), j_par (max motor torque, flag bits); its impulses
 * (kept across steps for warm starting): j_imp (x, y, motor, lower), j_imp2.x (upper); the
 * step's temporaries: j_rr (rA, rB), j_k (K ex.x, ex.y, ey.x, ey.y), j_m (1/mA, 1/mB, 1/IA, 1/IB),
 * j_s (axial mass, angle). Bodies are read and written in the global arrays; only dynamic bodies
 * are written (the others have zero inverse mass, so the reference leaves them unchanged).
 */
#ifndef B2G_JOINT_CUH
#define B2G_JOINT_CUH

#include "b2g.h"
#include "b2g_internal.h"

namespace b2g {
namespace {

constexpr float kAngularSlop = 2.0f / 180.0f * kPi;           /* B2_ANGULAR_SLOP */
constexpr float kMaxAngularCorrection = 8.0f / 180.0f * kPi;  /* B2_MAX_ANGULAR_CORRECTION */

__device__ __forceinline__ bool joint_body_dynamic(const DevWorld& w, int b) {
    return (w.b_flags[b] & BF_TYPE_MASK) == BODY_DYNAMIC;
}

/* B2Mat22::solve, src/b2_math.rs:278-293 */
__device__ __forceinline__ V2 mat22_solve(float a11, float a21, float a12, float a22, V2 b) {
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = fdiv(1.0f, det);
    return mk(det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x));
}

/* ---- distance joint (B2distanceJoint, private/dynamics/joints/b2_distance_joint.rs:78-319) ----
 * j_lim = (rest length, min length, max length, stiffness), j_par.x = damping, j_imp = (impulse,
 * lower, upper, -); the step's temporaries j_rr (rA, rB), j_k (u, current length, mass), j_s
 * (gamma, bias), j_imp2.y (soft mass). */

__device__ __forceinline__ void distance_apply(V2& vA, float& wA, V2& vB, float& wB, const float4& m, V2 rA, V2 rB,
                                               V2 P) {
    vA = sub(vA, scale(m.x, P));
    wA -= m.z * cross(rA, P);
    vB = add(vB, scale(m.y, P));
    wB += m.w * cross(rB, P);
}

/* init_velocity_constraints, :78-181 */
__device__ void distance_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float damping = w.j_par[j].x;
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float4 m = make_float4(massA.y, massB.y, massA.w, massB.w);
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(pa.z), qB = rot(pb.z);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    V2 u = sub(sub(add(mk(pb.x, pb.y), rB), mk(pa.x, pa.y)), rA);
    float4 imp = w.j_imp[j];
    const float current = length(u);
    if (current > kLinearSlop) {
        const float inv = fdiv(1.0f, current);
        u.x *= inv;
        u.y *= inv;
    } else {
        u = mk(0.0f, 0.0f);
        imp.x = 0.0f;
        imp.y = 0.0f;
        imp.z = 0.0f;
    }
    const float crAu = cross(rA, u);
    const float crBu = cross(rB, u);
    float inv_mass = m.x + m.z * crAu * crAu + m.y + m.w * crBu * crBu;
    const float mass = inv_mass != 0.0f ? fdiv(1.0f, inv_mass) : 0.0f;
    float gamma, bias, soft_mass;
    if (lim.w > 0.0f && lim.y < lim.z) {
        const float C = current - lim.x;
        const float d = damping;
        const float k = lim.w;
        const float h = sp.dt;
        gamma = h * (d + h * k);
        gamma = gamma != 0.0f ? fdiv(1.0f, gamma) : 0.0f;
        bias = C * h * k * gamma;
        inv_mass += gamma;
        soft_mass = inv_mass != 0.0f ? fdiv(1.0f, inv_mass) : 0.0f;
    } else {
        gamma = 0.0f;
        bias = 0.0f;
        soft_mass = mass;
    }
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        const V2 P = scale(imp.x + imp.y - imp.z, u);
        distance_apply(vA, wA, vB, wB, m, rA, rB, P);
    } else {
        imp.x = 0.0f;  /* the reference zeroes only the spring impulse here */
    }
    w.j_imp[j] = imp;
    w.j_rr[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    w.j_k[j] = make_float4(u.x, u.y, current, mass);
    w.j_m[j] = m;
    w.j_s[j] = make_float2(gamma, bias);
    w.j_imp2[j].y = soft_mass;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_velocity_constraints, :183-274 */
__device__ void distance_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 lim = w.j_lim[j];
    const float4 m = w.j_m[j];
    const float4 rr = w.j_rr[j];
    const V2 rA = mk(rr.x, rr.y), rB = mk(rr.z, rr.w);
    const float4 uk = w.j_k[j];
    const V2 u = mk(uk.x, uk.y);
    const float current = uk.z, mass = uk.w;
    const float2 gb = w.j_s[j];
    const float soft_mass = w.j_imp2[j].y;
    float4 imp = w.j_imp[j];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    if (lim.y < lim.z) {
        if (lim.w > 0.0f) {
            const V2 vpA = add(vA, cross_sv(wA, rA));
            const V2 vpB = add(vB, cross_sv(wB, rB));
            const float cdot = dot(u, sub(vpB, vpA));
            const float impulse = -soft_mass * (cdot + gb.y + gb.x * imp.x);
            imp.x += impulse;
            distance_apply(vA, wA, vB, wB, m, rA, rB, scale(impulse, u));
        }
        {
            const float C = current - lim.y;
            const float bias = fmaxr(0.0f, C) * sp.inv_dt;
            const V2 vpA = add(vA, cross_sv(wA, rA));
            const V2 vpB = add(vB, cross_sv(wB, rB));
            const float cdot = dot(u, sub(vpB, vpA));
            float impulse = -mass * (cdot + bias);
            const float old_impulse = imp.y;
            imp.y = fmaxr(0.0f, imp.y + impulse);
            impulse = imp.y - old_impulse;
            distance_apply(vA, wA, vB, wB, m, rA, rB, scale(impulse, u));
        }
        {
            const float C = lim.z - current;
            const float bias = fmaxr(0.0f, C) * sp.inv_dt;
            const V2 vpA = add(vA, cross_sv(wA, rA));
            const V2 vpB = add(vB, cross_sv(wB, rB));
            const float cdot = dot(u, sub(vpA, vpB));
            float impulse = -mass * (cdot + bias);
            const float old_impulse = imp.z;
            imp.z = fmaxr(0.0f, imp.z + impulse);
            impulse = imp.z - old_impulse;
            distance_apply(vA, wA, vB, wB, m, rA, rB, scale(-impulse, u));
        }
    } else {
        const V2 vpA = add(vA, cross_sv(wA, rA));
        const V2 vpB = add(vB, cross_sv(wB, rB));
        const float cdot = dot(u, sub(vpB, vpA));
        const float impulse = -mass * cdot;
        imp.x += impulse;
        distance_apply(vA, wA, vB, wB, m, rA, rB, scale(impulse, u));
    }
    w.j_imp[j] = imp;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_position_constraints, :276-319 */
__device__ bool distance_solve_position(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 m = w.j_m[j];
    const float mass = w.j_k[j].w;
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    V2 u = sub(sub(add(cB, rB), cA), rA);
    const float len = normalize(u);
    float C;
    if (lim.y == lim.z) C = len - lim.y;
    else if (len < lim.y) C = len - lim.y;
    else if (lim.z < len) C = len - lim.z;
    else return true;
    const float impulse = -mass * C;
    const V2 P = scale(impulse, u);
    cA = sub(cA, scale(m.x, P));
    aA -= m.z * cross(rA, P);
    cB = add(cB, scale(m.y, P));
    aB += m.w * cross(rB, P);
    if (joint_body_dynamic(w, bd.x)) w.b_pos[bd.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, bd.y)) w.b_pos[bd.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return fabsr(C) < kLinearSlop;
}

/* ---- weld joint (B2weldJoint, private/dynamics/joints/b2_weld_joint.rs) with B2Mat33
 * (src/b2_math.rs:569-608, private/common/b2_math.rs:5-71) ----
 * j_lim = (reference angle, stiffness, damping, -), j_imp = (x, y, angular, -); the step's mass
 * matrix: columns ex = j_k.xyz, ey = (j_k.w, j_imp2.x, j_imp2.y), ez = (j_imp2.z, j_imp2.w, j_x.x);
 * j_s = (gamma, bias). */

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) {
    V3 r;
    r.x = x;
    r.y = y;
    r.z = z;
    return r;
}
__device__ __forceinline__ V3 v3add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 v3scale(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float v3dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 v3cross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
struct M33 {
    V3 ex, ey, ez;
};
__device__ __forceinline__ M33 weld_k(float mA, float mB, float iA, float iB, V2 rA, V2 rB) {
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
__device__ __forceinline__ void m33_inverse22(const M33& a, M33& m) {
    const float A = a.ex.x, B = a.ey.x, C = a.ex.y, D = a.ey.y;
    float det = A * D - B * C;
    if (det != 0.0f) det = fdiv(1.0f, det);
    m.ex = v3(det * D, -det * C, 0.0f);
    m.ey = v3(-det * B, det * A, 0.0f);
    m.ez = v3(0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ void m33_sym_inverse33(const M33& a, M33& m) {
    float det = v3dot(a.ex, v3cross(a.ey, a.ez));
    if (det != 0.0f) det = fdiv(1.0f, det);
    const float a11 = a.ex.x, a12 = a.ey.x, a13 = a.ez.x, a22 = a.ey.y, a23 = a.ez.y, a33 = a.ez.z;
    m.ex = v3(det * (a22 * a33 - a23 * a23), det * (a13 * a23 - a12 * a33), det * (a12 * a23 - a13 * a22));
    m.ey = v3(m.ex.y, det * (a11 * a33 - a13 * a13), det * (a13 * a12 - a11 * a23));
    m.ez = v3(m.ex.z, m.ey.z, det * (a11 * a22 - a12 * a12));
}
__device__ __forceinline__ V3 m33_solve33(const M33& a, V3 b) {
    float det = v3dot(a.ex, v3cross(a.ey, a.ez));
    if (det != 0.0f) det = fdiv(1.0f, det);
    return v3(det * v3dot(b, v3cross(a.ey, a.ez)), det * v3dot(a.ex, v3cross(b, a.ez)),
              det * v3dot(a.ex, v3cross(a.ey, b)));
}

/* init_velocity_constraints */
__device__ void weld_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float aA = w.b_pos[bd.x].z, aB = w.b_pos[bd.y].z;
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    const M33 k = weld_k(mA, mB, iA, iB, rA, rB);
    M33 mass;
    float gamma, bias;
    if (lim.y > 0.0f) {
        m33_inverse22(k, mass);
        float inv_m = iA + iB;
        const float C = aB - aA - lim.x;
        const float d = lim.z;
        const float kk = lim.y;
        const float h = sp.dt;
        gamma = h * (d + h * kk);
        gamma = gamma != 0.0f ? fdiv(1.0f, gamma) : 0.0f;
        bias = C * h * kk * gamma;
        inv_m += gamma;
        mass.ez.z = inv_m != 0.0f ? fdiv(1.0f, inv_m) : 0.0f;
    } else if (k.ez.z == 0.0f) {
        m33_inverse22(k, mass);
        gamma = 0.0f;
        bias = 0.0f;
    } else {
        m33_sym_inverse33(k, mass);
        gamma = 0.0f;
        bias = 0.0f;
    }
    float4 imp = w.j_imp[j];
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        const V2 P = mk(imp.x, imp.y);
        vA = sub(vA, scale(mA, P));
        wA -= iA * (cross(rA, P) + imp.z);
        vB = add(vB, scale(mB, P));
        wB += iB * (cross(rB, P) + imp.z);
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    w.j_imp[j] = imp;
    w.j_rr[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    w.j_k[j] = make_float4(mass.ex.x, mass.ex.y, mass.ex.z, mass.ey.x);
    w.j_imp2[j] = make_float4(mass.ey.y, mass.ey.z, mass.ez.x, mass.ez.y);
    w.j_x[j] = make_float4(mass.ez.z, 0.0f, 0.0f, 0.0f);
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(gamma, bias);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_velocity_constraints */
__device__ void weld_solve_velocity(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float stiffness = w.j_lim[j].y;
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 rA = mk(rr.x, rr.y), rB = mk(rr.z, rr.w);
    const float4 k0 = w.j_k[j], k1 = w.j_imp2[j];
    M33 mass;
    mass.ex = v3(k0.x, k0.y, k0.z);
    mass.ey = v3(k0.w, k1.x, k1.y);
    mass.ez = v3(k1.z, k1.w, w.j_x[j].x);
    const float2 gb = w.j_s[j];
    float4 imp = w.j_imp[j];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    if (stiffness > 0.0f) {
        const float cdot2 = wB - wA;
        const float impulse2 = -mass.ez.z * (cdot2 + gb.y + gb.x * imp.z);
        imp.z += impulse2;
        wA -= iA * impulse2;
        wB += iB * impulse2;
        const V2 cdot1 = sub(sub(add(vB, cross_sv(wB, rB)), vA), cross_sv(wA, rA));
        const V2 impulse1 = neg(mk(mass.ex.x * cdot1.x + mass.ey.x * cdot1.y, mass.ex.y * cdot1.x + mass.ey.y * cdot1.y));
        imp.x += impulse1.x;
        imp.y += impulse1.y;
        vA = sub(vA, scale(mA, impulse1));
        wA -= iA * cross(rA, impulse1);
        vB = add(vB, scale(mB, impulse1));
        wB += iB * cross(rB, impulse1);
    } else {
        const V2 cdot1 = sub(sub(add(vB, cross_sv(wB, rB)), vA), cross_sv(wA, rA));
        const float cdot2 = wB - wA;
        const V3 mc = v3add(v3add(v3scale(cdot1.x, mass.ex), v3scale(cdot1.y, mass.ey)), v3scale(cdot2, mass.ez));
        const V3 impulse = v3(-mc.x, -mc.y, -mc.z);
        imp.x += impulse.x;
        imp.y += impulse.y;
        imp.z += impulse.z;
        const V2 P = mk(impulse.x, impulse.y);
        vA = sub(vA, scale(mA, P));
        wA -= iA * (cross(rA, P) + impulse.z);
        vB = add(vB, scale(mB, P));
        wB += iB * (cross(rB, P) + impulse.z);
    }
    w.j_imp[j] = imp;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_position_constraints, b2_weld_joint.rs:230-287 */
__device__ bool weld_solve_position(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    float position_error, angular_error;
    const M33 K = weld_k(mA, mB, iA, iB, rA, rB);
    if (lim.y > 0.0f) {
        const V2 C1 = sub(sub(add(cB, rB), cA), rA);
        position_error = length(C1);
        angular_error = 0.0f;
        const V2 P = neg(mat22_solve(K.ex.x, K.ex.y, K.ey.x, K.ey.y, C1));
        cA = sub(cA, scale(mA, P));
        aA -= iA * cross(rA, P);
        cB = add(cB, scale(mB, P));
        aB += iB * cross(rB, P);
    } else {
        const V2 C1 = sub(sub(add(cB, rB), cA), rA);
        const float C2 = aB - aA - lim.x;
        position_error = length(C1);
        angular_error = fabsr(C2);
        V3 impulse;
        if (K.ez.z > 0.0f) {
            const V3 x = m33_solve33(K, v3(C1.x, C1.y, C2));
            impulse = v3(-x.x, -x.y, -x.z);
        } else {
            const V2 i2 = neg(mat22_solve(K.ex.x, K.ex.y, K.ey.x, K.ey.y, C1));
            impulse = v3(i2.x, i2.y, 0.0f);
        }
        const V2 P = mk(impulse.x, impulse.y);
        cA = sub(cA, scale(mA, P));
        aA -= iA * (cross(rA, P) + impulse.z);
        cB = add(cB, scale(mB, P));
        aB += iB * (cross(rB, P) + impulse.z);
    }
    if (joint_body_dynamic(w, bd.x)) w.b_pos[bd.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, bd.y)) w.b_pos[bd.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return position_error <= kLinearSlop && angular_error <= kAngularSlop;
}

/* ---- friction joint (B2frictionJoint, private/dynamics/joints/b2_friction_joint.rs) ----
 * j_lim = (max force, max torque, -, -), j_imp = (linear x, y, angular, -); the step's linear mass
 * (B2Mat22::get_inverse of K) in j_k (ex.x, ex.y, ey.x, ey.y), angular mass in j_s.x. No position
 * correction. */

__device__ void friction_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float aA = w.b_pos[bd.x].z, aB = w.b_pos[bd.y].z;
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    const float kxx = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
    const float kxy = -iA * rA.x * rA.y - iB * rB.x * rB.y;
    const float kyy = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
    /* B2Mat22::get_inverse, src/b2_math.rs:261-276 (a = ex.x, b = ey.x, c = ex.y, d = ey.y) */
    float det = kxx * kyy - kxy * kxy;
    if (det != 0.0f) det = fdiv(1.0f, det);
    const float4 lm = make_float4(det * kyy, -det * kxy, -det * kxy, det * kxx);  /* ex.x, ex.y, ey.x, ey.y */
    float angular_mass = iA + iB;
    if (angular_mass > 0.0f) angular_mass = fdiv(1.0f, angular_mass);
    float4 imp = w.j_imp[j];
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        const V2 P = mk(imp.x, imp.y);
        vA = sub(vA, scale(mA, P));
        wA -= iA * (cross(rA, P) + imp.z);
        vB = add(vB, scale(mB, P));
        wB += iB * (cross(rB, P) + imp.z);
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    w.j_imp[j] = imp;
    w.j_rr[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    w.j_k[j] = lm;
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(angular_mass, 0.0f);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ void friction_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 lim = w.j_lim[j];
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 rA = mk(rr.x, rr.y), rB = mk(rr.z, rr.w);
    const float4 lm = w.j_k[j];
    const float angular_mass = w.j_s[j].x;
    float4 imp = w.j_imp[j];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const float h = sp.dt;
    {
        const float cdot = wB - wA;
        float impulse = -angular_mass * cdot;
        const float old_impulse = imp.z;
        const float max_impulse = h * lim.y;
        imp.z = fclampr(imp.z + impulse, -max_impulse, max_impulse);
        impulse = imp.z - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        const V2 cdot = sub(sub(add(vB, cross_sv(wB, rB)), vA), cross_sv(wA, rA));
        V2 impulse = neg(mk(lm.x * cdot.x + lm.z * cdot.y, lm.y * cdot.x + lm.w * cdot.y));
        const V2 old_impulse = mk(imp.x, imp.y);
        V2 li = add(old_impulse, impulse);
        const float max_impulse = h * lim.x;
        if (dot(li, li) > max_impulse * max_impulse) {
            normalize(li);
            li.x *= max_impulse;
            li.y *= max_impulse;
        }
        impulse = sub(li, old_impulse);
        imp.x = li.x;
        imp.y = li.y;
        vA = sub(vA, scale(mA, impulse));
        wA -= iA * cross(rA, impulse);
        vB = add(vB, scale(mB, impulse));
        wB += iB * cross(rB, impulse);
    }
    w.j_imp[j] = imp;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* ---- motor joint (B2motorJoint, private/dynamics/joints/b2_motor_joint.rs) ----
 * j_anchor = (linear offset x, y, -, -), j_lim = (max force, max torque, correction factor, angular
 * offset), j_imp = (linear x, y, angular, -); the step's linear mass (B2Mat22::get_inverse of K) in
 * j_k, (angular mass, angular error) in j_s, linear error in j_x.xy. No position correction. */

__device__ void motor_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    const float aA = pa.z, aB = pb.z;
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, mk(-lcB.x, -lcB.y));
    const float kxx = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
    const float kxy = -iA * rA.x * rA.y - iB * rB.x * rB.y;
    const float kyy = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
    float det = kxx * kyy - kxy * kxy;
    if (det != 0.0f) det = fdiv(1.0f, det);
    const float4 lm = make_float4(det * kyy, -det * kxy, -det * kxy, det * kxx);  /* ex.x, ex.y, ey.x, ey.y */
    float angular_mass = iA + iB;
    if (angular_mass > 0.0f) angular_mass = fdiv(1.0f, angular_mass);
    const V2 linear_error = sub(sub(add(mk(pb.x, pb.y), rB), mk(pa.x, pa.y)), rA);
    const float angular_error = aB - aA - lim.w;
    float4 imp = w.j_imp[j];
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        const V2 P = mk(imp.x, imp.y);
        vA = sub(vA, scale(mA, P));
        wA -= iA * (cross(rA, P) + imp.z);
        vB = add(vB, scale(mB, P));
        wB += iB * (cross(rB, P) + imp.z);
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    w.j_imp[j] = imp;
    w.j_rr[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    w.j_k[j] = lm;
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(angular_mass, angular_error);
    w.j_x[j] = make_float4(linear_error.x, linear_error.y, 0.0f, 0.0f);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ void motor_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 lim = w.j_lim[j];
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 rA = mk(rr.x, rr.y), rB = mk(rr.z, rr.w);
    const float4 lm = w.j_k[j];
    const float2 as = w.j_s[j];
    const float4 le = w.j_x[j];
    const float cf = lim.z;
    float4 imp = w.j_imp[j];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const float h = sp.dt, inv_h = sp.inv_dt;
    {
        const float cdot = wB - wA + inv_h * cf * as.y;
        float impulse = -as.x * cdot;
        const float old_impulse = imp.z;
        const float max_impulse = h * lim.y;
        imp.z = fclampr(imp.z + impulse, -max_impulse, max_impulse);
        impulse = imp.z - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    {
        const float s = inv_h * cf;
        const V2 cdot = add(sub(sub(add(vB, cross_sv(wB, rB)), vA), cross_sv(wA, rA)), mk(s * le.x, s * le.y));
        V2 impulse = neg(mk(lm.x * cdot.x + lm.z * cdot.y, lm.y * cdot.x + lm.w * cdot.y));
        const V2 old_impulse = mk(imp.x, imp.y);
        V2 li = add(old_impulse, impulse);
        const float max_impulse = h * lim.x;
        if (dot(li, li) > max_impulse * max_impulse) {
            normalize(li);
            li.x *= max_impulse;
            li.y *= max_impulse;
        }
        impulse = sub(li, old_impulse);
        imp.x = li.x;
        imp.y = li.y;
        vA = sub(vA, scale(mA, impulse));
        wA -= iA * cross(rA, impulse);
        vB = add(vB, scale(mB, impulse));
        wB += iB * cross(rB, impulse);
    }
    w.j_imp[j] = imp;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* ---- mouse joint (B2mouseJoint, private/dynamics/joints/b2_mouse_joint.rs) ----
 * j_anchor = (target x, y, local anchor B x, y), j_lim = (max force, stiffness, damping, -),
 * j_imp = (x, y, -, -); the step's mass (B2Mat22::get_inverse of K + gamma I) in j_k, r_b in j_rr.zw,
 * gamma in j_s.x, beta-scaled position error in j_x.xy. Acts on body B only; no position correction. */

__device__ void mouse_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int b = w.j_body[j].y;
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 massB = w.b_mass[b];
    const float2 lcB = w.b_lc[b];
    const float mB = massB.y, iB = massB.w;
    const float4 pb = w.b_pos[b];
    float4 vb = w.b_vel[b];
    V2 vB = mk(vb.x, vb.y);
    float wB = vb.z;
    const Rot qB = rot(pb.z);
    const float d = lim.z, k = lim.y, h = sp.dt;
    float gamma = h * (d + h * k);
    if (gamma != 0.0f) gamma = fdiv(1.0f, gamma);
    const float beta = h * k * gamma;
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    const float kxx = mB + iB * rB.y * rB.y + gamma;
    const float kxy = -iB * rB.x * rB.y;
    const float kyy = mB + iB * rB.x * rB.x + gamma;
    float det = kxx * kyy - kxy * kxy;
    if (det != 0.0f) det = fdiv(1.0f, det);
    const float4 lm = make_float4(det * kyy, -det * kxy, -det * kxy, det * kxx);  /* ex.x, ex.y, ey.x, ey.y */
    V2 C = sub(add(mk(pb.x, pb.y), rB), mk(an.x, an.y));
    C = mk(C.x * beta, C.y * beta);
    wB *= 0.98f;
    float4 imp = w.j_imp[j];
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        const V2 P = mk(imp.x, imp.y);
        vB = add(vB, scale(mB, P));
        wB += iB * cross(rB, P);
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    w.j_imp[j] = imp;
    w.j_rr[j] = make_float4(0.0f, 0.0f, rB.x, rB.y);
    w.j_k[j] = lm;
    w.j_m[j] = make_float4(0.0f, mB, 0.0f, iB);
    w.j_s[j] = make_float2(gamma, 0.0f);
    w.j_x[j] = make_float4(C.x, C.y, 0.0f, 0.0f);
    if (joint_body_dynamic(w, b)) w.b_vel[b] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ void mouse_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int b = w.j_body[j].y;
    const float4 lim = w.j_lim[j];
    const float4 m = w.j_m[j];
    const float mB = m.y, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 rB = mk(rr.z, rr.w);
    const float4 lm = w.j_k[j];
    const float gamma = w.j_s[j].x;
    const float4 C = w.j_x[j];
    float4 imp = w.j_imp[j];
    float4 vb = w.b_vel[b];
    V2 vB = mk(vb.x, vb.y);
    float wB = vb.z;
    const V2 cdot = add(vB, cross_sv(wB, rB));
    const V2 rhs = neg(add(add(cdot, mk(C.x, C.y)), mk(gamma * imp.x, gamma * imp.y)));
    V2 impulse = mk(lm.x * rhs.x + lm.z * rhs.y, lm.y * rhs.x + lm.w * rhs.y);
    const V2 old_impulse = mk(imp.x, imp.y);
    V2 li = add(old_impulse, impulse);
    const float max_impulse = sp.dt * lim.x;
    if (dot(li, li) > max_impulse * max_impulse) {
        const float s = fdiv(max_impulse, length(li));
        li.x *= s;
        li.y *= s;
    }
    impulse = sub(li, old_impulse);
    imp.x = li.x;
    imp.y = li.y;
    vB = add(vB, scale(mB, impulse));
    wB += iB * cross(rB, impulse);
    w.j_imp[j] = imp;
    if (joint_body_dynamic(w, b)) w.b_vel[b] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* ---- prismatic joint (B2prismaticJoint, private/dynamics/joints/b2_prismatic_joint.rs:120-460) ----
 * j_lim = (lower, upper translation, motor speed, max motor force), j_par = (reference angle, flags,
 * unit local axis x, y), j_imp = (x, y, motor, lower), j_imp2.x = upper; the step's axis and perp in
 * j_rr, (a1, a2, s1, s2) in j_k, (k11, k12, k22, axial mass) in j_x, translation in j_s.x. */

__device__ void prismatic_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 par = w.j_par[j];
    const uint32_t jf = __float_as_uint(par.y);
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(pa.z), qB = rot(pb.z);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    const V2 d = sub(add(sub(mk(pb.x, pb.y), mk(pa.x, pa.y)), rB), rA);
    const V2 xaxis = mk(par.z, par.w);
    const V2 axis = mul(qA, xaxis);
    const float a1 = cross(add(d, rA), axis), a2 = cross(rB, axis);
    float axial_mass = mA + mB + iA * a1 * a1 + iB * a2 * a2;
    if (axial_mass > 0.0f) axial_mass = fdiv(1.0f, axial_mass);
    const V2 perp = mul(qA, cross_sv(1.0f, xaxis));
    const float s1 = cross(add(d, rA), perp), s2 = cross(rB, perp);
    const float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
    const float k12 = iA * s1 + iB * s2;
    float k22 = iA + iB;
    if (k22 == 0.0f) k22 = 1.0f;
    float4 imp = w.j_imp[j];
    float4 imp2 = w.j_imp2[j];
    float translation = 0.0f;
    if (jf & JF_LIMIT) {
        translation = dot(axis, d);
    } else {
        imp.w = 0.0f;
        imp2.x = 0.0f;
    }
    if (!(jf & JF_MOTOR)) imp.z = 0.0f;
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        imp.w *= sp.dt_ratio;
        imp2.x *= sp.dt_ratio;
        const float axial = imp.z + imp.w - imp2.x;
        const V2 P = add(scale(imp.x, perp), scale(axial, axis));
        const float LA = imp.x * s1 + imp.y + axial * a1;
        const float LB = imp.x * s2 + imp.y + axial * a2;
        vA = sub(vA, scale(mA, P));
        wA -= iA * LA;
        vB = add(vB, scale(mB, P));
        wB += iB * LB;
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        imp2.x = 0.0f;
    }
    w.j_imp[j] = imp;
    w.j_imp2[j] = imp2;
    w.j_rr[j] = make_float4(axis.x, axis.y, perp.x, perp.y);
    w.j_k[j] = make_float4(a1, a2, s1, s2);
    w.j_x[j] = make_float4(k11, k12, k22, axial_mass);
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(translation, 0.0f);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ void prismatic_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 lim = w.j_lim[j];
    const uint32_t jf = __float_as_uint(w.j_par[j].y);
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 axis = mk(rr.x, rr.y), perp = mk(rr.z, rr.w);
    const float4 ak = w.j_k[j];
    const float a1 = ak.x, a2 = ak.y, s1 = ak.z, s2 = ak.w;
    const float4 kx = w.j_x[j];
    const float axial_mass = kx.w, translation = w.j_s[j].x;
    float4 imp = w.j_imp[j];
    float4 imp2 = w.j_imp2[j];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    if (jf & JF_MOTOR) {
        const float cdot = dot(axis, sub(vB, vA)) + a2 * wB - a1 * wA;
        float impulse = axial_mass * (lim.z - cdot);
        const float old_impulse = imp.z;
        const float max_impulse = sp.dt * lim.w;
        imp.z = fclampr(imp.z + impulse, -max_impulse, max_impulse);
        impulse = imp.z - old_impulse;
        const V2 P = scale(impulse, axis);
        const float LA = impulse * a1, LB = impulse * a2;
        vA = sub(vA, scale(mA, P));
        wA -= iA * LA;
        vB = add(vB, scale(mB, P));
        wB += iB * LB;
    }
    if (jf & JF_LIMIT) {
        {
            const float C = translation - lim.x;
            const float cdot = dot(axis, sub(vB, vA)) + a2 * wB - a1 * wA;
            float impulse = -axial_mass * (cdot + fmaxr(C, 0.0f) * sp.inv_dt);
            const float old_impulse = imp.w;
            imp.w = fmaxr(imp.w + impulse, 0.0f);
            impulse = imp.w - old_impulse;
            const V2 P = scale(impulse, axis);
            const float LA = impulse * a1, LB = impulse * a2;
            vA = sub(vA, scale(mA, P));
            wA -= iA * LA;
            vB = add(vB, scale(mB, P));
            wB += iB * LB;
        }
        {
            const float C = lim.y - translation;
            const float cdot = dot(axis, sub(vA, vB)) + a1 * wA - a2 * wB;
            float impulse = -axial_mass * (cdot + fmaxr(C, 0.0f) * sp.inv_dt);
            const float old_impulse = imp2.x;
            imp2.x = fmaxr(imp2.x + impulse, 0.0f);
            impulse = imp2.x - old_impulse;
            const V2 P = scale(impulse, axis);
            const float LA = impulse * a1, LB = impulse * a2;
            vA = add(vA, scale(mA, P));
            wA += iA * LA;
            vB = sub(vB, scale(mB, P));
            wB -= iB * LB;
        }
    }
    {
        const V2 cdot = mk(dot(perp, sub(vB, vA)) + s2 * wB - s1 * wA, wB - wA);
        const V2 df = mat22_solve(kx.x, kx.y, kx.y, kx.z, neg(cdot));
        imp.x += df.x;
        imp.y += df.y;
        const V2 P = scale(df.x, perp);
        const float LA = df.x * s1 + df.y, LB = df.x * s2 + df.y;
        vA = sub(vA, scale(mA, P));
        wA -= iA * LA;
        vB = add(vB, scale(mB, P));
        wB += iB * LB;
    }
    w.j_imp[j] = imp;
    w.j_imp2[j] = imp2;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ bool prismatic_solve_position(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 par = w.j_par[j];
    const uint32_t jf = __float_as_uint(par.y);
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    const V2 d = sub(sub(add(cB, rB), cA), rA);
    const V2 xaxis = mk(par.z, par.w);
    const V2 axis = mul(qA, xaxis);
    const float a1 = cross(add(d, rA), axis), a2 = cross(rB, axis);
    const V2 perp = mul(qA, cross_sv(1.0f, xaxis));
    const float s1 = cross(add(d, rA), perp), s2 = cross(rB, perp);
    const V2 C1 = mk(dot(perp, d), aB - aA - par.x);
    float linear_error = fabsr(C1.x);
    const float angular_error = fabsr(C1.y);
    bool active = false;
    float C2 = 0.0f;
    if (jf & JF_LIMIT) {
        const float translation = dot(axis, d);
        if (fabsr(lim.y - lim.x) < 2.0f * kLinearSlop) {
            C2 = translation;
            linear_error = fmaxr(linear_error, fabsr(translation));
            active = true;
        } else if (translation <= lim.x) {
            C2 = fminr(translation - lim.x, 0.0f);
            linear_error = fmaxr(linear_error, lim.x - translation);
            active = true;
        } else if (translation >= lim.y) {
            C2 = fmaxr(translation - lim.y, 0.0f);
            linear_error = fmaxr(linear_error, translation - lim.y);
            active = true;
        }
    }
    V3 impulse;
    const float k11 = mA + mB + iA * s1 * s1 + iB * s2 * s2;
    const float k12 = iA * s1 + iB * s2;
    if (active) {
        const float k13 = iA * s1 * a1 + iB * s2 * a2;
        float k22 = iA + iB;
        if (k22 == 0.0f) k22 = 1.0f;
        const float k23 = iA * a1 + iB * a2;
        const float k33 = mA + mB + iA * a1 * a1 + iB * a2 * a2;
        M33 K;
        K.ex = v3(k11, k12, k13);
        K.ey = v3(k12, k22, k23);
        K.ez = v3(k13, k23, k33);
        impulse = m33_solve33(K, v3(-C1.x, -C1.y, -C2));
    } else {
        float k22 = iA + iB;
        if (k22 == 0.0f) k22 = 1.0f;
        const V2 i1 = mat22_solve(k11, k12, k12, k22, neg(C1));
        impulse = v3(i1.x, i1.y, 0.0f);
    }
    const V2 P = add(scale(impulse.x, perp), scale(impulse.z, axis));
    const float LA = impulse.x * s1 + impulse.y + impulse.z * a1;
    const float LB = impulse.x * s2 + impulse.y + impulse.z * a2;
    cA = sub(cA, scale(mA, P));
    aA -= iA * LA;
    cB = add(cB, scale(mB, P));
    aB += iB * LB;
    if (joint_body_dynamic(w, bd.x)) w.b_pos[bd.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, bd.y)) w.b_pos[bd.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return linear_error <= kLinearSlop && angular_error <= kAngularSlop;
}

/* ---- wheel joint (B2wheelJoint, private/dynamics/joints/b2_wheel_joint.rs:24-398) ----
 * j_lim = (lower, upper translation, motor speed, max motor torque), j_par = (stiffness, flags, local
 * axis x, y), j_imp = (impulse, spring, motor, lower), j_imp2 = (upper, translation, -, damping); the
 * step's ax and ay in j_rr, (s_ax, s_bx, s_ay, s_by) in j_k, (mass, axial mass, spring mass, motor
 * mass) in j_x, (bias, gamma) in j_s. As the reference does: the warm start does not scale the limit
 * impulses, and the position pass reuses the step's ax, s_ay and s_by where it says so. */

__device__ void wheel_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 par = w.j_par[j];
    const uint32_t jf = __float_as_uint(par.y);
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(pa.z), qB = rot(pb.z);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    const V2 d = sub(sub(add(mk(pb.x, pb.y), rB), mk(pa.x, pa.y)), rA);
    const V2 xaxis = mk(par.z, par.w);
    const V2 ay = mul(qA, cross_sv(1.0f, xaxis));
    const float s_ay = cross(add(d, rA), ay), s_by = cross(rB, ay);
    float mass = mA + mB + iA * s_ay * s_ay + iB * s_by * s_by;
    if (mass > 0.0f) mass = fdiv(1.0f, mass);
    const V2 ax = mul(qA, xaxis);
    const float s_ax = cross(add(d, rA), ax), s_bx = cross(rB, ax);
    const float inv_mass = mA + mB + iA * s_ax * s_ax + iB * s_bx * s_bx;
    const float axial_mass = inv_mass > 0.0f ? fdiv(1.0f, inv_mass) : 0.0f;
    float4 imp = w.j_imp[j];
    float4 imp2 = w.j_imp2[j];
    const float stiffness = par.x, damping = imp2.w;
    float spring_mass = 0.0f, bias = 0.0f, gamma = 0.0f;
    if (stiffness > 0.0f && inv_mass > 0.0f) {
        const float C = dot(d, ax);
        const float h = sp.dt;
        gamma = h * (damping + h * stiffness);
        if (gamma > 0.0f) gamma = fdiv(1.0f, gamma);
        bias = C * h * stiffness * gamma;
        spring_mass = inv_mass + gamma;
        if (spring_mass > 0.0f) spring_mass = fdiv(1.0f, spring_mass);
    } else {
        imp.y = 0.0f;
    }
    if (jf & JF_LIMIT) {
        imp2.y = dot(ax, d);
    } else {
        imp.w = 0.0f;
        imp2.x = 0.0f;
    }
    float motor_mass = 0.0f;
    if (jf & JF_MOTOR) {
        motor_mass = iA + iB;
        if (motor_mass > 0.0f) motor_mass = fdiv(1.0f, motor_mass);
    } else {
        imp.z = 0.0f;
    }
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        const float axial = imp.y + imp.w - imp2.x;
        const V2 P = add(scale(imp.x, ay), scale(axial, ax));
        const float LA = imp.x * s_ay + axial * s_ax + imp.z;
        const float LB = imp.x * s_by + axial * s_bx + imp.z;
        vA = sub(vA, scale(mA, P));
        wA -= iA * LA;
        vB = add(vB, scale(mB, P));
        wB += iB * LB;
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        imp2.x = 0.0f;
    }
    w.j_imp[j] = imp;
    w.j_imp2[j] = imp2;
    w.j_rr[j] = make_float4(ax.x, ax.y, ay.x, ay.y);
    w.j_k[j] = make_float4(s_ax, s_bx, s_ay, s_by);
    w.j_x[j] = make_float4(mass, axial_mass, spring_mass, motor_mass);
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(bias, gamma);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ void wheel_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 lim = w.j_lim[j];
    const uint32_t jf = __float_as_uint(w.j_par[j].y);
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 ax = mk(rr.x, rr.y), ay = mk(rr.z, rr.w);
    const float4 sk = w.j_k[j];
    const float s_ax = sk.x, s_bx = sk.y, s_ay = sk.z, s_by = sk.w;
    const float4 ms = w.j_x[j];
    const float2 bg = w.j_s[j];
    float4 imp = w.j_imp[j];
    float4 imp2 = w.j_imp2[j];
    const float translation = imp2.y;
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    {
        const float cdot = dot(ax, sub(vB, vA)) + s_bx * wB - s_ax * wA;
        const float impulse = -ms.z * (cdot + bg.x + bg.y * imp.y);
        imp.y += impulse;
        const V2 P = scale(impulse, ax);
        const float LA = impulse * s_ax, LB = impulse * s_bx;
        vA = sub(vA, scale(mA, P));
        wA -= iA * LA;
        vB = add(vB, scale(mB, P));
        wB += iB * LB;
    }
    {
        const float cdot = wB - wA - lim.z;
        float impulse = -ms.w * cdot;
        const float old_impulse = imp.z;
        const float max_impulse = sp.dt * lim.w;
        imp.z = fclampr(imp.z + impulse, -max_impulse, max_impulse);
        impulse = imp.z - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    if (jf & JF_LIMIT) {
        {
            const float C = translation - lim.x;
            const float cdot = dot(ax, sub(vB, vA)) + s_bx * wB - s_ax * wA;
            float impulse = -ms.y * (cdot + fmaxr(C, 0.0f) * sp.inv_dt);
            const float old_impulse = imp.w;
            imp.w = fmaxr(imp.w + impulse, 0.0f);
            impulse = imp.w - old_impulse;
            const V2 P = scale(impulse, ax);
            const float LA = impulse * s_ax, LB = impulse * s_bx;
            vA = sub(vA, scale(mA, P));
            wA -= iA * LA;
            vB = add(vB, scale(mB, P));
            wB += iB * LB;
        }
        {
            const float C = lim.y - translation;
            const float cdot = dot(ax, sub(vA, vB)) + s_ax * wA - s_bx * wB;
            float impulse = -ms.y * (cdot + fmaxr(C, 0.0f) * sp.inv_dt);
            const float old_impulse = imp2.x;
            imp2.x = fmaxr(imp2.x + impulse, 0.0f);
            impulse = imp2.x - old_impulse;
            const V2 P = scale(impulse, ax);
            const float LA = impulse * s_ax, LB = impulse * s_bx;
            vA = add(vA, scale(mA, P));
            wA += iA * LA;
            vB = sub(vB, scale(mB, P));
            wB -= iB * LB;
        }
    }
    {
        const float cdot = dot(ay, sub(vB, vA)) + s_by * wB - s_ay * wA;
        const float impulse = -ms.x * cdot;
        imp.x += impulse;
        const V2 P = scale(impulse, ay);
        const float LA = impulse * s_ay, LB = impulse * s_by;
        vA = sub(vA, scale(mA, P));
        wA -= iA * LA;
        vB = add(vB, scale(mB, P));
        wB += iB * LB;
    }
    w.j_imp[j] = imp;
    w.j_imp2[j] = imp2;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ bool wheel_solve_position(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const float4 par = w.j_par[j];
    const uint32_t jf = __float_as_uint(par.y);
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 step_ax = mk(rr.x, rr.y);
    const float4 sk = w.j_k[j];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const V2 xaxis = mk(par.z, par.w);
    float linear_error = 0.0f;
    if (jf & JF_LIMIT) {
        const Rot qA = rot(aA), qB = rot(aB);
        const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
        const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
        const V2 d = sub(add(sub(cB, cA), rB), rA);
        const V2 ax = mul(qA, xaxis);
        const float s_ax = cross(add(d, rA), step_ax), s_bx = cross(rB, step_ax);
        float C = 0.0f;
        const float translation = dot(ax, d);
        if (fabsr(lim.y - lim.x) < 2.0f * kLinearSlop) C = translation;
        else if (translation <= lim.x) C = fminr(translation - lim.x, 0.0f);
        else if (translation >= lim.y) C = fmaxr(translation - lim.y, 0.0f);
        if (C != 0.0f) {
            const float inv_mass = mA + mB + iA * s_ax * s_ax + iB * s_bx * s_bx;
            float impulse = 0.0f;
            if (inv_mass != 0.0f) impulse = fdiv(-C, inv_mass);
            const V2 P = scale(impulse, ax);
            const float LA = impulse * s_ax, LB = impulse * s_bx;
            cA = sub(cA, scale(mA, P));
            aA -= iA * LA;
            cB = add(cB, scale(mB, P));
            aB += iB * LB;
            linear_error = fabsr(C);
        }
    }
    {
        const Rot qA = rot(aA), qB = rot(aB);
        const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
        const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
        const V2 d = sub(add(sub(cB, cA), rB), rA);
        const V2 ay = mul(qA, cross_sv(1.0f, xaxis));
        const float s_ay = cross(add(d, rA), ay), s_by = cross(rB, ay);
        const float C = dot(d, ay);
        const float inv_mass = mA + mB + iA * sk.z * sk.z + iB * sk.w * sk.w;
        float impulse = 0.0f;
        if (inv_mass != 0.0f) impulse = fdiv(-C, inv_mass);
        const V2 P = scale(impulse, ay);
        const float LA = impulse * s_ay, LB = impulse * s_by;
        cA = sub(cA, scale(mA, P));
        aA -= iA * LA;
        cB = add(cB, scale(mB, P));
        aB += iB * LB;
        linear_error = fmaxr(linear_error, fabsr(C));
    }
    if (joint_body_dynamic(w, bd.x)) w.b_pos[bd.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, bd.y)) w.b_pos[bd.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return linear_error <= kLinearSlop;
}

/* ---- pulley joint (B2pulleyJoint, private/dynamics/joints/b2_pulley_joint.rs) ----
 * j_lim = (ground anchor A x, y, ground anchor B x, y), j_par = (ratio, flags, length A, length B), j_imp.x =
 * impulse; the step's r_a, r_b in j_rr, u_a, u_b in j_k, mass in j_s.x. */

struct PulleyFrame {
    V2 rA, rB, uA, uB;
    float lenA, lenB, mass;
};

__device__ __forceinline__ PulleyFrame pulley_frame(const DevWorld& w, int j, V2 cA, float aA, V2 cB, float aB,
                                                    float mA, float mB, float iA, float iB) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 g = w.j_lim[j];
    const float ratio = w.j_par[j].x;
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    PulleyFrame f;
    f.rA = mul(rot(aA), sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    f.rB = mul(rot(aB), sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    f.uA = sub(add(cA, f.rA), mk(g.x, g.y));
    f.uB = sub(add(cB, f.rB), mk(g.z, g.w));
    f.lenA = length(f.uA);
    f.lenB = length(f.uB);
    if (f.lenA > 10.0f * kLinearSlop) {
        const float s = fdiv(1.0f, f.lenA);
        f.uA = mk(f.uA.x * s, f.uA.y * s);
    } else {
        f.uA = mk(0.0f, 0.0f);
    }
    if (f.lenB > 10.0f * kLinearSlop) {
        const float s = fdiv(1.0f, f.lenB);
        f.uB = mk(f.uB.x * s, f.uB.y * s);
    } else {
        f.uB = mk(0.0f, 0.0f);
    }
    const float ruA = cross(f.rA, f.uA), ruB = cross(f.rB, f.uB);
    const float mAe = mA + iA * ruA * ruA, mBe = mB + iB * ruB * ruB;
    f.mass = mAe + ratio * ratio * mBe;
    if (f.mass > 0.0f) f.mass = fdiv(1.0f, f.mass);
    return f;
}

__device__ void pulley_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float ratio = w.j_par[j].x;
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    const PulleyFrame f = pulley_frame(w, j, mk(pa.x, pa.y), pa.z, mk(pb.x, pb.y), pb.z, mA, mB, iA, iB);
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    float4 imp = w.j_imp[j];
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        const V2 PA = scale(-imp.x, f.uA);
        const V2 PB = scale(-ratio * imp.x, f.uB);
        vA = add(vA, scale(mA, PA));
        wA += iA * cross(f.rA, PA);
        vB = add(vB, scale(mB, PB));
        wB += iB * cross(f.rB, PB);
    } else {
        imp.x = 0.0f;
    }
    w.j_imp[j] = imp;
    w.j_rr[j] = make_float4(f.rA.x, f.rA.y, f.rB.x, f.rB.y);
    w.j_k[j] = make_float4(f.uA.x, f.uA.y, f.uB.x, f.uB.y);
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(f.mass, 0.0f);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ void pulley_solve_velocity(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float ratio = w.j_par[j].x;
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j], uu = w.j_k[j];
    const V2 rA = mk(rr.x, rr.y), rB = mk(rr.z, rr.w), uA = mk(uu.x, uu.y), uB = mk(uu.z, uu.w);
    const float mass = w.j_s[j].x;
    float4 imp = w.j_imp[j];
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const V2 vpA = add(vA, cross_sv(wA, rA)), vpB = add(vB, cross_sv(wB, rB));
    const float cdot = -dot(uA, vpA) - ratio * dot(uB, vpB);
    const float impulse = -mass * cdot;
    imp.x += impulse;
    const V2 PA = scale(-impulse, uA);
    const V2 PB = scale(-ratio * impulse, uB);
    vA = add(vA, scale(mA, PA));
    wA += iA * cross(rA, PA);
    vB = add(vB, scale(mB, PB));
    wB += iB * cross(rB, PB);
    w.j_imp[j] = imp;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

__device__ bool pulley_solve_position(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float4 par = w.j_par[j];
    const float ratio = par.x;
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    const PulleyFrame f = pulley_frame(w, j, cA, aA, cB, aB, mA, mB, iA, iB);
    const float constant = par.z + ratio * par.w;
    const float C = constant - f.lenA - ratio * f.lenB;
    const float linear_error = fabsr(C);
    const float impulse = -f.mass * C;
    const V2 PA = scale(-impulse, f.uA);
    const V2 PB = scale(-ratio * impulse, f.uB);
    cA = add(cA, scale(mA, PA));
    aA += iA * cross(f.rA, PA);
    cB = add(cB, scale(mB, PB));
    aB += iB * cross(f.rB, PB);
    if (joint_body_dynamic(w, bd.x)) w.b_pos[bd.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, bd.y)) w.b_pos[bd.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return linear_error < kLinearSlop;
}

/* ---- gear joint (B2gearJoint, private/dynamics/joints/b2_gear_joint.rs) ----
 * Couples two revolute or prismatic joints: A and B are the second bodies of joint 1 and joint 2, C and
 * D their first bodies (grounds, usually). j_body = (A, B), j_body2 = (C, D), j_anchor = (local anchor
 * A, local anchor B), j_lim = (local anchor C, local anchor D), j_x = (local axis C, local axis D; zero
 * for a revolute side), j_s = (reference angle A, reference angle B), j_par = (ratio, flags, constant,
 * -) with JF_GEAR_A_PRISMATIC / JF_GEAR_B_PRISMATIC; j_imp.x = impulse. The step's temporaries: j_rr =
 * (jv_ac, jv_bd), j_k = (jw_a, jw_b, jw_c, jw_d), j_m.x = effective mass. */

struct GearJacobian {
    V2 jv_ac, jv_bd;
    float jw_a, jw_b, jw_c, jw_d, mass;
};

/* the Jacobian rows and the (not yet inverted) mass sum of :209-241 and :326-359, from the bodies'
 * rotations; mA..mD are the bodies' (m, 1/m, I, 1/I) */
__device__ __forceinline__ GearJacobian gear_jacobian(const DevWorld& w, int j, const Rot& qA, const Rot& qB,
                                                      const Rot& qC, const Rot& qD, const float4& mA,
                                                      const float4& mB, const float4& mC, const float4& mD) {
    const int2 ab = w.j_body[j], cd = w.j_body2[j];
    const float4 an = w.j_anchor[j], an2 = w.j_lim[j], ax = w.j_x[j], par = w.j_par[j];
    const uint32_t fl = __float_as_uint(par.y);
    const float ratio = par.x;
    GearJacobian g;
    g.mass = 0.0f;
    if (!(fl & JF_GEAR_A_PRISMATIC)) {
        g.jv_ac = mk(0.0f, 0.0f);
        g.jw_a = 1.0f;
        g.jw_c = 1.0f;
        g.mass += mA.w + mC.w;
    } else {
        const float2 lcA = w.b_lc[ab.x], lcC = w.b_lc[cd.x];
        const V2 u = mul(qC, mk(ax.x, ax.y));
        const V2 rC = mul(qC, sub(mk(an2.x, an2.y), mk(lcC.x, lcC.y)));
        const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
        g.jv_ac = u;
        g.jw_c = cross(rC, u);
        g.jw_a = cross(rA, u);
        g.mass += mC.y + mA.y + mC.w * g.jw_c * g.jw_c + mA.w * g.jw_a * g.jw_a;
    }
    if (!(fl & JF_GEAR_B_PRISMATIC)) {
        g.jv_bd = mk(0.0f, 0.0f);
        g.jw_b = ratio;
        g.jw_d = ratio;
        g.mass += ratio * ratio * (mB.w + mD.w);
    } else {
        const float2 lcB = w.b_lc[ab.y], lcD = w.b_lc[cd.y];
        const V2 u = mul(qD, mk(ax.z, ax.w));
        const V2 rD = mul(qD, sub(mk(an2.z, an2.w), mk(lcD.x, lcD.y)));
        const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
        g.jv_bd = scale(ratio, u);
        g.jw_d = ratio * cross(rD, u);
        g.jw_b = ratio * cross(rB, u);
        g.mass += ratio * ratio * (mD.y + mB.y) + mD.w * g.jw_d * g.jw_d + mB.w * g.jw_b * g.jw_b;
    }
    return g;
}

/* the four bodies' velocities changed by the gear impulse (:264-273, :300-307): all four are read, then
 * written back in the order A, B, C, D, so a body that is both A and D keeps D's result, as in the
 * reference */
__device__ __forceinline__ void gear_apply(const DevWorld& w, int j, const GearJacobian& g, float impulse,
                                           const float4& mA, const float4& mB, const float4& mC, const float4& mD) {
    const int2 ab = w.j_body[j], cd = w.j_body2[j];
    const float4 va = w.b_vel[ab.x], vb = w.b_vel[ab.y], vc = w.b_vel[cd.x], vd = w.b_vel[cd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y), vC = mk(vc.x, vc.y), vD = mk(vd.x, vd.y);
    float wA = va.z, wB = vb.z, wC = vc.z, wD = vd.z;
    vA = add(vA, scale(mA.y * impulse, g.jv_ac));
    wA += mA.w * impulse * g.jw_a;
    vB = add(vB, scale(mB.y * impulse, g.jv_bd));
    wB += mB.w * impulse * g.jw_b;
    vC = sub(vC, scale(mC.y * impulse, g.jv_ac));
    wC -= mC.w * impulse * g.jw_c;
    vD = sub(vD, scale(mD.y * impulse, g.jv_bd));
    wD -= mD.w * impulse * g.jw_d;
    if (joint_body_dynamic(w, ab.x)) w.b_vel[ab.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, ab.y)) w.b_vel[ab.y] = make_float4(vB.x, vB.y, wB, vb.w);
    if (joint_body_dynamic(w, cd.x)) w.b_vel[cd.x] = make_float4(vC.x, vC.y, wC, vc.w);
    if (joint_body_dynamic(w, cd.y)) w.b_vel[cd.y] = make_float4(vD.x, vD.y, wD, vd.w);
}

/* init_velocity_constraints, :190-289 */
__device__ void gear_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 ab = w.j_body[j], cd = w.j_body2[j];
    const float4 mA = w.b_mass[ab.x], mB = w.b_mass[ab.y], mC = w.b_mass[cd.x], mD = w.b_mass[cd.y];
    const Rot qA = rot(w.b_pos[ab.x].z), qB = rot(w.b_pos[ab.y].z), qC = rot(w.b_pos[cd.x].z),
              qD = rot(w.b_pos[cd.y].z);
    GearJacobian g = gear_jacobian(w, j, qA, qB, qC, qD, mA, mB, mC, mD);
    g.mass = g.mass > 0.0f ? fdiv(1.0f, g.mass) : 0.0f;
    w.j_rr[j] = make_float4(g.jv_ac.x, g.jv_ac.y, g.jv_bd.x, g.jv_bd.y);
    w.j_k[j] = make_float4(g.jw_a, g.jw_b, g.jw_c, g.jw_d);
    w.j_m[j] = make_float4(g.mass, 0.0f, 0.0f, 0.0f);
    float4 imp = w.j_imp[j];
    if (sp.warm) {
        gear_apply(w, j, g, imp.x, mA, mB, mC, mD);  /* the stored impulse, not scaled by dt_ratio (:264) */
    } else {
        imp.x = 0.0f;
        w.j_imp[j] = imp;
    }
}

/* solve_velocity_constraints, :291-319 */
__device__ void gear_solve_velocity(const DevWorld& w, int j) {
    const int2 ab = w.j_body[j], cd = w.j_body2[j];
    const float4 mA = w.b_mass[ab.x], mB = w.b_mass[ab.y], mC = w.b_mass[cd.x], mD = w.b_mass[cd.y];
    const float4 rr = w.j_rr[j], kk = w.j_k[j];
    GearJacobian g;
    g.jv_ac = mk(rr.x, rr.y);
    g.jv_bd = mk(rr.z, rr.w);
    g.jw_a = kk.x;
    g.jw_b = kk.y;
    g.jw_c = kk.z;
    g.jw_d = kk.w;
    g.mass = w.j_m[j].x;
    const float4 va = w.b_vel[ab.x], vb = w.b_vel[ab.y], vc = w.b_vel[cd.x], vd = w.b_vel[cd.y];
    float cdot = dot(g.jv_ac, sub(mk(va.x, va.y), mk(vc.x, vc.y))) + dot(g.jv_bd, sub(mk(vb.x, vb.y), mk(vd.x, vd.y)));
    cdot += (g.jw_a * va.z - g.jw_c * vc.z) + (g.jw_b * vb.z - g.jw_d * vd.z);
    const float impulse = -g.mass * cdot;
    float4 imp = w.j_imp[j];
    imp.x += impulse;
    w.j_imp[j] = imp;
    gear_apply(w, j, g, impulse, mA, mB, mC, mD);
}

/* solve_position_constraints, :321-393 (the linear error is never measured: the joint always reports
 * itself solved) */
__device__ bool gear_solve_position(const DevWorld& w, int j) {
    const int2 ab = w.j_body[j], cd = w.j_body2[j];
    const float4 mA = w.b_mass[ab.x], mB = w.b_mass[ab.y], mC = w.b_mass[cd.x], mD = w.b_mass[cd.y];
    const float4 pa = w.b_pos[ab.x], pb = w.b_pos[ab.y], pc = w.b_pos[cd.x], pd = w.b_pos[cd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y), cC = mk(pc.x, pc.y), cD = mk(pd.x, pd.y);
    float aA = pa.z, aB = pb.z, aC = pc.z, aD = pd.z;
    const Rot qA = rot(aA), qB = rot(aB), qC = rot(aC), qD = rot(aD);
    const GearJacobian g = gear_jacobian(w, j, qA, qB, qC, qD, mA, mB, mC, mD);
    const float4 an = w.j_anchor[j], an2 = w.j_lim[j], ax = w.j_x[j], par = w.j_par[j];
    const float2 ref = w.j_s[j];
    const uint32_t fl = __float_as_uint(par.y);
    float coordinate_a, coordinate_b;
    if (!(fl & JF_GEAR_A_PRISMATIC)) {
        coordinate_a = aA - aC - ref.x;
    } else {
        const float2 lcA = w.b_lc[ab.x], lcC = w.b_lc[cd.x];
        const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
        const V2 p_c = sub(mk(an2.x, an2.y), mk(lcC.x, lcC.y));
        const V2 p_a = mul_t(qC, add(rA, sub(cA, cC)));
        coordinate_a = dot(sub(p_a, p_c), mk(ax.x, ax.y));
    }
    if (!(fl & JF_GEAR_B_PRISMATIC)) {
        coordinate_b = aB - aD - ref.y;
    } else {
        const float2 lcB = w.b_lc[ab.y], lcD = w.b_lc[cd.y];
        const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
        const V2 p_d = sub(mk(an2.z, an2.w), mk(lcD.x, lcD.y));
        const V2 p_b = mul_t(qD, add(rB, sub(cB, cD)));
        coordinate_b = dot(sub(p_b, p_d), mk(ax.z, ax.w));
    }
    const float C = (coordinate_a + par.x * coordinate_b) - par.z;
    float impulse = 0.0f;
    if (g.mass > 0.0f) impulse = fdiv(-C, g.mass);
    cA = add(cA, scale(mA.y * impulse, g.jv_ac));
    aA += mA.w * impulse * g.jw_a;
    cB = add(cB, scale(mB.y * impulse, g.jv_bd));
    aB += mB.w * impulse * g.jw_b;
    cC = sub(cC, scale(mC.y * impulse, g.jv_ac));
    aC -= mC.w * impulse * g.jw_c;
    cD = sub(cD, scale(mD.y * impulse, g.jv_bd));
    aD -= mD.w * impulse * g.jw_d;
    if (joint_body_dynamic(w, ab.x)) w.b_pos[ab.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, ab.y)) w.b_pos[ab.y] = make_float4(cB.x, cB.y, aB, pb.w);
    if (joint_body_dynamic(w, cd.x)) w.b_pos[cd.x] = make_float4(cC.x, cC.y, aC, pc.w);
    if (joint_body_dynamic(w, cd.y)) w.b_pos[cd.y] = make_float4(cD.x, cD.y, aD, pd.w);
    return true;
}

__device__ __forceinline__ uint32_t joint_type(const DevWorld& w, int j) {
    return (__float_as_uint(w.j_par[j].y) >> JF_TYPE_SHIFT) & 0xffu;
}

__device__ __forceinline__ bool joint_is_distance(const DevWorld& w, int j) {
    return ((__float_as_uint(w.j_par[j].y) >> JF_TYPE_SHIFT) & 0xffu) == B2G_JOINT_DISTANCE;
}

/* init_velocity_constraints, b2_revolute_joint.rs:21-116 */
__device__ void revolute_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const uint32_t jf = __float_as_uint(w.j_par[j].y);
    const float4 massA = w.b_mass[bd.x], massB = w.b_mass[bd.y];
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    const float mA = massA.y, mB = massB.y, iA = massA.w, iB = massB.w;
    const float aA = w.b_pos[bd.x].z, aB = w.b_pos[bd.y].z;
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const Rot qA = rot(aA), qB = rot(aB);
    const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
    const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
    float4 K;
    K.x = mA + mB + rA.y * rA.y * iA + rB.y * rB.y * iB;     /* ex.x */
    K.z = -rA.y * rA.x * iA - rB.y * rB.x * iB;              /* ey.x */
    K.y = K.z;                                               /* ex.y */
    K.w = mA + mB + rA.x * rA.x * iA + rB.x * rB.x * iB;     /* ey.y */
    float axial = iA + iB;
    bool fixed_rotation;
    if (axial > 0.0f) {
        axial = fdiv(1.0f, axial);
        fixed_rotation = false;
    } else {
        fixed_rotation = true;
    }
    const float angle = aB - aA - lim.x;
    float4 imp = w.j_imp[j];
    float upper = w.j_imp2[j].x;
    if (!(jf & JF_LIMIT) || fixed_rotation) {
        imp.w = 0.0f;
        upper = 0.0f;
    }
    if (!(jf & JF_MOTOR) || fixed_rotation) imp.z = 0.0f;
    if (sp.warm) {
        imp.x *= sp.dt_ratio;
        imp.y *= sp.dt_ratio;
        imp.z *= sp.dt_ratio;
        imp.w *= sp.dt_ratio;
        upper *= sp.dt_ratio;
        const float axial_impulse = imp.z + imp.w - upper;
        const V2 P = mk(imp.x, imp.y);
        vA = sub(vA, scale(mA, P));
        wA -= iA * (cross(rA, P) + axial_impulse);
        vB = add(vB, scale(mB, P));
        wB += iB * (cross(rB, P) + axial_impulse);
    } else {
        imp = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        upper = 0.0f;
    }
    w.j_imp[j] = imp;
    w.j_imp2[j] = make_float4(upper, 0.0f, 0.0f, 0.0f);
    w.j_rr[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    w.j_k[j] = K;
    w.j_m[j] = make_float4(mA, mB, iA, iB);
    w.j_s[j] = make_float2(axial, angle);
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_velocity_constraints, b2_revolute_joint.rs:118-208 */
__device__ void revolute_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const int2 bd = w.j_body[j];
    const float4 lim = w.j_lim[j];
    const float4 par = w.j_par[j];
    const uint32_t jf = __float_as_uint(par.y);
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float4 rr = w.j_rr[j];
    const V2 rA = mk(rr.x, rr.y), rB = mk(rr.z, rr.w);
    const float2 s = w.j_s[j];
    const float axial = s.x, angle = s.y;
    float4 imp = w.j_imp[j];
    float upper = w.j_imp2[j].x;
    float4 va = w.b_vel[bd.x], vb = w.b_vel[bd.y];
    V2 vA = mk(va.x, va.y), vB = mk(vb.x, vb.y);
    float wA = va.z, wB = vb.z;
    const bool fixed_rotation = iA + iB == 0.0f;
    if ((jf & JF_MOTOR) && !fixed_rotation) {
        const float cdot = wB - wA - lim.w;
        float impulse = -axial * cdot;
        const float old_impulse = imp.z;
        const float max_impulse = sp.dt * par.x;
        imp.z = fclampr(imp.z + impulse, -max_impulse, max_impulse);
        impulse = imp.z - old_impulse;
        wA -= iA * impulse;
        wB += iB * impulse;
    }
    if ((jf & JF_LIMIT) && !fixed_rotation) {
        {
            const float C = angle - lim.y;
            const float cdot = wB - wA;
            float impulse = -axial * (cdot + fmaxr(C, 0.0f) * sp.inv_dt);
            const float old_impulse = imp.w;
            imp.w = fmaxr(imp.w + impulse, 0.0f);
            impulse = imp.w - old_impulse;
            wA -= iA * impulse;
            wB += iB * impulse;
        }
        {
            const float C = lim.z - angle;
            const float cdot = wA - wB;
            float impulse = -axial * (cdot + fmaxr(C, 0.0f) * sp.inv_dt);
            const float old_impulse = upper;
            upper = fmaxr(upper + impulse, 0.0f);
            impulse = upper - old_impulse;
            wA += iA * impulse;
            wB -= iB * impulse;
        }
    }
    {
        const V2 cdot = sub(sub(add(vB, cross_sv(wB, rB)), vA), cross_sv(wA, rA));
        const float4 K = w.j_k[j];
        const V2 impulse = mat22_solve(K.x, K.y, K.z, K.w, neg(cdot));
        imp.x += impulse.x;
        imp.y += impulse.y;
        vA = sub(vA, scale(mA, impulse));
        wA -= iA * cross(rA, impulse);
        vB = add(vB, scale(mB, impulse));
        wB += iB * cross(rB, impulse);
    }
    w.j_imp[j] = imp;
    w.j_imp2[j].x = upper;
    if (joint_body_dynamic(w, bd.x)) w.b_vel[bd.x] = make_float4(vA.x, vA.y, wA, va.w);
    if (joint_body_dynamic(w, bd.y)) w.b_vel[bd.y] = make_float4(vB.x, vB.y, wB, vb.w);
}

/* solve_position_constraints, b2_revolute_joint.rs:210-287; returns whether the joint is
 * within the linear and angular slop */
__device__ bool revolute_solve_position(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const float4 an = w.j_anchor[j];
    const float4 lim = w.j_lim[j];
    const uint32_t jf = __float_as_uint(w.j_par[j].y);
    const float4 m = w.j_m[j];
    const float mA = m.x, mB = m.y, iA = m.z, iB = m.w;
    const float axial = w.j_s[j].x;
    const float2 lcA = w.b_lc[bd.x], lcB = w.b_lc[bd.y];
    float4 pa = w.b_pos[bd.x], pb = w.b_pos[bd.y];
    V2 cA = mk(pa.x, pa.y), cB = mk(pb.x, pb.y);
    float aA = pa.z, aB = pb.z;
    float angular_error = 0.0f;
    const bool fixed_rotation = iA + iB == 0.0f;
    if ((jf & JF_LIMIT) && !fixed_rotation) {
        const float angle = aB - aA - lim.x;
        float C = 0.0f;
        if (fabsr(lim.z - lim.y) < 2.0f * kAngularSlop) {
            C = fclampr(angle - lim.y, -kMaxAngularCorrection, kMaxAngularCorrection);
        } else if (angle <= lim.y) {
            C = fclampr(angle - lim.y + kAngularSlop, -kMaxAngularCorrection, 0.0f);
        } else if (angle >= lim.z) {
            C = fclampr(angle - lim.z - kAngularSlop, 0.0f, kMaxAngularCorrection);
        }
        const float limit_impulse = -axial * C;
        aA -= iA * limit_impulse;
        aB += iB * limit_impulse;
        angular_error = fabsr(C);
    }
    float position_error;
    {
        const Rot qA = rot(aA), qB = rot(aB);
        const V2 rA = mul(qA, sub(mk(an.x, an.y), mk(lcA.x, lcA.y)));
        const V2 rB = mul(qB, sub(mk(an.z, an.w), mk(lcB.x, lcB.y)));
        const V2 C = sub(sub(add(cB, rB), cA), rA);
        position_error = length(C);
        const float kxx = mA + mB + iA * rA.y * rA.y + iB * rB.y * rB.y;
        const float kxy = -iA * rA.x * rA.y - iB * rB.x * rB.y;
        const float kyy = mA + mB + iA * rA.x * rA.x + iB * rB.x * rB.x;
        const V2 impulse = neg(mat22_solve(kxx, kxy, kxy, kyy, C));
        cA = sub(cA, scale(mA, impulse));
        aA -= iA * cross(rA, impulse);
        cB = add(cB, scale(mB, impulse));
        aB += iB * cross(rB, impulse);
    }
    if (joint_body_dynamic(w, bd.x)) w.b_pos[bd.x] = make_float4(cA.x, cA.y, aA, pa.w);
    if (joint_body_dynamic(w, bd.y)) w.b_pos[bd.y] = make_float4(cB.x, cB.y, aB, pb.w);
    return position_error <= kLinearSlop && angular_error <= kAngularSlop;
}

/* the joint routines by type */
__device__ __forceinline__ void joint_init_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const uint32_t t = joint_type(w, j);
    if (t == B2G_JOINT_DISTANCE) distance_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_WELD) weld_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_FRICTION) friction_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_MOTOR) motor_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_MOUSE) mouse_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_PRISMATIC) prismatic_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_WHEEL) wheel_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_PULLEY) pulley_init_velocity(w, sp, j);
    else if (t == B2G_JOINT_GEAR) gear_init_velocity(w, sp, j);
    else revolute_init_velocity(w, sp, j);
}
__device__ __forceinline__ void joint_solve_velocity(const DevWorld& w, const StepParams& sp, int j) {
    const uint32_t t = joint_type(w, j);
    if (t == B2G_JOINT_DISTANCE) distance_solve_velocity(w, sp, j);
    else if (t == B2G_JOINT_WELD) weld_solve_velocity(w, j);
    else if (t == B2G_JOINT_FRICTION) friction_solve_velocity(w, sp, j);
    else if (t == B2G_JOINT_MOTOR) motor_solve_velocity(w, sp, j);
    else if (t == B2G_JOINT_MOUSE) mouse_solve_velocity(w, sp, j);
    else if (t == B2G_JOINT_PRISMATIC) prismatic_solve_velocity(w, sp, j);
    else if (t == B2G_JOINT_WHEEL) wheel_solve_velocity(w, sp, j);
    else if (t == B2G_JOINT_PULLEY) pulley_solve_velocity(w, j);
    else if (t == B2G_JOINT_GEAR) gear_solve_velocity(w, j);
    else revolute_solve_velocity(w, sp, j);
}
__device__ __forceinline__ bool joint_solve_position(const DevWorld& w, int j) {
    const uint32_t t = joint_type(w, j);
    if (t == B2G_JOINT_DISTANCE) return distance_solve_position(w, j);
    if (t == B2G_JOINT_WELD) return weld_solve_position(w, j);
    if (t == B2G_JOINT_FRICTION || t == B2G_JOINT_MOTOR || t == B2G_JOINT_MOUSE) return true;
    if (t == B2G_JOINT_PRISMATIC) return prismatic_solve_position(w, j);
    if (t == B2G_JOINT_WHEEL) return wheel_solve_position(w, j);
    if (t == B2G_JOINT_PULLEY) return pulley_solve_position(w, j);
    if (t == B2G_JOINT_GEAR) return gear_solve_position(w, j);
    return revolute_solve_position(w, j);
}

/* the joint belongs to an island solved this step (a body of it is non-static and in one); both
 * bodies enabled (private/dynamics/b2_world.rs:476-479) */
__device__ __forceinline__ int joint_island(const DevWorld& w, int j) {
    const int2 bd = w.j_body[j];
    const uint32_t fa = w.b_flags[bd.x], fb = w.b_flags[bd.y];
    if (!(fa & BF_ENABLED) || !(fb & BF_ENABLED)) return -1;
    if ((fa & BF_TYPE_MASK) != BODY_STATIC && (fa & BF_ISLAND)) return w.b_island[bd.x];
    if ((fb & BF_TYPE_MASK) != BODY_STATIC && (fb & BF_ISLAND)) return w.b_island[bd.y];
    return -1;
}

}  // namespace
}  // namespace b2g
#endif
