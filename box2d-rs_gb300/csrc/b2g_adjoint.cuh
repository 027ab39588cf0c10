/*
 * b2g_adjoint.cuh — the differentiable step: forward replay and hand-written adjoint.
 *
 * The model differentiated is one world step of B2island::solve
 * (src/private/dynamics/b2_island_private.rs:129-328) with B2contactSolver
 * (src/private/dynamics/b2_contact_solver_private.rs:20-730) and its discrete decisions frozen
 * from the forward pass: the contact set with each manifold in local coordinates and its
 * feature matching to the previous step, the Gauss-Seidel order (colours), the block-solver
 * reduction, the restitution trigger, every friction-cone and normal clamp state, the 2-point
 * block-LCP case, the translation/rotation clamps, every position-correction clamp and each
 * island's position-iteration count. Everything else is differentiated exactly: velocity
 * integration, the world manifold from the body poses (rotations included), effective masses,
 * restitution bias, warm starting with impulses carried across steps, velocity iterations,
 * position integration and the non-linear Gauss-Seidel position iterations.
 *
 * Every function is templated on the scalar type. With T = float the forward functions repeat
 * the solver kernel's IEEE operations in the same order, so a replay reproduces the GPU forward
 * bit for bit; with T = double they are the host reference used to check the GPU gradient.
 */
#ifndef B2G_ADJOINT_CUH
#define B2G_ADJOINT_CUH

#include "b2g_math.cuh"

#if !defined(__CUDA_ARCH__)
#include <cmath>
#endif

namespace b2g {
namespace adj {

template <class T>
struct P2 {
    T x, y;
};
template <class T> B2G_HD P2<T> p2(T x, T y) { P2<T> r; r.x = x; r.y = y; return r; }
template <class T> B2G_HD P2<T> operator+(P2<T> a, P2<T> b) { return p2(a.x + b.x, a.y + b.y); }
template <class T> B2G_HD P2<T> operator-(P2<T> a, P2<T> b) { return p2(a.x - b.x, a.y - b.y); }
template <class T> B2G_HD P2<T> operator-(P2<T> a) { return p2(-a.x, -a.y); }
template <class T> B2G_HD P2<T> operator*(T s, P2<T> a) { return p2(s * a.x, s * a.y); }
template <class T> B2G_HD P2<T>& operator+=(P2<T>& a, P2<T> b) { a.x += b.x; a.y += b.y; return a; }
template <class T> B2G_HD P2<T>& operator-=(P2<T>& a, P2<T> b) { a.x -= b.x; a.y -= b.y; return a; }
template <class T> B2G_HD T dot(P2<T> a, P2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> B2G_HD T cross(P2<T> a, P2<T> b) { return a.x * b.y - a.y * b.x; }
template <class T> B2G_HD P2<T> cross_vs(P2<T> a, T s) { return p2(s * a.y, -s * a.x); }
template <class T> B2G_HD P2<T> cross_sv(T s, P2<T> a) { return p2(-s * a.y, s * a.x); }
/* adjoint of cross(a, b) = a.x b.y - a.y b.x */
template <class T> B2G_HD void cross_bwd(P2<T> a, P2<T> b, T g, P2<T>& ga, P2<T>& gb) {
    ga.x += g * b.y;
    ga.y -= g * b.x;
    gb.x -= g * a.y;
    gb.y += g * a.x;
}
/* cross_sv(s, a) = (-s a.y, s a.x) */
template <class T> B2G_HD void cross_sv_bwd(T s, P2<T> a, P2<T> g, T& gs, P2<T>& ga) {
    gs += -g.x * a.y + g.y * a.x;
    ga.x += g.y * s;
    ga.y += -g.x * s;
}

/* manifold types, numbered as in the narrowphase (circles 0, face A 1, face B 2) */
enum { ADJ_CIRCLES = 0, ADJ_FACE_A = 1, ADJ_FACE_B = 2 };

/* correctly rounded square root in both precisions (the solver kernel's fsqrt for float) */
B2G_HD float tsqrt(float x) { return fsqrt(x); }
B2G_HD double tsqrt(double x) { return sqrt(x); }

template <class T>
struct R2 {
    T s, c;
};
B2G_HD R2<float> rot_t(float a) {
    R2<float> q;
    b2g_sincosf(a, &q.s, &q.c);
    return q;
}
B2G_HD R2<double> rot_t(double a) {
    R2<double> q;
    q.s = sin(a);
    q.c = cos(a);
    return q;
}
template <class T> B2G_HD P2<T> mulq(R2<T> q, P2<T> v) { return p2(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
/* d/da of R(a) v */
template <class T> B2G_HD P2<T> dmulq(R2<T> q, P2<T> v) { return p2(-q.s * v.x - q.c * v.y, q.c * v.x - q.s * v.y); }
/* transform: p = c - R(a) lc; x = (R v) + p with the reference's grouping ((c v.x - s v.y) + p.x) */
template <class T> B2G_HD P2<T> xf_apply(R2<T> q, P2<T> p, P2<T> v) {
    return p2((q.c * v.x - q.s * v.y) + p.x, (q.s * v.x + q.c * v.y) + p.y);
}

/* ---- per-body static data and per-slot frozen structure ---- */
struct BodyStatic {
    float m, invm, I, invI;
    float lin_damp, ang_damp, gscale;
    float lcx, lcy;
    int type;  /* 0 static, 1 kinematic, 2 dynamic */
};

struct SlotStatic {
    int a, b;             /* world-local body indices */
    int flags;            /* bit0: A dynamic, bit1: B dynamic */
    int mtype, count;     /* manifold type and point count */
    int colour;           /* dense colour of the slot within the step */
    int island;           /* island id within the world */
    int carry[2];         /* impulse source per point: previous step's slot * 2 + point, or -1 */
    float ln[2], lpt[2], lp[4];
    float mA, mB, iA, iB, rA, rB;
    float friction, restitution, threshold;
};

/* velocity-constraint data computed at initialisation (the same values the solver kernel stores) */
template <class T>
struct VC {
    P2<T> n;
    P2<T> ra[2], rb[2];
    T nm[2], tm[2], bias[2];
    T k11, k12, k22, na, nbc, nd;
    int vcount;
    int bias_on[2];
};

/* decisions of one velocity update of a slot: friction state per point (0 interior, 1 +max,
 * 2 -max), normal state (1-point: 0 interior, 1 clamped at zero; 2-point: block case 1..4,
 * 0 = none solved) */
struct VelDecision {
    unsigned char fr[2];
    unsigned char nrm;
};

/* ---------------- forward functions (mirror k_solve arithmetic) ---------------- */

template <class T>
B2G_HD void integrate_velocity(const BodyStatic& bs, T h, T gx, T gy, P2<T>& v, T& w) {
    if (bs.type != 2) return;
    const T s = h * (T)bs.invm;
    const T gm = (T)bs.gscale * (T)bs.m;
    const T fx = gm * gx + (T)0;
    const T fy = gm * gy + (T)0;
    v.x += s * fx;
    v.y += s * fy;
    w += h * (T)bs.invI * (T)0;
    const T ld = (T)1 / ((T)1 + h * (T)bs.lin_damp);
    const T ad = (T)1 / ((T)1 + h * (T)bs.ang_damp);
    v.x *= ld;
    v.y *= ld;
    w *= ad;
}

template <class T>
B2G_HD void world_manifold(const SlotStatic& s, R2<T> qA, P2<T> pA, R2<T> qB, P2<T> pB, P2<T>& normal, P2<T> wp[2]) {
    const P2<T> ln = p2((T)s.ln[0], (T)s.ln[1]), lpt = p2((T)s.lpt[0], (T)s.lpt[1]);
    const P2<T> lp[2] = {p2((T)s.lp[0], (T)s.lp[1]), p2((T)s.lp[2], (T)s.lp[3])};
    const T rA = (T)s.rA, rB = (T)s.rB;
    normal = p2((T)1, (T)0);
    if (s.mtype == ADJ_CIRCLES) {
        P2<T> pa = xf_apply(qA, pA, lpt);
        P2<T> pb = xf_apply(qB, pB, lp[0]);
        P2<T> d = pa - pb;
        if (dot(d, d) > (T)kEpsilon * (T)kEpsilon) {
            normal = pb - pa;
            T len = tsqrt(normal.x * normal.x + normal.y * normal.y);
            if (len >= (T)kEpsilon) {
                T inv = (T)1 / len;
                normal.x *= inv;
                normal.y *= inv;
            }
        }
        P2<T> ca = pa + rA * normal;
        P2<T> cb = pb - rB * normal;
        wp[0] = (T)0.5 * (ca + cb);
    } else if (s.mtype == ADJ_FACE_A) {
        normal = mulq(qA, ln);
        P2<T> plane = xf_apply(qA, pA, lpt);
        for (int j = 0; j < s.count; ++j) {
            P2<T> clip = xf_apply(qB, pB, lp[j]);
            P2<T> ca = clip + (rA - dot(clip - plane, normal)) * normal;
            P2<T> cb = clip - rB * normal;
            wp[j] = (T)0.5 * (ca + cb);
        }
    } else {
        normal = mulq(qB, ln);
        P2<T> plane = xf_apply(qB, pB, lpt);
        for (int j = 0; j < s.count; ++j) {
            P2<T> clip = xf_apply(qA, pA, lp[j]);
            P2<T> cb = clip + (rB - dot(clip - plane, normal)) * normal;
            P2<T> ca = clip - rA * normal;
            wp[j] = (T)0.5 * (ca + cb);
        }
        normal = -normal;
    }
}

/* B2contactSolver::initialize_velocity_constraints for one slot. With frozen set, the caller
 * fills vc.vcount and vc.bias_on[] and they replace the block-solver condition test and the
 * restitution trigger. */
template <class T>
B2G_HD void init_slot(const SlotStatic& s, P2<T> cA, T aA, P2<T> cB, T aB, P2<T> vA, T wA, P2<T> vB, T wB,
                      const P2<T>& lcA, const P2<T>& lcB, VC<T>& vc, bool frozen = false) {
    const int fz_vcount = frozen ? vc.vcount : 0;
    const int fz_bias[2] = {frozen ? vc.bias_on[0] : 0, frozen ? vc.bias_on[1] : 0};
    const T mA = (T)s.mA, mB = (T)s.mB, iA = (T)s.iA, iB = (T)s.iB;
    R2<T> qA = rot_t(aA), qB = rot_t(aB);
    P2<T> pA = cA - mulq(qA, lcA), pB = cB - mulq(qB, lcB);
    P2<T> wp[2] = {p2((T)0, (T)0), p2((T)0, (T)0)};
    world_manifold(s, qA, pA, qB, pB, vc.n, wp);
    const P2<T> t = cross_vs(vc.n, (T)1);
    for (int j = 0; j < 2; ++j) {
        vc.ra[j] = vc.rb[j] = p2((T)0, (T)0);
        vc.nm[j] = vc.tm[j] = vc.bias[j] = (T)0;
        vc.bias_on[j] = 0;
    }
    for (int j = 0; j < s.count; ++j) {
        vc.ra[j] = wp[j] - cA;
        vc.rb[j] = wp[j] - cB;
        T rnA = cross(vc.ra[j], vc.n), rnB = cross(vc.rb[j], vc.n);
        T kN = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        vc.nm[j] = kN > (T)0 ? (T)1 / kN : (T)0;
        T rtA = cross(vc.ra[j], t), rtB = cross(vc.rb[j], t);
        T kT = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
        vc.tm[j] = kT > (T)0 ? (T)1 / kT : (T)0;
        T vRel = dot(vc.n, ((vB + cross_sv(wB, vc.rb[j])) - vA) - cross_sv(wA, vc.ra[j]));
        if (frozen ? fz_bias[j] != 0 : (vRel < -(T)s.threshold)) {
            vc.bias[j] = -(T)s.restitution * vRel;
            vc.bias_on[j] = 1;
        }
    }
    vc.vcount = s.count;
    vc.k11 = vc.k12 = vc.k22 = vc.na = vc.nbc = vc.nd = (T)0;
    if (s.count == 2) {
        T rn1A = cross(vc.ra[0], vc.n), rn1B = cross(vc.rb[0], vc.n);
        T rn2A = cross(vc.ra[1], vc.n), rn2B = cross(vc.rb[1], vc.n);
        T k11 = mA + mB + iA * rn1A * rn1A + iB * rn1B * rn1B;
        T k22 = mA + mB + iA * rn2A * rn2A + iB * rn2B * rn2B;
        T k12 = mA + mB + iA * rn1A * rn2A + iB * rn1B * rn2B;
        if (frozen ? fz_vcount == 2 : (k11 * k11 < (T)1000 * (k11 * k22 - k12 * k12))) {
            T det = k11 * k22 - k12 * k12;
            if (det != (T)0) det = (T)1 / det;
            vc.k11 = k11;
            vc.k12 = k12;
            vc.k22 = k22;
            vc.na = det * k22;
            vc.nbc = -det * k12;
            vc.nd = det * k11;
        } else {
            vc.vcount = 1;
        }
    }
}

template <class T>
B2G_HD void warm_slot(const SlotStatic& s, const VC<T>& vc, const T ni[2], const T ti[2], P2<T>& vA, T& wA, P2<T>& vB,
                      T& wB) {
    const P2<T> t = cross_vs(vc.n, (T)1);
    for (int j = 0; j < vc.vcount; ++j) {
        P2<T> P = ni[j] * vc.n + ti[j] * t;
        wA -= (T)s.iA * cross(vc.ra[j], P);
        vA -= (T)s.mA * P;
        wB += (T)s.iB * cross(vc.rb[j], P);
        vB += (T)s.mB * P;
    }
}

template <class T>
B2G_HD T fmin_r(T a, T b) { return a < b ? a : b; }
template <class T>
B2G_HD T fmax_r(T a, T b) { return a > b ? a : b; }

/* One velocity update of a slot. record: write the decisions taken; replay with frozen
 * decisions is done by solve_velocity_frozen (used by finite differences of the frozen model). */
template <class T>
B2G_HD void solve_velocity(const SlotStatic& s, const VC<T>& vc, T ni[2], T ti[2], P2<T>& vA, T& wA, P2<T>& vB, T& wB,
                           VelDecision& dec, bool frozen) {
    const T mA = (T)s.mA, mB = (T)s.mB, iA = (T)s.iA, iB = (T)s.iB;
    const P2<T> n = vc.n, t = cross_vs(vc.n, (T)1);
    const T friction = (T)s.friction;
    for (int j = 0; j < vc.vcount; ++j) {
        P2<T> dv = ((vB + cross_sv(wB, vc.rb[j])) - vA) - cross_sv(wA, vc.ra[j]);
        T vt = dot(dv, t) - (T)0;
        T lambda = vc.tm[j] * (-vt);
        T maxF = friction * ni[j];
        T cand = ti[j] + lambda;
        T newI;
        if (!frozen) {
            /* fclampr(cand, -maxF, maxF) = max(-maxF, min(cand, maxF)) */
            T mn = fmin_r(cand, maxF);
            unsigned char st = (cand < maxF) ? 0 : 1;
            newI = fmax_r(-maxF, mn);
            if (!(-maxF > mn)) {
                dec.fr[j] = st;
            } else {
                dec.fr[j] = 2;
            }
        } else {
            newI = dec.fr[j] == 0 ? cand : (dec.fr[j] == 1 ? maxF : -maxF);
        }
        lambda = newI - ti[j];
        ti[j] = newI;
        P2<T> P = lambda * t;
        vA -= mA * P;
        wA -= iA * cross(vc.ra[j], P);
        vB += mB * P;
        wB += iB * cross(vc.rb[j], P);
    }
    if (vc.vcount == 1) {
        P2<T> dv = ((vB + cross_sv(wB, vc.rb[0])) - vA) - cross_sv(wA, vc.ra[0]);
        T vn = dot(dv, n);
        T lambda = -vc.nm[0] * (vn - vc.bias[0]);
        T cand = ni[0] + lambda;
        T newI;
        if (!frozen) {
            newI = fmax_r(cand, (T)0);
            dec.nrm = (cand > (T)0) ? 0 : 1;
        } else {
            newI = dec.nrm == 0 ? cand : (T)0;
        }
        lambda = newI - ni[0];
        ni[0] = newI;
        P2<T> P = lambda * n;
        vA -= mA * P;
        wA -= iA * cross(vc.ra[0], P);
        vB += mB * P;
        wB += iB * cross(vc.rb[0], P);
    } else {
        const P2<T> a = p2(ni[0], ni[1]);
        P2<T> dv1 = ((vB + cross_sv(wB, vc.rb[0])) - vA) - cross_sv(wA, vc.ra[0]);
        P2<T> dv2 = ((vB + cross_sv(wB, vc.rb[1])) - vA) - cross_sv(wA, vc.ra[1]);
        T vn1 = dot(dv1, n), vn2 = dot(dv2, n);
        P2<T> b = p2(vn1 - vc.bias[0], vn2 - vc.bias[1]);
        b = b - p2(vc.k11 * a.x + vc.k12 * a.y, vc.k12 * a.x + vc.k22 * a.y);
        P2<T> x = p2((T)0, (T)0);
        int cs = 0;
        if (!frozen) {
            x = -p2(vc.na * b.x + vc.nbc * b.y, vc.nbc * b.x + vc.nd * b.y);
            if (x.x >= (T)0 && x.y >= (T)0) cs = 1;
            if (!cs) {
                x.x = -vc.nm[0] * b.x;
                x.y = (T)0;
                vn2 = vc.k12 * x.x + b.y;
                if (x.x >= (T)0 && vn2 >= (T)0) cs = 2;
            }
            if (!cs) {
                x.x = (T)0;
                x.y = -vc.nm[1] * b.y;
                vn1 = vc.k12 * x.y + b.x;
                if (x.y >= (T)0 && vn1 >= (T)0) cs = 3;
            }
            if (!cs) {
                x.x = (T)0;
                x.y = (T)0;
                vn1 = b.x;
                vn2 = b.y;
                if (vn1 >= (T)0 && vn2 >= (T)0) cs = 4;
            }
            dec.nrm = (unsigned char)cs;
        } else {
            cs = dec.nrm;
            if (cs == 1) x = -p2(vc.na * b.x + vc.nbc * b.y, vc.nbc * b.x + vc.nd * b.y);
            else if (cs == 2) x = p2(-vc.nm[0] * b.x, (T)0);
            else if (cs == 3) x = p2((T)0, -vc.nm[1] * b.y);
            else x = p2((T)0, (T)0);
        }
        if (cs) {
            P2<T> d = x - a;
            P2<T> P1 = d.x * n, P2_ = d.y * n;
            vA -= mA * (P1 + P2_);
            wA -= iA * (cross(vc.ra[0], P1) + cross(vc.ra[1], P2_));
            vB += mB * (P1 + P2_);
            wB += iB * (cross(vc.rb[0], P1) + cross(vc.rb[1], P2_));
            ni[0] = x.x;
            ni[1] = x.y;
        }
    }
}

/* translation / rotation clamps of position integration (b2_island_private.rs:222-252) */
template <class T>
B2G_HD void integrate_position(T h, P2<T>& c, T& a, P2<T>& v, T& w, unsigned char& clamp, bool frozen) {
    P2<T> tr = h * v;
    unsigned char cl = 0;
    if (frozen ? (clamp & 1) : (dot(tr, tr) > (T)kMaxTranslationSquared)) {
        T ratio = (T)kMaxTranslation / tsqrt(tr.x * tr.x + tr.y * tr.y);
        v.x *= ratio;
        v.y *= ratio;
        cl |= 1;
    }
    T r = h * w;
    if (frozen ? (clamp & 2) : (r * r > (T)kMaxRotationSquared)) {
        T ratio = (T)kMaxRotation / (r < (T)0 ? -r : r);
        w *= ratio;
        cl |= 2;
    }
    c.x += h * v.x;
    c.y += h * v.y;
    a += h * w;
    if (!frozen) clamp = cl;
}

/* position manifold of one point (B2positionSolverManifold::initialize) */
template <class T>
B2G_HD void position_manifold(const SlotStatic& s, int j, R2<T> qA, P2<T> pA, R2<T> qB, P2<T> pB, P2<T>& normal,
                              P2<T>& point, T& sep) {
    const P2<T> ln = p2((T)s.ln[0], (T)s.ln[1]), lpt = p2((T)s.lpt[0], (T)s.lpt[1]);
    const P2<T> lp = p2((T)s.lp[2 * j], (T)s.lp[2 * j + 1]);
    const T rA = (T)s.rA, rB = (T)s.rB;
    if (s.mtype == ADJ_CIRCLES) {
        P2<T> pa = xf_apply(qA, pA, lpt);
        P2<T> pb = xf_apply(qB, pB, p2((T)s.lp[0], (T)s.lp[1]));
        normal = pb - pa;
        T len = tsqrt(normal.x * normal.x + normal.y * normal.y);
        if (len >= (T)kEpsilon) {
            T inv = (T)1 / len;
            normal.x *= inv;
            normal.y *= inv;
        }
        point = (T)0.5 * (pa + pb);
        sep = dot(pb - pa, normal) - rA - rB;
    } else if (s.mtype == ADJ_FACE_A) {
        normal = mulq(qA, ln);
        P2<T> plane = xf_apply(qA, pA, lpt);
        P2<T> clip = xf_apply(qB, pB, lp);
        sep = dot(clip - plane, normal) - rA - rB;
        point = clip;
    } else {
        normal = mulq(qB, ln);
        P2<T> plane = xf_apply(qB, pB, lpt);
        P2<T> clip = xf_apply(qA, pA, lp);
        sep = dot(clip - plane, normal) - rA - rB;
        point = clip;
        normal = -normal;
    }
}

/* one slot of solve_position_constraints; dec holds the C clamp state per point
 * (0 interior, 1 at -max correction, 2 at 0). Returns the slot's min separation (<= 0). */
template <class T>
B2G_HD T solve_position(const SlotStatic& s, const P2<T>& lcA, const P2<T>& lcB, P2<T>& cA, T& aA, P2<T>& cB, T& aB,
                        unsigned char dec[2], bool frozen) {
    const T mA = (T)s.mA, mB = (T)s.mB, iA = (T)s.iA, iB = (T)s.iB;
    T minSep = (T)0;
    for (int j = 0; j < s.count; ++j) {
        R2<T> qA = rot_t(aA), qB = rot_t(aB);
        P2<T> pA = cA - mulq(qA, lcA), pB = cB - mulq(qB, lcB);
        P2<T> normal, point;
        T sep;
        position_manifold(s, j, qA, pA, qB, pB, normal, point, sep);
        P2<T> ra = point - cA, rb = point - cB;
        minSep = fmin_r(minSep, sep);
        T arg = (T)kBaumgarte * (sep + (T)kLinearSlop);
        T C;
        if (!frozen) {
            /* clamp(arg, -maxCorr, 0) = max(-maxCorr, min(arg, 0)) */
            T mn = fmin_r(arg, (T)0);
            C = fmax_r(-(T)kMaxLinearCorrection, mn);
            dec[j] = (-(T)kMaxLinearCorrection > mn) ? 1 : ((arg < (T)0) ? 0 : 2);
        } else {
            C = dec[j] == 0 ? arg : (dec[j] == 1 ? -(T)kMaxLinearCorrection : (T)0);
        }
        T rnA = cross(ra, normal), rnB = cross(rb, normal);
        T K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        T impulse = K > (T)0 ? -C / K : (T)0;
        P2<T> P = impulse * normal;
        cA -= mA * P;
        aA -= iA * cross(ra, P);
        cB += mB * P;
        aB += iB * cross(rb, P);
    }
    return minSep;
}

/* ======================= reverse mode (adjoints accumulate with +=) ======================= */

/* d/da of (s, c) = (c, -s): accumulate the angle adjoint from adjoints of s and c */
template <class T> B2G_HD T rot_bwd(R2<T> q, T gs, T gc) { return gs * q.c - gc * q.s; }

/* y = R v (v constant): adjoints of (s, c) */
template <class T> B2G_HD void mulq_bwd_q(P2<T> v, P2<T> gy, T& gs, T& gc) {
    gc += gy.x * v.x + gy.y * v.y;
    gs += -gy.x * v.y + gy.y * v.x;
}

template <class T> struct VCGrad {
    P2<T> n;
    P2<T> ra[2], rb[2];
    T nm[2], tm[2], bias[2];
    T k11, k12, k22, na, nbc, nd;
};
template <class T> B2G_HD void zero(VCGrad<T>& g) {
    g.n = p2((T)0, (T)0);
    for (int j = 0; j < 2; ++j) {
        g.ra[j] = g.rb[j] = p2((T)0, (T)0);
        g.nm[j] = g.tm[j] = g.bias[j] = (T)0;
    }
    g.k11 = g.k12 = g.k22 = g.na = g.nbc = g.nd = (T)0;
}
/* t = cross_vs(n, 1) = (n.y, -n.x): fold a tangent adjoint into the normal adjoint */
template <class T> B2G_HD void tangent_bwd(P2<T> gt, P2<T>& gn) {
    gn.x += -gt.y;
    gn.y += gt.x;
}

template <class T>
B2G_HD void integrate_velocity_bwd(const BodyStatic& bs, T h, P2<T>& gv, T& gw) {
    if (bs.type != 2) return;
    const T ld = (T)1 / ((T)1 + h * (T)bs.lin_damp);
    const T ad = (T)1 / ((T)1 + h * (T)bs.ang_damp);
    gv.x *= ld;
    gv.y *= ld;
    gw *= ad;
}

/* body update v -= m P, w -= i cross(r, P) (sign = -1) or += (sign = +1): adjoint of P and r */
template <class T>
B2G_HD void apply_bwd(T sign, T m, T i, P2<T> r, P2<T> P, P2<T> gv, T gw, P2<T>& gP, P2<T>& gr) {
    gP += (sign * m) * gv;
    P2<T> dPr = p2((T)0, (T)0), dPp = p2((T)0, (T)0);
    cross_bwd(r, P, sign * i * gw, dPr, dPp);
    gr += dPr;
    gP += dPp;
}

template <class T>
B2G_HD void warm_slot_bwd(const SlotStatic& s, const VC<T>& vc, const T ni[2], const T ti[2], P2<T> gvA, T gwA,
                          P2<T> gvB, T gwB, T gni[2], T gti[2], VCGrad<T>& g) {
    const P2<T> t = cross_vs(vc.n, (T)1);
    P2<T> gt = p2((T)0, (T)0);
    for (int j = 0; j < vc.vcount; ++j) {
        P2<T> P = ni[j] * vc.n + ti[j] * t;
        P2<T> gP = p2((T)0, (T)0);
        apply_bwd((T)-1, (T)s.mA, (T)s.iA, vc.ra[j], P, gvA, gwA, gP, g.ra[j]);
        apply_bwd((T)1, (T)s.mB, (T)s.iB, vc.rb[j], P, gvB, gwB, gP, g.rb[j]);
        gni[j] += dot(gP, vc.n);
        gti[j] += dot(gP, t);
        g.n += ni[j] * gP;
        gt += ti[j] * gP;
    }
    tangent_bwd(gt, g.n);
}

/* dv = ((vB + cross_sv(wB, rb)) - vA) - cross_sv(wA, ra): adjoints from gdv */
template <class T>
B2G_HD void relvel_bwd(T wA, T wB, P2<T> ra, P2<T> rb, P2<T> gdv, P2<T>& gvA, T& gwA, P2<T>& gvB, T& gwB, P2<T>& gra,
                       P2<T>& grb) {
    gvB += gdv;
    gvA -= gdv;
    cross_sv_bwd(wB, rb, gdv, gwB, grb);
    cross_sv_bwd(wA, ra, -gdv, gwA, gra);
}

/* Adjoint of solve_velocity with frozen decisions. Inputs are the pre-update values; the
 * adjoint arguments hold the post-update adjoints on entry and the pre-update ones on exit. */
template <class T>
B2G_HD void solve_velocity_bwd(const SlotStatic& s, const VC<T>& vc, const VelDecision& dec, const T ni_in[2],
                               const T ti_in[2], P2<T> vA, T wA, P2<T> vB, T wB, T gni[2], T gti[2], P2<T>& gvA,
                               T& gwA, P2<T>& gvB, T& gwB, VCGrad<T>& g) {
    const T mA = (T)s.mA, mB = (T)s.mB, iA = (T)s.iA, iB = (T)s.iB;
    const P2<T> n = vc.n, t = cross_vs(vc.n, (T)1);
    const T friction = (T)s.friction;
    /* forward again, keeping the intermediates */
    T ni[2] = {ni_in[0], ni_in[1]}, ti[2] = {ti_in[0], ti_in[1]};
    P2<T> fvA[2], fvB[2];
    T fwA[2], fwB[2], flam[2];
    for (int j = 0; j < vc.vcount; ++j) {
        fvA[j] = vA; fwA[j] = wA; fvB[j] = vB; fwB[j] = wB;
        P2<T> dv = ((vB + cross_sv(wB, vc.rb[j])) - vA) - cross_sv(wA, vc.ra[j]);
        T vt = dot(dv, t) - (T)0;
        T lambda = vc.tm[j] * (-vt);
        T maxF = friction * ni[j];
        T cand = ti[j] + lambda;
        T newI = dec.fr[j] == 0 ? cand : (dec.fr[j] == 1 ? maxF : -maxF);
        lambda = newI - ti[j];
        flam[j] = lambda;
        ti[j] = newI;
        P2<T> P = lambda * t;
        vA -= mA * P;
        wA -= iA * cross(vc.ra[j], P);
        vB += mB * P;
        wB += iB * cross(vc.rb[j], P);
    }
    P2<T> gt = p2((T)0, (T)0);
    /* ---- normal part, reversed ---- */
    if (vc.vcount == 1) {
        P2<T> dv = ((vB + cross_sv(wB, vc.rb[0])) - vA) - cross_sv(wA, vc.ra[0]);
        T vn = dot(dv, n);
        T lambda = -vc.nm[0] * (vn - vc.bias[0]);
        T cand = ni[0] + lambda;
        T newI = dec.nrm == 0 ? cand : (T)0;
        T lam2 = newI - ni[0];
        P2<T> P = lam2 * n;
        P2<T> gP = p2((T)0, (T)0);
        apply_bwd((T)-1, mA, iA, vc.ra[0], P, gvA, gwA, gP, g.ra[0]);
        apply_bwd((T)1, mB, iB, vc.rb[0], P, gvB, gwB, gP, g.rb[0]);
        T glam2 = dot(gP, n);
        g.n += lam2 * gP;
        /* ni' = newI; lam2 = newI - ni */
        T gnew = gni[0] + glam2;
        T gni_pre = -glam2;
        T gcand = dec.nrm == 0 ? gnew : (T)0;
        gni_pre += gcand;
        T glam = gcand;
        /* lambda = -nm (vn - bias) */
        g.nm[0] += -(vn - vc.bias[0]) * glam;
        T gvn = -vc.nm[0] * glam;
        g.bias[0] += vc.nm[0] * glam;
        P2<T> gdv = gvn * n;
        g.n += gvn * dv;
        relvel_bwd(wA, wB, vc.ra[0], vc.rb[0], gdv, gvA, gwA, gvB, gwB, g.ra[0], g.rb[0]);
        gni[0] = gni_pre;
    } else {
        const P2<T> a = p2(ni[0], ni[1]);
        P2<T> dv1 = ((vB + cross_sv(wB, vc.rb[0])) - vA) - cross_sv(wA, vc.ra[0]);
        P2<T> dv2 = ((vB + cross_sv(wB, vc.rb[1])) - vA) - cross_sv(wA, vc.ra[1]);
        T vn1 = dot(dv1, n), vn2 = dot(dv2, n);
        P2<T> b0 = p2(vn1 - vc.bias[0], vn2 - vc.bias[1]);
        P2<T> b = b0 - p2(vc.k11 * a.x + vc.k12 * a.y, vc.k12 * a.x + vc.k22 * a.y);
        const int cs = dec.nrm;
        P2<T> x = a;
        if (cs == 1) x = -p2(vc.na * b.x + vc.nbc * b.y, vc.nbc * b.x + vc.nd * b.y);
        else if (cs == 2) x = p2(-vc.nm[0] * b.x, (T)0);
        else if (cs == 3) x = p2((T)0, -vc.nm[1] * b.y);
        else if (cs == 4) x = p2((T)0, (T)0);
        P2<T> gx = p2(gni[0], gni[1]);  /* ni' = x */
        P2<T> ga = p2((T)0, (T)0);
        if (cs) {
            P2<T> d = x - a;
            P2<T> P1 = d.x * n, P2_ = d.y * n;
            /* vA -= mA (P1 + P2); wA -= iA (cross(ra0, P1) + cross(ra1, P2)); same for B with + */
            P2<T> gP1 = p2((T)0, (T)0), gP2 = p2((T)0, (T)0);
            gP1 += (-mA) * gvA;
            gP2 += (-mA) * gvA;
            gP1 += mB * gvB;
            gP2 += mB * gvB;
            cross_bwd(vc.ra[0], P1, -iA * gwA, g.ra[0], gP1);
            cross_bwd(vc.ra[1], P2_, -iA * gwA, g.ra[1], gP2);
            cross_bwd(vc.rb[0], P1, iB * gwB, g.rb[0], gP1);
            cross_bwd(vc.rb[1], P2_, iB * gwB, g.rb[1], gP2);
            P2<T> gd = p2(dot(gP1, n), dot(gP2, n));
            g.n += d.x * gP1 + d.y * gP2;
            gx += gd;
            ga -= gd;
        } else {
            ga += gx;  /* no update: ni' = a */
            gx = p2((T)0, (T)0);
        }
        P2<T> gb = p2((T)0, (T)0);
        if (cs == 1) {
            gb.x += -(vc.na * gx.x + vc.nbc * gx.y);
            gb.y += -(vc.nbc * gx.x + vc.nd * gx.y);
            g.na += -b.x * gx.x;
            g.nbc += -(b.y * gx.x + b.x * gx.y);
            g.nd += -b.y * gx.y;
        } else if (cs == 2) {
            gb.x += -vc.nm[0] * gx.x;
            g.nm[0] += -b.x * gx.x;
        } else if (cs == 3) {
            gb.y += -vc.nm[1] * gx.y;
            g.nm[1] += -b.y * gx.y;
        }
        /* b = b0 - K a */
        ga.x -= vc.k11 * gb.x + vc.k12 * gb.y;
        ga.y -= vc.k12 * gb.x + vc.k22 * gb.y;
        g.k11 += -a.x * gb.x;
        g.k12 += -(a.y * gb.x + a.x * gb.y);
        g.k22 += -a.y * gb.y;
        T gvn1 = gb.x, gvn2 = gb.y;
        g.bias[0] += -gb.x;
        g.bias[1] += -gb.y;
        g.n += gvn1 * dv1 + gvn2 * dv2;
        relvel_bwd(wA, wB, vc.ra[0], vc.rb[0], gvn1 * n, gvA, gwA, gvB, gwB, g.ra[0], g.rb[0]);
        relvel_bwd(wA, wB, vc.ra[1], vc.rb[1], gvn2 * n, gvA, gwA, gvB, gwB, g.ra[1], g.rb[1]);
        gni[0] = ga.x;
        gni[1] = ga.y;
    }
    /* ---- friction part, reversed ---- */
    for (int j = vc.vcount - 1; j >= 0; --j) {
        const T lambda = flam[j];
        const P2<T> P = lambda * t;
        P2<T> gP = p2((T)0, (T)0);
        apply_bwd((T)-1, mA, iA, vc.ra[j], P, gvA, gwA, gP, g.ra[j]);
        apply_bwd((T)1, mB, iB, vc.rb[j], P, gvB, gwB, gP, g.rb[j]);
        T glam2 = dot(gP, t);
        gt += lambda * gP;
        /* ti' = newI; lambda2 = newI - ti */
        T gnew = gti[j] + glam2;
        T gti_pre = -glam2;
        T gcand = (T)0, gmax = (T)0;
        if (dec.fr[j] == 0) gcand = gnew;
        else if (dec.fr[j] == 1) gmax = gnew;
        else gmax = -gnew;
        gni[j] += friction * gmax;  /* maxF = friction * ni (ni unchanged by friction) */
        gti_pre += gcand;
        T glam = gcand;
        /* lambda = tm * (-vt); vt = dot(dv, t) */
        P2<T> dv = ((fvB[j] + cross_sv(fwB[j], vc.rb[j])) - fvA[j]) - cross_sv(fwA[j], vc.ra[j]);
        T vt = dot(dv, t);
        g.tm[j] += -vt * glam;
        T gvt = -vc.tm[j] * glam;
        gt += gvt * dv;
        relvel_bwd(fwA[j], fwB[j], vc.ra[j], vc.rb[j], gvt * t, gvA, gwA, gvB, gwB, g.ra[j], g.rb[j]);
        gti[j] = gti_pre;
    }
    tangent_bwd(gt, g.n);
}

/* adjoint of the world manifold (normal, points) w.r.t. (qA, pA, qB, pB) */
template <class T>
B2G_HD void world_manifold_bwd(const SlotStatic& s, R2<T> qA, P2<T> pA, R2<T> qB, P2<T> pB, P2<T> gn, const P2<T> gwp[2],
                               T& gsA, T& gcA, P2<T>& gpA, T& gsB, T& gcB, P2<T>& gpB) {
    const P2<T> ln = p2((T)s.ln[0], (T)s.ln[1]), lpt = p2((T)s.lpt[0], (T)s.lpt[1]);
    const P2<T> lp[2] = {p2((T)s.lp[0], (T)s.lp[1]), p2((T)s.lp[2], (T)s.lp[3])};
    const T rA = (T)s.rA, rB = (T)s.rB;
    if (s.mtype == ADJ_CIRCLES) {
        P2<T> pa = xf_apply(qA, pA, lpt);
        P2<T> pb = xf_apply(qB, pB, lp[0]);
        P2<T> d = pa - pb;
        bool normalised = false;
        P2<T> n = p2((T)1, (T)0);
        P2<T> dd = pb - pa;
        T len = (T)0;
        if (dot(d, d) > (T)kEpsilon * (T)kEpsilon) {
            n = dd;
            len = tsqrt(n.x * n.x + n.y * n.y);
            if (len >= (T)kEpsilon) {
                T inv = (T)1 / len;
                n.x *= inv;
                n.y *= inv;
                normalised = true;
            }
        }
        /* wp0 = 0.5 (pa + rA n + pb - rB n) */
        P2<T> gw = gwp[0];
        P2<T> gpa = (T)0.5 * gw, gpb = (T)0.5 * gw;
        P2<T> gnn = gn + ((T)0.5 * (rA - rB)) * gw;
        if (dot(d, d) > (T)kEpsilon * (T)kEpsilon) {
            P2<T> gdd = normalised ? ((T)1 / len) * (gnn - dot(gnn, n) * n) : gnn;
            gpb += gdd;
            gpa -= gdd;
        }
        gpA += gpa;
        mulq_bwd_q(lpt, gpa, gsA, gcA);
        gpB += gpb;
        mulq_bwd_q(lp[0], gpb, gsB, gcB);
        return;
    }
    const bool faceA = s.mtype == ADJ_FACE_A;
    /* reference body R (face owner) and incident body I */
    R2<T> qR = faceA ? qA : qB, qI = faceA ? qB : qA;
    P2<T> pR = faceA ? pA : pB, pI = faceA ? pB : pA;
    const T rR = faceA ? rA : rB, rI = faceA ? rB : rA;
    P2<T> nr = mulq(qR, ln);               /* raw normal (before the FaceB flip) */
    P2<T> plane = xf_apply(qR, pR, lpt);
    P2<T> gnr = faceA ? gn : -gn;
    T gsR = (T)0, gcR = (T)0, gsI = (T)0, gcI = (T)0;
    P2<T> gpR = p2((T)0, (T)0), gpI = p2((T)0, (T)0), gplane = p2((T)0, (T)0);
    for (int j = 0; j < s.count; ++j) {
        P2<T> clip = xf_apply(qI, pI, lp[j]);
        T u = rR - dot(clip - plane, nr);
        /* wp = 0.5 ((clip + u nr) + (clip - rI nr)) */
        P2<T> gw = gwp[j];
        P2<T> gc_on = (T)0.5 * gw, gc_in = (T)0.5 * gw;
        P2<T> gclip = gc_on + gc_in;
        gnr += (-rI) * gc_in;
        T gu = dot(gc_on, nr);
        gnr += u * gc_on;
        gclip += (-gu) * nr;
        gplane += gu * nr;
        gnr += (-gu) * (clip - plane);
        gpI += gclip;
        mulq_bwd_q(lp[j], gclip, gsI, gcI);
    }
    gpR += gplane;
    mulq_bwd_q(lpt, gplane, gsR, gcR);
    mulq_bwd_q(ln, gnr, gsR, gcR);
    if (faceA) {
        gsA += gsR; gcA += gcR; gpA += gpR; gsB += gsI; gcB += gcI; gpB += gpI;
    } else {
        gsB += gsR; gcB += gcR; gpB += gpR; gsA += gsI; gcA += gcI; gpA += gpI;
    }
}

/* adjoint of init_slot: from the VC adjoint to the poses (c, a) at solve start and the
 * velocities after integration (restitution bias) */
template <class T>
B2G_HD void init_slot_bwd(const SlotStatic& s, P2<T> cA, T aA, P2<T> cB, T aB, P2<T> vA, T wA, P2<T> vB, T wB,
                          const P2<T>& lcA, const P2<T>& lcB, const VC<T>& vc, VCGrad<T> g, P2<T>& gcA, T& gaA,
                          P2<T>& gcB, T& gaB, P2<T>& gvA, T& gwA, P2<T>& gvB, T& gwB) {
    const T mA = (T)s.mA, mB = (T)s.mB, iA = (T)s.iA, iB = (T)s.iB;
    const P2<T> n = vc.n, t = cross_vs(vc.n, (T)1);
    P2<T> gt = p2((T)0, (T)0);
    /* block matrix and its inverse */
    if (s.count == 2 && vc.vcount == 2) {
        const T k11 = vc.k11, k12 = vc.k12, k22 = vc.k22;
        T D = k11 * k22 - k12 * k12;
        T det = D != (T)0 ? (T)1 / D : (T)0;
        T gk11 = g.k11, gk12 = g.k12, gk22 = g.k22;
        T gdet = k22 * g.na - k12 * g.nbc + k11 * g.nd;
        gk22 += det * g.na;
        gk12 += -det * g.nbc;
        gk11 += det * g.nd;
        if (D != (T)0) {
            T gD = -det * det * gdet;
            gk11 += k22 * gD;
            gk22 += k11 * gD;
            gk12 += (T)-2 * k12 * gD;
        }
        T rn1A = cross(vc.ra[0], n), rn1B = cross(vc.rb[0], n);
        T rn2A = cross(vc.ra[1], n), rn2B = cross(vc.rb[1], n);
        T grn1A = (T)2 * iA * rn1A * gk11 + iA * rn2A * gk12;
        T grn1B = (T)2 * iB * rn1B * gk11 + iB * rn2B * gk12;
        T grn2A = (T)2 * iA * rn2A * gk22 + iA * rn1A * gk12;
        T grn2B = (T)2 * iB * rn2B * gk22 + iB * rn1B * gk12;
        cross_bwd(vc.ra[0], n, grn1A, g.ra[0], g.n);
        cross_bwd(vc.rb[0], n, grn1B, g.rb[0], g.n);
        cross_bwd(vc.ra[1], n, grn2A, g.ra[1], g.n);
        cross_bwd(vc.rb[1], n, grn2B, g.rb[1], g.n);
    }
    P2<T> gwp[2] = {p2((T)0, (T)0), p2((T)0, (T)0)};
    for (int j = s.count - 1; j >= 0; --j) {
        const P2<T> ra = vc.ra[j], rb = vc.rb[j];
        if (vc.bias_on[j]) {
            P2<T> dv = ((vB + cross_sv(wB, rb)) - vA) - cross_sv(wA, ra);
            T gvrel = -(T)s.restitution * g.bias[j];
            g.n += gvrel * dv;
            relvel_bwd(wA, wB, ra, rb, gvrel * n, gvA, gwA, gvB, gwB, g.ra[j], g.rb[j]);
        }
        T rtA = cross(ra, t), rtB = cross(rb, t);
        T kT = mA + mB + iA * rtA * rtA + iB * rtB * rtB;
        if (kT > (T)0) {
            T gkT = -vc.tm[j] * vc.tm[j] * g.tm[j];
            cross_bwd(ra, t, (T)2 * iA * rtA * gkT, g.ra[j], gt);
            cross_bwd(rb, t, (T)2 * iB * rtB * gkT, g.rb[j], gt);
        }
        T rnA = cross(ra, n), rnB = cross(rb, n);
        T kN = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        if (kN > (T)0) {
            T gkN = -vc.nm[j] * vc.nm[j] * g.nm[j];
            cross_bwd(ra, n, (T)2 * iA * rnA * gkN, g.ra[j], g.n);
            cross_bwd(rb, n, (T)2 * iB * rnB * gkN, g.rb[j], g.n);
        }
        /* ra = wp - cA, rb = wp - cB */
        gwp[j] += g.ra[j] + g.rb[j];
        gcA -= g.ra[j];
        gcB -= g.rb[j];
    }
    tangent_bwd(gt, g.n);
    R2<T> qA = rot_t(aA), qB = rot_t(aB);
    P2<T> pA = cA - mulq(qA, lcA), pB = cB - mulq(qB, lcB);
    T gsA = (T)0, gcA_ = (T)0, gsB = (T)0, gcB_ = (T)0;
    P2<T> gpA = p2((T)0, (T)0), gpB = p2((T)0, (T)0);
    world_manifold_bwd(s, qA, pA, qB, pB, g.n, gwp, gsA, gcA_, gpA, gsB, gcB_, gpB);
    /* p = c - R(a) lc */
    gcA += gpA;
    gcB += gpB;
    mulq_bwd_q(lcA, -gpA, gsA, gcA_);
    mulq_bwd_q(lcB, -gpB, gsB, gcB_);
    gaA += rot_bwd(qA, gsA, gcA_);
    gaB += rot_bwd(qB, gsB, gcB_);
}

template <class T>
B2G_HD void integrate_position_bwd(T h, P2<T> v_in, T w_in, unsigned char clamp, P2<T>& gc, T& ga, P2<T>& gv, T& gw) {
    /* c' = c + h v1, a' = a + h w1, v' = v1, w' = w1 */
    P2<T> gv1 = gv + h * gc;
    T gw1 = gw + h * ga;
    if (clamp & 1) {
        P2<T> tr = h * v_in;
        T len = tsqrt(tr.x * tr.x + tr.y * tr.y);
        T ratio = (T)kMaxTranslation / len;
        T vv = dot(v_in, v_in);
        gv = ratio * gv1 - (ratio * dot(gv1, v_in) / vv) * v_in;
    } else {
        gv = gv1;
    }
    gw = (clamp & 2) ? (T)0 : gw1;
}

template <class T>
B2G_HD void position_manifold_bwd(const SlotStatic& s, int j, R2<T> qA, P2<T> pA, R2<T> qB, P2<T> pB, P2<T> gn,
                                  P2<T> gpoint, T gsep, T& gsA, T& gcA, P2<T>& gpA, T& gsB, T& gcB, P2<T>& gpB) {
    const P2<T> ln = p2((T)s.ln[0], (T)s.ln[1]), lpt = p2((T)s.lpt[0], (T)s.lpt[1]);
    const P2<T> lp = p2((T)s.lp[2 * j], (T)s.lp[2 * j + 1]);
    if (s.mtype == ADJ_CIRCLES) {
        const P2<T> lp0 = p2((T)s.lp[0], (T)s.lp[1]);
        P2<T> pa = xf_apply(qA, pA, lpt);
        P2<T> pb = xf_apply(qB, pB, lp0);
        P2<T> d = pb - pa;
        T len = tsqrt(d.x * d.x + d.y * d.y);
        P2<T> n = d;
        bool normalised = len >= (T)kEpsilon;
        if (normalised) n = ((T)1 / len) * d;
        /* sep = dot(d, n) - rA - rB; point = 0.5 (pa + pb) */
        P2<T> gd = gsep * n;
        P2<T> gnn = gn + gsep * d;
        gd += normalised ? ((T)1 / len) * (gnn - dot(gnn, n) * n) : gnn;
        P2<T> gpa = (T)0.5 * gpoint - gd, gpb = (T)0.5 * gpoint + gd;
        gpA += gpa;
        mulq_bwd_q(lpt, gpa, gsA, gcA);
        gpB += gpb;
        mulq_bwd_q(lp0, gpb, gsB, gcB);
        return;
    }
    const bool faceA = s.mtype == ADJ_FACE_A;
    R2<T> qR = faceA ? qA : qB, qI = faceA ? qB : qA;
    P2<T> pR = faceA ? pA : pB, pI = faceA ? pB : pA;
    P2<T> nr = mulq(qR, ln);
    P2<T> plane = xf_apply(qR, pR, lpt);
    P2<T> clip = xf_apply(qI, pI, lp);
    P2<T> gnr = faceA ? gn : -gn;
    /* sep = dot(clip - plane, nr) - rA - rB; point = clip */
    P2<T> gclip = gpoint + gsep * nr;
    P2<T> gplane = (-gsep) * nr;
    gnr += gsep * (clip - plane);
    T gsR = (T)0, gcR = (T)0, gsI = (T)0, gcI = (T)0;
    P2<T> gpR = gplane, gpI = gclip;
    mulq_bwd_q(lpt, gplane, gsR, gcR);
    mulq_bwd_q(ln, gnr, gsR, gcR);
    mulq_bwd_q(lp, gclip, gsI, gcI);
    if (faceA) {
        gsA += gsR; gcA += gcR; gpA += gpR; gsB += gsI; gcB += gcI; gpB += gpI;
    } else {
        gsB += gsR; gcB += gcR; gpB += gpR; gsA += gsI; gcA += gcI; gpA += gpI;
    }
}

/* Adjoint of one slot of solve_position with frozen clamp decisions; inputs are the pre-slot
 * poses; the pose adjoints hold post-slot values on entry and pre-slot values on exit. */
template <class T>
B2G_HD void solve_position_bwd(const SlotStatic& s, const P2<T>& lcA, const P2<T>& lcB, P2<T> cA, T aA, P2<T> cB, T aB,
                               const unsigned char dec[2], P2<T>& gcA, T& gaA, P2<T>& gcB, T& gaB) {
    const T mA = (T)s.mA, mB = (T)s.mB, iA = (T)s.iA, iB = (T)s.iB;
    P2<T> pc[2], pcB[2];
    T pa[2], paB[2];
    for (int j = 0; j < s.count; ++j) {  /* forward again to get the pre-point poses */
        pc[j] = cA; pa[j] = aA; pcB[j] = cB; paB[j] = aB;
        R2<T> qA = rot_t(aA), qB = rot_t(aB);
        P2<T> pA = cA - mulq(qA, lcA), pB = cB - mulq(qB, lcB);
        P2<T> normal, point;
        T sep;
        position_manifold(s, j, qA, pA, qB, pB, normal, point, sep);
        P2<T> ra = point - cA, rb = point - cB;
        T arg = (T)kBaumgarte * (sep + (T)kLinearSlop);
        T C = dec[j] == 0 ? arg : (dec[j] == 1 ? -(T)kMaxLinearCorrection : (T)0);
        T rnA = cross(ra, normal), rnB = cross(rb, normal);
        T K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        T impulse = K > (T)0 ? -C / K : (T)0;
        P2<T> P = impulse * normal;
        cA -= mA * P;
        aA -= iA * cross(ra, P);
        cB += mB * P;
        aB += iB * cross(rb, P);
    }
    for (int j = s.count - 1; j >= 0; --j) {
        const P2<T> cA0 = pc[j], cB0 = pcB[j];
        const T aA0 = pa[j], aB0 = paB[j];
        R2<T> qA = rot_t(aA0), qB = rot_t(aB0);
        P2<T> pA = cA0 - mulq(qA, lcA), pB = cB0 - mulq(qB, lcB);
        P2<T> normal, point;
        T sep;
        position_manifold(s, j, qA, pA, qB, pB, normal, point, sep);
        P2<T> ra = point - cA0, rb = point - cB0;
        T arg = (T)kBaumgarte * (sep + (T)kLinearSlop);
        T C = dec[j] == 0 ? arg : (dec[j] == 1 ? -(T)kMaxLinearCorrection : (T)0);
        T rnA = cross(ra, normal), rnB = cross(rb, normal);
        T K = mA + mB + iA * rnA * rnA + iB * rnB * rnB;
        T impulse = K > (T)0 ? -C / K : (T)0;
        P2<T> P = impulse * normal;
        /* cA' = cA - mA P; aA' = aA - iA cross(ra, P); cB' = cB + mB P; aB' = aB + iB cross(rb, P) */
        P2<T> gP = p2((T)0, (T)0), gra = p2((T)0, (T)0), grb = p2((T)0, (T)0);
        gP += (-mA) * gcA;
        gP += mB * gcB;
        cross_bwd(ra, P, -iA * gaA, gra, gP);
        cross_bwd(rb, P, iB * gaB, grb, gP);
        P2<T> gnormal = impulse * gP;
        T gimp = dot(gP, normal);
        T gC = (T)0, gK = (T)0;
        if (K > (T)0) {
            gC = -gimp / K;
            gK = C * gimp / (K * K);
        }
        cross_bwd(ra, normal, (T)2 * iA * rnA * gK, gra, gnormal);
        cross_bwd(rb, normal, (T)2 * iB * rnB * gK, grb, gnormal);
        T gsep = dec[j] == 0 ? (T)kBaumgarte * gC : (T)0;
        /* ra = point - cA, rb = point - cB */
        P2<T> gpoint = gra + grb;
        gcA -= gra;
        gcB -= grb;
        T gsA = (T)0, gcqA = (T)0, gsB = (T)0, gcqB = (T)0;
        P2<T> gpA = p2((T)0, (T)0), gpB = p2((T)0, (T)0);
        position_manifold_bwd(s, j, qA, pA, qB, pB, gnormal, gpoint, gsep, gsA, gcqA, gpA, gsB, gcqB, gpB);
        gcA += gpA;
        gcB += gpB;
        mulq_bwd_q(lcA, -gpA, gsA, gcqA);
        mulq_bwd_q(lcB, -gpB, gsB, gcqB);
        gaA += rot_bwd(qA, gsA, gcqA);
        gaB += rot_bwd(qB, gsB, gcqB);
    }
}

}  // namespace adj
}  // namespace b2g
#endif
