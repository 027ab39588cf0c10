/*
 * adjoint_unit.cpp — finite-difference check of every reverse-mode function in
 * b2g_adjoint.cuh, in double precision on the host.
 *
 * For random slots (circle, face-A and face-B manifolds; one and two points) and random
 * states, each forward function f is wrapped as a map from a flat input vector x to a flat
 * output vector y (decisions frozen from an unfrozen evaluation at x), a random weight vector
 * r defines L = r . y, and the hand-written adjoint's dL/dx is compared with a central
 * difference of L. Prints one line per case and exits non-zero if any relative error exceeds
 * the tolerance.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <random>
#include <vector>

#include "b2g_adjoint.cuh"

using namespace b2g::adj;
typedef double T;
typedef std::vector<double> Vec;

static std::mt19937_64 rng(12345);
static double U(double lo, double hi) { return std::uniform_real_distribution<double>(lo, hi)(rng); }

static SlotStatic random_slot(int mtype, int count) {
    SlotStatic s{};
    s.a = 0;
    s.b = 1;
    s.flags = 3;
    s.mtype = mtype;
    s.count = count;
    float ang = (float)U(0, 6.283);
    s.ln[0] = std::cos(ang);
    s.ln[1] = std::sin(ang);
    s.lpt[0] = (float)U(-0.3, 0.3);
    s.lpt[1] = (float)U(-0.3, 0.3);
    for (int i = 0; i < 4; ++i) s.lp[i] = (float)U(-0.4, 0.4);
    s.mA = (float)U(0.5, 2.0);
    s.mB = (float)U(0.5, 2.0);
    s.iA = (float)U(0.5, 4.0);
    s.iB = (float)U(0.5, 4.0);
    s.rA = mtype == ADJ_CIRCLES ? (float)U(0.2, 0.5) : 0.01f;
    s.rB = mtype == ADJ_CIRCLES ? (float)U(0.2, 0.5) : 0.01f;
    s.friction = (float)U(0.2, 0.8);
    s.restitution = (float)U(0.0, 0.5);
    s.threshold = 1.0f;
    return s;
}

static double check(const char* name, int n_in, const std::function<Vec(const Vec&)>& f,
                    const std::function<Vec(const Vec&, const Vec&)>& bwd, const Vec& x0) {
    Vec y0 = f(x0);
    Vec r(y0.size());
    for (double& v : r) v = U(-1, 1);
    Vec g = bwd(x0, r);
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n_in; ++i) {
        const double h = 1e-6 * std::max(1.0, std::fabs(x0[i]));
        Vec xp = x0, xm = x0;
        xp[i] += h;
        xm[i] -= h;
        Vec yp = f(xp), ym = f(xm);
        double lp = 0, lm = 0;
        for (size_t k = 0; k < r.size(); ++k) {
            lp += r[k] * yp[k];
            lm += r[k] * ym[k];
        }
        const double fd = (lp - lm) / (2 * h);
        num += (fd - g[i]) * (fd - g[i]);
        den += fd * fd;
    }
    const double rel = std::sqrt(num / std::max(den, 1e-30));
    std::printf("%-34s rel err %.3e\n", name, rel);
    return rel;
}

/* x layout for a pair of bodies: cA(2) aA vA(2) wA cB(2) aB vB(2) wB */
struct Pair {
    P2<T> cA, vA, cB, vB;
    T aA, wA, aB, wB;
};
static Pair unpack_pair(const Vec& x, int o) {
    Pair p;
    p.cA = p2(x[o + 0], x[o + 1]);
    p.aA = x[o + 2];
    p.vA = p2(x[o + 3], x[o + 4]);
    p.wA = x[o + 5];
    p.cB = p2(x[o + 6], x[o + 7]);
    p.aB = x[o + 8];
    p.vB = p2(x[o + 9], x[o + 10]);
    p.wB = x[o + 11];
    return p;
}

/* a state where the manifold is geometrically plausible: B sits near A's reference face */
static Vec random_pair_state(const SlotStatic& s) {
    Vec x(12);
    x[0] = U(-1, 1);
    x[1] = U(-1, 1);
    x[2] = U(-3, 3);
    x[3] = U(-2, 2);
    x[4] = U(-2, 2);
    x[5] = U(-2, 2);
    x[6] = x[0] + U(-0.5, 0.5);
    x[7] = x[1] + U(-0.5, 0.5);
    x[8] = U(-3, 3);
    x[9] = U(-2, 2);
    x[10] = U(-2, 2);
    x[11] = U(-2, 2);
    (void)s;
    return x;
}

static void pack_vc(const VC<T>& vc, Vec& y) {
    y.push_back(vc.n.x);
    y.push_back(vc.n.y);
    for (int j = 0; j < 2; ++j) {
        y.push_back(vc.ra[j].x);
        y.push_back(vc.ra[j].y);
        y.push_back(vc.rb[j].x);
        y.push_back(vc.rb[j].y);
        y.push_back(vc.nm[j]);
        y.push_back(vc.tm[j]);
        y.push_back(vc.bias[j]);
    }
    y.push_back(vc.k11);
    y.push_back(vc.k12);
    y.push_back(vc.k22);
    y.push_back(vc.na);
    y.push_back(vc.nbc);
    y.push_back(vc.nd);
}
static VCGrad<T> unpack_vcgrad(const Vec& r, int o) {
    VCGrad<T> g;
    g.n = p2(r[o], r[o + 1]);
    o += 2;
    for (int j = 0; j < 2; ++j) {
        g.ra[j] = p2(r[o], r[o + 1]);
        g.rb[j] = p2(r[o + 2], r[o + 3]);
        g.nm[j] = r[o + 4];
        g.tm[j] = r[o + 5];
        g.bias[j] = r[o + 6];
        o += 7;
    }
    g.k11 = r[o];
    g.k12 = r[o + 1];
    g.k22 = r[o + 2];
    g.na = r[o + 3];
    g.nbc = r[o + 4];
    g.nd = r[o + 5];
    return g;
}
/* VC as an input vector (the fields the velocity solver reads) */
static VC<T> unpack_vc(const Vec& x, int o, int vcount) {
    VC<T> vc;
    vc.n = p2(x[o], x[o + 1]);
    o += 2;
    for (int j = 0; j < 2; ++j) {
        vc.ra[j] = p2(x[o], x[o + 1]);
        vc.rb[j] = p2(x[o + 2], x[o + 3]);
        vc.nm[j] = x[o + 4];
        vc.tm[j] = x[o + 5];
        vc.bias[j] = x[o + 6];
        vc.bias_on[j] = 1;
        o += 7;
    }
    vc.k11 = x[o];
    vc.k12 = x[o + 1];
    vc.k22 = x[o + 2];
    vc.na = x[o + 3];
    vc.nbc = x[o + 4];
    vc.nd = x[o + 5];
    vc.vcount = vcount;
    return vc;
}
static void grad_vc_into(const VCGrad<T>& g, Vec& out, int o) {
    out[o] = g.n.x;
    out[o + 1] = g.n.y;
    o += 2;
    for (int j = 0; j < 2; ++j) {
        out[o] = g.ra[j].x;
        out[o + 1] = g.ra[j].y;
        out[o + 2] = g.rb[j].x;
        out[o + 3] = g.rb[j].y;
        out[o + 4] = g.nm[j];
        out[o + 5] = g.tm[j];
        out[o + 6] = g.bias[j];
        o += 7;
    }
    out[o] = g.k11;
    out[o + 1] = g.k12;
    out[o + 2] = g.k22;
    out[o + 3] = g.na;
    out[o + 4] = g.nbc;
    out[o + 5] = g.nd;
}
static const int kVCN = 2 + 14 + 6;

int main() {
    const double tol = 1e-5;
    int fails = 0;
    auto rep = [&](double e) {
        if (!(e < tol)) ++fails;
    };
    const P2<T> lcA = p2(0.05, -0.02), lcB = p2(-0.03, 0.04);
    const int types[3] = {ADJ_CIRCLES, ADJ_FACE_A, ADJ_FACE_B};
    for (int trial = 0; trial < 6; ++trial) {
        for (int ti = 0; ti < 3; ++ti) {
            for (int count = 1; count <= 2; ++count) {
                if (types[ti] == ADJ_CIRCLES && count == 2) continue;
                const SlotStatic s = random_slot(types[ti], count);
                char name[64];
                /* ---- init_slot: (poses, velocities) -> VC ---- */
                {
                    Vec x0 = random_pair_state(s);
                    auto f = [&](const Vec& x) {
                        Pair p = unpack_pair(x, 0);
                        VC<T> vc;
                        init_slot(s, p.cA, p.aA, p.cB, p.aB, p.vA, p.wA, p.vB, p.wB, lcA, lcB, vc);
                        Vec y;
                        pack_vc(vc, y);
                        return y;
                    };
                    auto b = [&](const Vec& x, const Vec& r) {
                        Pair p = unpack_pair(x, 0);
                        VC<T> vc;
                        init_slot(s, p.cA, p.aA, p.cB, p.aB, p.vA, p.wA, p.vB, p.wB, lcA, lcB, vc);
                        VCGrad<T> g = unpack_vcgrad(r, 0);
                        P2<T> gcA = p2(0.0, 0.0), gcB = p2(0.0, 0.0), gvA = p2(0.0, 0.0), gvB = p2(0.0, 0.0);
                        T gaA = 0, gaB = 0, gwA = 0, gwB = 0;
                        init_slot_bwd(s, p.cA, p.aA, p.cB, p.aB, p.vA, p.wA, p.vB, p.wB, lcA, lcB, vc, g, gcA, gaA,
                                      gcB, gaB, gvA, gwA, gvB, gwB);
                        return Vec{gcA.x, gcA.y, gaA, gvA.x, gvA.y, gwA, gcB.x, gcB.y, gaB, gvB.x, gvB.y, gwB};
                    };
                    std::snprintf(name, sizeof(name), "init_slot type %d count %d", types[ti], count);
                    rep(check(name, 12, f, b, x0));
                }
                /* ---- warm_slot + solve_velocity: (VC, impulses, velocities) -> (impulses, velocities) ---- */
                for (int vcount = 1; vcount <= count; ++vcount) {
                    Vec x0;
                    {
                        Pair p = unpack_pair(random_pair_state(s), 0);
                        VC<T> vc;
                        init_slot(s, p.cA, p.aA, p.cB, p.aB, p.vA, p.wA, p.vB, p.wB, lcA, lcB, vc);
                        if (vc.vcount != vcount) {
                            if (vcount == 2) continue;
                            vc.vcount = 1;
                        }
                        pack_vc(vc, x0);
                        for (int j = 0; j < 4; ++j) x0.push_back(U(0.0, 1.0));
                        x0.push_back(p.vA.x);
                        x0.push_back(p.vA.y);
                        x0.push_back(p.wA);
                        x0.push_back(p.vB.x);
                        x0.push_back(p.vB.y);
                        x0.push_back(p.wB);
                    }
                    const int n = (int)x0.size();
                    const int oi = kVCN, ov = kVCN + 4;
                    VelDecision dec0{};
                    {
                        VC<T> vc = unpack_vc(x0, 0, vcount);
                        T ni[2] = {x0[oi], x0[oi + 2]}, tiv[2] = {x0[oi + 1], x0[oi + 3]};
                        P2<T> vA = p2(x0[ov], x0[ov + 1]), vB = p2(x0[ov + 3], x0[ov + 4]);
                        T wA = x0[ov + 2], wB = x0[ov + 5];
                        solve_velocity(s, vc, ni, tiv, vA, wA, vB, wB, dec0, false);
                    }
                    auto f = [&](const Vec& x) {
                        VC<T> vc = unpack_vc(x, 0, vcount);
                        T ni[2] = {x[oi], x[oi + 2]}, tiv[2] = {x[oi + 1], x[oi + 3]};
                        P2<T> vA = p2(x[ov], x[ov + 1]), vB = p2(x[ov + 3], x[ov + 4]);
                        T wA = x[ov + 2], wB = x[ov + 5];
                        warm_slot(s, vc, ni, tiv, vA, wA, vB, wB);
                        VelDecision d = dec0;
                        solve_velocity(s, vc, ni, tiv, vA, wA, vB, wB, d, true);
                        return Vec{ni[0], tiv[0], ni[1], tiv[1], vA.x, vA.y, wA, vB.x, vB.y, wB};
                    };
                    auto b = [&](const Vec& x, const Vec& r) {
                        VC<T> vc = unpack_vc(x, 0, vcount);
                        T ni[2] = {x[oi], x[oi + 2]}, tiv[2] = {x[oi + 1], x[oi + 3]};
                        P2<T> vA = p2(x[ov], x[ov + 1]), vB = p2(x[ov + 3], x[ov + 4]);
                        T wA = x[ov + 2], wB = x[ov + 5];
                        const T ni0[2] = {ni[0], ni[1]}, ti0[2] = {tiv[0], tiv[1]};
                        warm_slot(s, vc, ni, tiv, vA, wA, vB, wB);
                        T gni[2] = {r[0], r[2]}, gti[2] = {r[1], r[3]};
                        P2<T> gvA = p2(r[4], r[5]), gvB = p2(r[7], r[8]);
                        T gwA = r[6], gwB = r[9];
                        VCGrad<T> g;
                        zero(g);
                        solve_velocity_bwd(s, vc, dec0, ni, tiv, vA, wA, vB, wB, gni, gti, gvA, gwA, gvB, gwB, g);
                        warm_slot_bwd(s, vc, ni0, ti0, gvA, gwA, gvB, gwB, gni, gti, g);
                        Vec out(n, 0.0);
                        grad_vc_into(g, out, 0);
                        out[oi] = gni[0];
                        out[oi + 1] = gti[0];
                        out[oi + 2] = gni[1];
                        out[oi + 3] = gti[1];
                        out[ov] = gvA.x;
                        out[ov + 1] = gvA.y;
                        out[ov + 2] = gwA;
                        out[ov + 3] = gvB.x;
                        out[ov + 4] = gvB.y;
                        out[ov + 5] = gwB;
                        return out;
                    };
                    std::snprintf(name, sizeof(name), "warm+solve_vel t%d c%d v%d dec%d%d/%d", types[ti], count,
                                  vcount, dec0.fr[0], dec0.fr[1], dec0.nrm);
                    rep(check(name, n, f, b, x0));
                }
                /* ---- solve_position: poses -> poses ---- */
                {
                    Vec x0 = random_pair_state(s);
                    Vec xp{x0[0], x0[1], x0[2], x0[6], x0[7], x0[8]};
                    unsigned char dec0[2] = {0, 0};
                    {
                        P2<T> cA = p2(xp[0], xp[1]), cB = p2(xp[3], xp[4]);
                        T aA = xp[2], aB = xp[5];
                        solve_position(s, lcA, lcB, cA, aA, cB, aB, dec0, false);
                    }
                    auto f = [&](const Vec& x) {
                        P2<T> cA = p2(x[0], x[1]), cB = p2(x[3], x[4]);
                        T aA = x[2], aB = x[5];
                        unsigned char d[2] = {dec0[0], dec0[1]};
                        solve_position(s, lcA, lcB, cA, aA, cB, aB, d, true);
                        return Vec{cA.x, cA.y, aA, cB.x, cB.y, aB};
                    };
                    auto b = [&](const Vec& x, const Vec& r) {
                        P2<T> cA = p2(x[0], x[1]), cB = p2(x[3], x[4]);
                        T aA = x[2], aB = x[5];
                        P2<T> gcA = p2(r[0], r[1]), gcB = p2(r[3], r[4]);
                        T gaA = r[2], gaB = r[5];
                        solve_position_bwd(s, lcA, lcB, cA, aA, cB, aB, dec0, gcA, gaA, gcB, gaB);
                        return Vec{gcA.x, gcA.y, gaA, gcB.x, gcB.y, gaB};
                    };
                    std::snprintf(name, sizeof(name), "solve_position t%d c%d dec%d%d", types[ti], count, dec0[0],
                                  dec0[1]);
                    rep(check(name, 6, f, b, xp));
                }
            }
        }
    }
    /* ---- integrate_velocity and integrate_position (with and without the clamps) ---- */
    for (int trial = 0; trial < 4; ++trial) {
        BodyStatic bs{};
        bs.m = 2.0f;
        bs.invm = 0.5f;
        bs.I = 1.0f;
        bs.invI = 1.0f;
        bs.lin_damp = (float)U(0, 0.5);
        bs.ang_damp = (float)U(0, 0.5);
        bs.gscale = 1.0f;
        bs.type = 2;
        const T h = 1.0 / 60.0;
        const double vs = trial < 2 ? 1.0 : 300.0; /* large speeds trigger both clamps */
        Vec x0{U(-1, 1), U(-1, 1), U(-1, 1), vs * U(-1, 1), vs * U(-1, 1), vs * U(-1, 1)};
        unsigned char cl0 = 0;
        {
            P2<T> c = p2(x0[0], x0[1]), v = p2(x0[3], x0[4]);
            T a = x0[2], w = x0[5];
            integrate_velocity(bs, h, (T)0, (T)-10, v, w);
            integrate_position(h, c, a, v, w, cl0, false);
        }
        auto f = [&](const Vec& x) {
            P2<T> c = p2(x[0], x[1]), v = p2(x[3], x[4]);
            T a = x[2], w = x[5];
            integrate_velocity(bs, h, (T)0, (T)-10, v, w);
            unsigned char cl = cl0;
            integrate_position(h, c, a, v, w, cl, true);
            return Vec{c.x, c.y, a, v.x, v.y, w};
        };
        auto b = [&](const Vec& x, const Vec& r) {
            P2<T> v = p2(x[3], x[4]);
            T w = x[5];
            integrate_velocity(bs, h, (T)0, (T)-10, v, w);
            P2<T> gc = p2(r[0], r[1]), gv = p2(r[3], r[4]);
            T ga = r[2], gw = r[5];
            integrate_position_bwd(h, v, w, cl0, gc, ga, gv, gw);
            integrate_velocity_bwd(bs, h, gv, gw);
            return Vec{gc.x, gc.y, ga, gv.x, gv.y, gw};
        };
        char name[64];
        std::snprintf(name, sizeof(name), "integrate vel+pos clamp %d", cl0);
        rep(check(name, 6, f, b, x0));
    }
    std::printf("%s (%d failures)\n", fails ? "FAIL" : "OK", fails);
    return fails ? 1 : 0;
}
