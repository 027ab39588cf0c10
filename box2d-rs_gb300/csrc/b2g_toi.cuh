/*
 * b2g_toi.cuh — device routines of the time of impact, shared by the batched primitive
 * (k_toi.cu) and the continuous-physics pass of the step (k_continuous.cu).
 *
 * Reference: b2_time_of_impact (private/collision/b2_time_of_impact.rs:191-463) with its
 * separation function (:10-189), the GJK distance b2_distance_fn
 * (private/collision/b2_distance.rs:331-440) with the simplex (:58-329) and the distance proxy
 * (:8-47, src/b2_distance.rs:12-130), and the sweep (src/b2_math.rs:764-787).
 *
 * The conservative-advancement loop (at most 20 outer iterations, each with a GJK call, up to 8
 * push-back steps and up to 50 root-finder steps) is a long serial chain with little memory
 * traffic, so a pair stays in one thread's registers. Every float operation is the reference's in
 * the same order (the files are built without fused multiply-add), and the sweep's rotation uses
 * the project's sin/cos, so results equal the host restatement bit for bit.
 */
#ifndef B2G_TOI_CUH
#define B2G_TOI_CUH

#include "b2g.h"
#include "b2g_internal.h"

namespace b2g {
namespace {

/* B2distanceProxy: up to 8 vertices and a radius */
struct DistProxy {
    V2 v[kMaxPolygonVertices];
    int count;
    float radius;
};

__device__ __forceinline__ void make_proxy(const ShapeRec& s, DistProxy& p) {
    const int type = shape_type(s);
    p.radius = s.radius;
    if (type == SHAPE_CIRCLE) {
        p.count = 1;
        p.v[0] = s.v[0];
    } else if (type == SHAPE_EDGE) {
        p.count = 2;  /* vertex1, vertex2 */
        p.v[0] = s.v[1];
        p.v[1] = s.v[2];
    } else {
        p.count = shape_count(s);
        for (int i = 0; i < p.count; ++i) p.v[i] = s.v[i];
    }
}

/* get_support: the first vertex with the largest projection */
__device__ __forceinline__ int support(const DistProxy& p, V2 d) {
    int best = 0;
    float best_value = dot(p.v[0], d);
    for (int i = 1; i < p.count; ++i) {
        const float value = dot(p.v[i], d);
        if (value > best_value) {
            best = i;
            best_value = value;
        }
    }
    return best;
}

struct SimplexCache {
    float metric;
    int count;
    int ia[3], ib[3];
};

struct SimplexVertex {
    V2 wa, wb, w;
    float a;
    int ia, ib;
};

struct Simplex {
    SimplexVertex v[3];
    int count;
};

__device__ __forceinline__ float simplex_metric(const Simplex& s) {
    if (s.count == 2) return length(sub(s.v[0].w, s.v[1].w));
    if (s.count == 3) return cross(sub(s.v[1].w, s.v[0].w), sub(s.v[2].w, s.v[0].w));
    return 0.0f;
}

__device__ void read_cache(Simplex& s, const SimplexCache& c, const DistProxy& pa, const Xf& xa, const DistProxy& pb,
                           const Xf& xb) {
    s.count = c.count;
    for (int i = 0; i < s.count; ++i) {
        SimplexVertex& v = s.v[i];
        v.ia = c.ia[i];
        v.ib = c.ib[i];
        v.wa = mul(xa, pa.v[v.ia]);
        v.wb = mul(xb, pb.v[v.ib]);
        v.w = sub(v.wb, v.wa);
        v.a = 0.0f;
    }
    if (s.count > 1) {
        const float metric1 = c.metric;
        const float metric2 = simplex_metric(s);
        if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < kEpsilon) s.count = 0;
    }
    if (s.count == 0) {
        SimplexVertex& v = s.v[0];
        v.ia = 0;
        v.ib = 0;
        v.wa = mul(xa, pa.v[0]);
        v.wb = mul(xb, pb.v[0]);
        v.w = sub(v.wb, v.wa);
        v.a = 1.0f;
        s.count = 1;
    }
}

__device__ __forceinline__ void write_cache(const Simplex& s, SimplexCache& c) {
    c.metric = simplex_metric(s);
    c.count = s.count;
    for (int i = 0; i < s.count; ++i) {
        c.ia[i] = s.v[i].ia;
        c.ib[i] = s.v[i].ib;
    }
}

__device__ __forceinline__ V2 search_direction(const Simplex& s) {
    if (s.count == 1) return neg(s.v[0].w);
    const V2 e12 = sub(s.v[1].w, s.v[0].w);
    const float sgn = cross(e12, neg(s.v[0].w));
    return sgn > 0.0f ? cross_sv(1.0f, e12) : cross_vs(e12, 1.0f);
}

__device__ __forceinline__ void witness_points(const Simplex& s, V2& pa, V2& pb) {
    if (s.count == 1) {
        pa = s.v[0].wa;
        pb = s.v[0].wb;
    } else if (s.count == 2) {
        pa = add(scale(s.v[0].a, s.v[0].wa), scale(s.v[1].a, s.v[1].wa));
        pb = add(scale(s.v[0].a, s.v[0].wb), scale(s.v[1].a, s.v[1].wb));
    } else {
        pa = add(add(scale(s.v[0].a, s.v[0].wa), scale(s.v[1].a, s.v[1].wa)), scale(s.v[2].a, s.v[2].wa));
        pb = pa;
    }
}

/* b2_simplex_solve2, b2_distance.rs:240-264 */
__device__ void solve2(Simplex& s) {
    const V2 w1 = s.v[0].w, w2 = s.v[1].w;
    const V2 e12 = sub(w2, w1);
    const float d12_2 = -dot(w1, e12);
    if (d12_2 <= 0.0f) {
        s.v[0].a = 1.0f;
        s.count = 1;
        return;
    }
    const float d12_1 = dot(w2, e12);
    if (d12_1 <= 0.0f) {
        s.v[1].a = 1.0f;
        s.count = 1;
        s.v[0] = s.v[1];
        return;
    }
    const float inv_d12 = fdiv(1.0f, d12_1 + d12_2);
    s.v[0].a = d12_1 * inv_d12;
    s.v[1].a = d12_2 * inv_d12;
    s.count = 2;
}

/* b2_simplex_solve3, b2_distance.rs:266-329 */
__device__ void solve3(Simplex& s) {
    const V2 w1 = s.v[0].w, w2 = s.v[1].w, w3 = s.v[2].w;
    const V2 e12 = sub(w2, w1);
    const float w1e12 = dot(w1, e12), w2e12 = dot(w2, e12);
    const float d12_1 = w2e12, d12_2 = -w1e12;
    const V2 e13 = sub(w3, w1);
    const float w1e13 = dot(w1, e13), w3e13 = dot(w3, e13);
    const float d13_1 = w3e13, d13_2 = -w1e13;
    const V2 e23 = sub(w3, w2);
    const float w2e23 = dot(w2, e23), w3e23 = dot(w3, e23);
    const float d23_1 = w3e23, d23_2 = -w2e23;
    const float n123 = cross(e12, e13);
    const float d123_1 = n123 * cross(w2, w3);
    const float d123_2 = n123 * cross(w3, w1);
    const float d123_3 = n123 * cross(w1, w2);
    if (d12_2 <= 0.0f && d13_2 <= 0.0f) {
        s.v[0].a = 1.0f;
        s.count = 1;
        return;
    }
    if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
        const float inv = fdiv(1.0f, d12_1 + d12_2);
        s.v[0].a = d12_1 * inv;
        s.v[1].a = d12_2 * inv;
        s.count = 2;
        return;
    }
    if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
        const float inv = fdiv(1.0f, d13_1 + d13_2);
        s.v[0].a = d13_1 * inv;
        s.v[2].a = d13_2 * inv;
        s.count = 2;
        s.v[1] = s.v[2];
        return;
    }
    if (d12_1 <= 0.0f && d23_2 <= 0.0f) {
        s.v[1].a = 1.0f;
        s.count = 1;
        s.v[0] = s.v[1];
        return;
    }
    if (d13_1 <= 0.0f && d23_1 <= 0.0f) {
        s.v[2].a = 1.0f;
        s.count = 1;
        s.v[0] = s.v[2];
        return;
    }
    if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
        const float inv = fdiv(1.0f, d23_1 + d23_2);
        s.v[1].a = d23_1 * inv;
        s.v[2].a = d23_2 * inv;
        s.count = 2;
        s.v[0] = s.v[2];
        return;
    }
    const float inv = fdiv(1.0f, d123_1 + d123_2 + d123_3);
    s.v[0].a = d123_1 * inv;
    s.v[1].a = d123_2 * inv;
    s.v[2].a = d123_3 * inv;
    s.count = 3;
}

/* b2_distance_fn without radii (what the time of impact calls): returns the distance of the
 * core shapes and updates the cache */
__device__ float gjk_distance(const DistProxy& pa, const Xf& xa, const DistProxy& pb, const Xf& xb, SimplexCache& cache) {
    Simplex s;
    read_cache(s, cache, pa, xa, pb, xb);
    int save_a[3], save_b[3];
    for (int iter = 0; iter < 20; ++iter) {
        const int save_count = s.count;
        for (int i = 0; i < save_count; ++i) {
            save_a[i] = s.v[i].ia;
            save_b[i] = s.v[i].ib;
        }
        if (s.count == 2) solve2(s);
        else if (s.count == 3) solve3(s);
        if (s.count == 3) break;
        const V2 d = search_direction(s);
        if (dot(d, d) < kEpsilon * kEpsilon) break;
        SimplexVertex& v = s.v[s.count];
        v.ia = support(pa, mul_t(xa.q, neg(d)));
        v.wa = mul(xa, pa.v[v.ia]);
        v.ib = support(pb, mul_t(xb.q, d));
        v.wb = mul(xb, pb.v[v.ib]);
        v.w = sub(v.wb, v.wa);
        bool duplicate = false;
        for (int i = 0; i < save_count; ++i)
            if (v.ia == save_a[i] && v.ib == save_b[i]) {
                duplicate = true;
                break;
            }
        if (duplicate) break;
        ++s.count;
    }
    V2 wpa, wpb;
    witness_points(s, wpa, wpb);
    write_cache(s, cache);
    return length(sub(wpa, wpb));
}

struct Sweep {
    V2 lc, c0, c;
    float a0, a, alpha0;
};

/* B2Sweep::get_transform, src/b2_math.rs:764-771 */
__device__ __forceinline__ Xf sweep_xf(const Sweep& s, float beta) {
    Xf xf;
    xf.p = add(scale(1.0f - beta, s.c0), scale(beta, s.c));
    const float angle = (1.0f - beta) * s.a0 + beta * s.a;
    xf.q = rot(angle);
    xf.p = sub(xf.p, mul(xf.q, s.lc));
    return xf;
}

enum { SEP_POINTS = 0, SEP_FACE_A = 1, SEP_FACE_B = 2 };

/* B2separationFunction, b2_time_of_impact.rs:10-189 */
struct SepFn {
    int type;
    V2 local_point, axis;
};

__device__ SepFn sep_init(const SimplexCache& cache, const DistProxy& pa, const Sweep& sa, const DistProxy& pb,
                          const Sweep& sb, float t1) {
    SepFn f;
    f.local_point = mk(0.0f, 0.0f);
    const Xf xa = sweep_xf(sa, t1), xb = sweep_xf(sb, t1);
    if (cache.count == 1) {
        f.type = SEP_POINTS;
        const V2 point_a = mul(xa, pa.v[cache.ia[0]]);
        const V2 point_b = mul(xb, pb.v[cache.ib[0]]);
        f.axis = sub(point_b, point_a);
        normalize(f.axis);
    } else if (cache.ia[0] == cache.ia[1]) {
        f.type = SEP_FACE_B;
        const V2 b1 = pb.v[cache.ib[0]], b2 = pb.v[cache.ib[1]];
        f.axis = cross_vs(sub(b2, b1), 1.0f);
        normalize(f.axis);
        const V2 normal = mul(xb.q, f.axis);
        f.local_point = scale(0.5f, add(b1, b2));
        const V2 point_b = mul(xb, f.local_point);
        const V2 point_a = mul(xa, pa.v[cache.ia[0]]);
        const float s = dot(sub(point_a, point_b), normal);
        if (s < 0.0f) f.axis = neg(f.axis);
    } else {
        f.type = SEP_FACE_A;
        const V2 a1 = pa.v[cache.ia[0]], a2 = pa.v[cache.ia[1]];
        f.axis = cross_vs(sub(a2, a1), 1.0f);
        normalize(f.axis);
        const V2 normal = mul(xa.q, f.axis);
        f.local_point = scale(0.5f, add(a1, a2));
        const V2 point_a = mul(xa, f.local_point);
        const V2 point_b = mul(xb, pb.v[cache.ib[0]]);
        const float s = dot(sub(point_b, point_a), normal);
        if (s < 0.0f) f.axis = neg(f.axis);
    }
    return f;
}

__device__ float sep_find_min(const SepFn& f, const DistProxy& pa, const Sweep& sa, const DistProxy& pb, const Sweep& sb,
                              int& ia, int& ib, float t) {
    const Xf xa = sweep_xf(sa, t), xb = sweep_xf(sb, t);
    if (f.type == SEP_POINTS) {
        ia = support(pa, mul_t(xa.q, f.axis));
        ib = support(pb, mul_t(xb.q, neg(f.axis)));
        const V2 point_a = mul(xa, pa.v[ia]), point_b = mul(xb, pb.v[ib]);
        return dot(sub(point_b, point_a), f.axis);
    }
    if (f.type == SEP_FACE_A) {
        const V2 normal = mul(xa.q, f.axis);
        const V2 point_a = mul(xa, f.local_point);
        ia = -1;
        ib = support(pb, mul_t(xb.q, neg(normal)));
        const V2 point_b = mul(xb, pb.v[ib]);
        return dot(sub(point_b, point_a), normal);
    }
    const V2 normal = mul(xb.q, f.axis);
    const V2 point_b = mul(xb, f.local_point);
    ib = -1;
    ia = support(pa, mul_t(xa.q, neg(normal)));
    const V2 point_a = mul(xa, pa.v[ia]);
    return dot(sub(point_a, point_b), normal);
}

__device__ float sep_evaluate(const SepFn& f, const DistProxy& pa, const Sweep& sa, const DistProxy& pb, const Sweep& sb,
                              int ia, int ib, float t) {
    const Xf xa = sweep_xf(sa, t), xb = sweep_xf(sb, t);
    if (f.type == SEP_POINTS) {
        const V2 point_a = mul(xa, pa.v[ia]), point_b = mul(xb, pb.v[ib]);
        return dot(sub(point_b, point_a), f.axis);
    }
    if (f.type == SEP_FACE_A) {
        const V2 normal = mul(xa.q, f.axis);
        const V2 point_a = mul(xa, f.local_point);
        const V2 point_b = mul(xb, pb.v[ib]);
        return dot(sub(point_b, point_a), normal);
    }
    const V2 normal = mul(xb.q, f.axis);
    const V2 point_b = mul(xb, f.local_point);
    const V2 point_a = mul(xa, pa.v[ia]);
    return dot(sub(point_a, point_b), normal);
}

/* b2_time_of_impact, b2_time_of_impact.rs:191-463; state as B2G_TOI_* */
__device__ void time_of_impact(const DistProxy& pa, Sweep sa, const DistProxy& pb, Sweep sb, float t_max, int& state,
                               float& t_out) {
    state = B2G_TOI_UNKNOWN;
    t_out = t_max;
    /* B2Sweep::normalize, src/b2_math.rs:782-787 */
    const float two_pi = 2.0f * kPi;
    {
        const float d = two_pi * floorf(fdiv(sa.a0, two_pi));
        sa.a0 -= d;
        sa.a -= d;
    }
    {
        const float d = two_pi * floorf(fdiv(sb.a0, two_pi));
        sb.a0 -= d;
        sb.a -= d;
    }
    const float total_radius = pa.radius + pb.radius;
    const float target = fmaxr(kLinearSlop, total_radius - 3.0f * kLinearSlop);
    const float tolerance = 0.25f * kLinearSlop;
    float t1 = 0.0f;
    SimplexCache cache;
    cache.count = 0;
    cache.metric = 0.0f;
    for (int iter = 0;;) {
        const Xf xa = sweep_xf(sa, t1), xb = sweep_xf(sb, t1);
        const float distance = gjk_distance(pa, xa, pb, xb, cache);
        if (distance <= 0.0f) {
            state = B2G_TOI_OVERLAPPED;
            t_out = 0.0f;
            return;
        }
        if (distance < target + tolerance) {
            state = B2G_TOI_TOUCHING;
            t_out = t1;
            return;
        }
        const SepFn fcn = sep_init(cache, pa, sa, pb, sb, t1);
        bool done = false;
        float t2 = t_max;
        for (int push_back = 0;;) {
            int ia = 0, ib = 0;
            float s2 = sep_find_min(fcn, pa, sa, pb, sb, ia, ib, t2);
            if (s2 > target + tolerance) {
                state = B2G_TOI_SEPARATED;
                t_out = t_max;
                done = true;
                break;
            }
            if (s2 > target - tolerance) {
                t1 = t2;
                break;
            }
            float s1 = sep_evaluate(fcn, pa, sa, pb, sb, ia, ib, t1);
            if (s1 < target - tolerance) {
                state = B2G_TOI_FAILED;
                t_out = t1;
                done = true;
                break;
            }
            if (s1 <= target + tolerance) {
                state = B2G_TOI_TOUCHING;
                t_out = t1;
                done = true;
                break;
            }
            /* mixed bisection and secant steps */
            float a1 = t1, a2 = t2;
            for (int root_iter = 0;;) {
                float t;
                if (root_iter & 1) t = a1 + fdiv((target - s1) * (a2 - a1), s2 - s1);
                else t = 0.5f * (a1 + a2);
                ++root_iter;
                const float s = sep_evaluate(fcn, pa, sa, pb, sb, ia, ib, t);
                if (fabsr(s - target) < tolerance) {
                    t2 = t;
                    break;
                }
                if (s > target) {
                    a1 = t;
                    s1 = s;
                } else {
                    a2 = t;
                    s2 = s;
                }
                if (root_iter == 50) break;
            }
            ++push_back;
            if (push_back == kMaxPolygonVertices) break;
        }
        ++iter;
        if (done) return;
        if (iter == 20) {
            state = B2G_TOI_FAILED;
            t_out = t1;
            return;
        }
    }
}

}  // namespace
}  // namespace b2g
#endif
