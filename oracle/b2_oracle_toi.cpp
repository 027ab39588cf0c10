/*
 * b2_oracle_toi.cpp — TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of box2d-rs's time of impact: b2_time_of_impact
 * (private/collision/b2_time_of_impact.rs:191-463) with its separation function (:10-189), the
 * GJK distance b2_distance_fn (private/collision/b2_distance.rs:331-440), its simplex (:58-329)
 * and distance proxy (:8-47), and B2Sweep get_transform / normalize (src/b2_math.rs:764-787).
 * Same control flow and operand order as the reference; built with -ffp-contract=off. The GPU's
 * b2g_time_of_impact is checked against ora_time_of_impact bit for bit.
 */
#include <cmath>
#include <cstring>

#include "../include/b2g.h"
#include "b2_oracle_collide.h"

namespace ora {
namespace {

/* B2distanceProxy::set_shape, b2_distance.rs:8-41 */
struct Proxy {
    Vec2 v[kMaxPolygonVertices];
    int count = 0;
    float radius = 0.0f;
};

Proxy proxy_of(const Shape& s) {
    Proxy p;
    p.radius = s.radius;
    if (s.type == SHAPE_CIRCLE) {
        p.v[0] = s.p;
        p.count = 1;
    } else if (s.type == SHAPE_EDGE) {
        p.v[0] = s.v1;
        p.v[1] = s.v2;
        p.count = 2;
    } else {
        for (int i = 0; i < s.count; ++i) p.v[i] = s.verts[i];
        p.count = s.count;
    }
    return p;
}

/* B2distanceProxy::get_support, src/b2_distance.rs:113-125 */
int get_support(const Proxy& p, Vec2 d) {
    int best_index = 0;
    float best_value = dot(p.v[0], d);
    for (int i = 1; i < p.count; ++i) {
        float value = dot(p.v[i], d);
        if (value > best_value) {
            best_index = i;
            best_value = value;
        }
    }
    return best_index;
}

struct SimplexCache {
    float metric = 0.0f;
    int count = 0;
    int index_a[3] = {0, 0, 0};
    int index_b[3] = {0, 0, 0};
};

struct SimplexVertex {
    Vec2 w_a, w_b, w;
    float a = 0.0f;
    int index_a = 0, index_b = 0;
};

struct Simplex {
    SimplexVertex m_v[3];
    int m_count = 0;

    float get_metric() const {
        if (m_count == 2) return length(m_v[0].w - m_v[1].w);
        if (m_count == 3) return cross(m_v[1].w - m_v[0].w, m_v[2].w - m_v[0].w);
        return 0.0f;
    }

    void read_cache(const SimplexCache& cache, const Proxy& pa, const Xf& xa, const Proxy& pb, const Xf& xb) {
        m_count = cache.count;
        for (int i = 0; i < m_count; ++i) {
            SimplexVertex& v = m_v[i];
            v.index_a = cache.index_a[i];
            v.index_b = cache.index_b[i];
            v.w_a = mul(xa, pa.v[v.index_a]);
            v.w_b = mul(xb, pb.v[v.index_b]);
            v.w = v.w_b - v.w_a;
            v.a = 0.0f;
        }
        if (m_count > 1) {
            float metric1 = cache.metric;
            float metric2 = get_metric();
            if (metric2 < 0.5f * metric1 || 2.0f * metric1 < metric2 || metric2 < kEpsilon) m_count = 0;
        }
        if (m_count == 0) {
            SimplexVertex& v = m_v[0];
            v.index_a = 0;
            v.index_b = 0;
            v.w_a = mul(xa, pa.v[0]);
            v.w_b = mul(xb, pb.v[0]);
            v.w = v.w_b - v.w_a;
            v.a = 1.0f;
            m_count = 1;
        }
    }

    void write_cache(SimplexCache& cache) const {
        cache.metric = get_metric();
        cache.count = m_count;
        for (int i = 0; i < m_count; ++i) {
            cache.index_a[i] = m_v[i].index_a;
            cache.index_b[i] = m_v[i].index_b;
        }
    }

    Vec2 get_search_direction() const {
        if (m_count == 1) return -m_v[0].w;
        Vec2 e12 = m_v[1].w - m_v[0].w;
        float sgn = cross(e12, -m_v[0].w);
        if (sgn > 0.0f) return cross_sv(1.0f, e12);
        return cross_vs(e12, 1.0f);
    }

    void get_witness_points(Vec2& p_a, Vec2& p_b) const {
        if (m_count == 1) {
            p_a = m_v[0].w_a;
            p_b = m_v[0].w_b;
        } else if (m_count == 2) {
            p_a = m_v[0].a * m_v[0].w_a + m_v[1].a * m_v[1].w_a;
            p_b = m_v[0].a * m_v[0].w_b + m_v[1].a * m_v[1].w_b;
        } else {
            p_a = m_v[0].a * m_v[0].w_a + m_v[1].a * m_v[1].w_a + m_v[2].a * m_v[2].w_a;
            p_b = p_a;
        }
    }

    /* b2_simplex_solve2 */
    void solve2() {
        Vec2 w1 = m_v[0].w, w2 = m_v[1].w;
        Vec2 e12 = w2 - w1;
        float d12_2 = -dot(w1, e12);
        if (d12_2 <= 0.0f) {
            m_v[0].a = 1.0f;
            m_count = 1;
            return;
        }
        float d12_1 = dot(w2, e12);
        if (d12_1 <= 0.0f) {
            m_v[1].a = 1.0f;
            m_count = 1;
            m_v[0] = m_v[1];
            return;
        }
        float inv_d12 = 1.0f / (d12_1 + d12_2);
        m_v[0].a = d12_1 * inv_d12;
        m_v[1].a = d12_2 * inv_d12;
        m_count = 2;
    }

    /* b2_simplex_solve3 */
    void solve3() {
        Vec2 w1 = m_v[0].w, w2 = m_v[1].w, w3 = m_v[2].w;
        Vec2 e12 = w2 - w1;
        float w1e12 = dot(w1, e12), w2e12 = dot(w2, e12);
        float d12_1 = w2e12, d12_2 = -w1e12;
        Vec2 e13 = w3 - w1;
        float w1e13 = dot(w1, e13), w3e13 = dot(w3, e13);
        float d13_1 = w3e13, d13_2 = -w1e13;
        Vec2 e23 = w3 - w2;
        float w2e23 = dot(w2, e23), w3e23 = dot(w3, e23);
        float d23_1 = w3e23, d23_2 = -w2e23;
        float n123 = cross(e12, e13);
        float d123_1 = n123 * cross(w2, w3);
        float d123_2 = n123 * cross(w3, w1);
        float d123_3 = n123 * cross(w1, w2);
        if (d12_2 <= 0.0f && d13_2 <= 0.0f) {
            m_v[0].a = 1.0f;
            m_count = 1;
            return;
        }
        if (d12_1 > 0.0f && d12_2 > 0.0f && d123_3 <= 0.0f) {
            float inv_d12 = 1.0f / (d12_1 + d12_2);
            m_v[0].a = d12_1 * inv_d12;
            m_v[1].a = d12_2 * inv_d12;
            m_count = 2;
            return;
        }
        if (d13_1 > 0.0f && d13_2 > 0.0f && d123_2 <= 0.0f) {
            float inv_d13 = 1.0f / (d13_1 + d13_2);
            m_v[0].a = d13_1 * inv_d13;
            m_v[2].a = d13_2 * inv_d13;
            m_count = 2;
            m_v[1] = m_v[2];
            return;
        }
        if (d12_1 <= 0.0f && d23_2 <= 0.0f) {
            m_v[1].a = 1.0f;
            m_count = 1;
            m_v[0] = m_v[1];
            return;
        }
        if (d13_1 <= 0.0f && d23_1 <= 0.0f) {
            m_v[2].a = 1.0f;
            m_count = 1;
            m_v[0] = m_v[2];
            return;
        }
        if (d23_1 > 0.0f && d23_2 > 0.0f && d123_1 <= 0.0f) {
            float inv_d23 = 1.0f / (d23_1 + d23_2);
            m_v[1].a = d23_1 * inv_d23;
            m_v[2].a = d23_2 * inv_d23;
            m_count = 2;
            m_v[0] = m_v[2];
            return;
        }
        float inv_d123 = 1.0f / (d123_1 + d123_2 + d123_3);
        m_v[0].a = d123_1 * inv_d123;
        m_v[1].a = d123_2 * inv_d123;
        m_v[2].a = d123_3 * inv_d123;
        m_count = 3;
    }
};

/* b2_distance_fn with use_radii = false: the distance between the core shapes */
float distance(const Proxy& pa, const Xf& xa, const Proxy& pb, const Xf& xb, SimplexCache& cache) {
    Simplex simplex;
    simplex.read_cache(cache, pa, xa, pb, xb);
    const int kMaxIters = 20;
    int save_a[3], save_b[3];
    int iter = 0;
    while (iter < kMaxIters) {
        int save_count = simplex.m_count;
        for (int i = 0; i < save_count; ++i) {
            save_a[i] = simplex.m_v[i].index_a;
            save_b[i] = simplex.m_v[i].index_b;
        }
        if (simplex.m_count == 2) simplex.solve2();
        else if (simplex.m_count == 3) simplex.solve3();
        if (simplex.m_count == 3) break;
        Vec2 d = simplex.get_search_direction();
        if (length_sq(d) < kEpsilon * kEpsilon) break;
        SimplexVertex& vertex = simplex.m_v[simplex.m_count];
        vertex.index_a = get_support(pa, mul_t(xa.q, -d));
        vertex.w_a = mul(xa, pa.v[vertex.index_a]);
        vertex.index_b = get_support(pb, mul_t(xb.q, d));
        vertex.w_b = mul(xb, pb.v[vertex.index_b]);
        vertex.w = vertex.w_b - vertex.w_a;
        ++iter;
        bool duplicate = false;
        for (int i = 0; i < save_count; ++i) {
            if (vertex.index_a == save_a[i] && vertex.index_b == save_b[i]) {
                duplicate = true;
                break;
            }
        }
        if (duplicate) break;
        ++simplex.m_count;
    }
    Vec2 point_a, point_b;
    simplex.get_witness_points(point_a, point_b);
    simplex.write_cache(cache);
    return length(point_a - point_b);
}

/* b2_sweep_get_transform */
Xf get_transform(const Sweep& s, float beta) {
    Xf xf;
    xf.p = (1.0f - beta) * s.c0 + beta * s.c;
    float angle = (1.0f - beta) * s.a0 + beta * s.a;
    xf.q = rot(angle);
    xf.p -= mul(xf.q, s.local_center);
    return xf;
}

/* b2_sweep_normalize */
void normalize_sweep(Sweep& s) {
    float two_pi = 2.0f * kPi;
    float d = two_pi * std::floor(s.a0 / two_pi);
    s.a0 -= d;
    s.a -= d;
}

enum SepType { kPoints, kFaceA, kFaceB };

struct SeparationFunction {
    const Proxy* pa;
    const Proxy* pb;
    Sweep sa, sb;
    SepType type = kPoints;
    Vec2 local_point{0.0f, 0.0f};
    Vec2 axis{0.0f, 0.0f};

    void initialize(const SimplexCache& cache, const Proxy& proxy_a, const Sweep& sweep_a, const Proxy& proxy_b,
                    const Sweep& sweep_b, float t1) {
        pa = &proxy_a;
        pb = &proxy_b;
        sa = sweep_a;
        sb = sweep_b;
        Xf xf_a = get_transform(sa, t1), xf_b = get_transform(sb, t1);
        if (cache.count == 1) {
            type = kPoints;
            Vec2 point_a = mul(xf_a, pa->v[cache.index_a[0]]);
            Vec2 point_b = mul(xf_b, pb->v[cache.index_b[0]]);
            axis = point_b - point_a;
            normalize(axis);
        } else if (cache.index_a[0] == cache.index_a[1]) {
            type = kFaceB;
            Vec2 b1 = pb->v[cache.index_b[0]], b2 = pb->v[cache.index_b[1]];
            axis = cross_vs(b2 - b1, 1.0f);
            normalize(axis);
            Vec2 normal = mul(xf_b.q, axis);
            local_point = 0.5f * (b1 + b2);
            Vec2 point_b = mul(xf_b, local_point);
            Vec2 point_a = mul(xf_a, pa->v[cache.index_a[0]]);
            float s = dot(point_a - point_b, normal);
            if (s < 0.0f) axis = -axis;
        } else {
            type = kFaceA;
            Vec2 a1 = pa->v[cache.index_a[0]], a2 = pa->v[cache.index_a[1]];
            axis = cross_vs(a2 - a1, 1.0f);
            normalize(axis);
            Vec2 normal = mul(xf_a.q, axis);
            local_point = 0.5f * (a1 + a2);
            Vec2 point_a = mul(xf_a, local_point);
            Vec2 point_b = mul(xf_b, pb->v[cache.index_b[0]]);
            float s = dot(point_b - point_a, normal);
            if (s < 0.0f) axis = -axis;
        }
    }

    float find_min_separation(int& index_a, int& index_b, float t) const {
        Xf xf_a = get_transform(sa, t), xf_b = get_transform(sb, t);
        if (type == kPoints) {
            index_a = get_support(*pa, mul_t(xf_a.q, axis));
            index_b = get_support(*pb, mul_t(xf_b.q, -axis));
            Vec2 point_a = mul(xf_a, pa->v[index_a]);
            Vec2 point_b = mul(xf_b, pb->v[index_b]);
            return dot(point_b - point_a, axis);
        }
        if (type == kFaceA) {
            Vec2 normal = mul(xf_a.q, axis);
            Vec2 point_a = mul(xf_a, local_point);
            index_a = -1;
            index_b = get_support(*pb, mul_t(xf_b.q, -normal));
            Vec2 point_b = mul(xf_b, pb->v[index_b]);
            return dot(point_b - point_a, normal);
        }
        Vec2 normal = mul(xf_b.q, axis);
        Vec2 point_b = mul(xf_b, local_point);
        index_b = -1;
        index_a = get_support(*pa, mul_t(xf_a.q, -normal));
        Vec2 point_a = mul(xf_a, pa->v[index_a]);
        return dot(point_a - point_b, normal);
    }

    float evaluate(int index_a, int index_b, float t) const {
        Xf xf_a = get_transform(sa, t), xf_b = get_transform(sb, t);
        if (type == kPoints) {
            Vec2 point_a = mul(xf_a, pa->v[index_a]);
            Vec2 point_b = mul(xf_b, pb->v[index_b]);
            return dot(point_b - point_a, axis);
        }
        if (type == kFaceA) {
            Vec2 normal = mul(xf_a.q, axis);
            Vec2 point_a = mul(xf_a, local_point);
            Vec2 point_b = mul(xf_b, pb->v[index_b]);
            return dot(point_b - point_a, normal);
        }
        Vec2 normal = mul(xf_b.q, axis);
        Vec2 point_b = mul(xf_b, local_point);
        Vec2 point_a = mul(xf_a, pa->v[index_a]);
        return dot(point_a - point_b, normal);
    }
};

void time_of_impact(const Proxy& pa, Sweep sa, const Proxy& pb, Sweep sb, float t_max, int& state, float& t_out) {
    state = B2G_TOI_UNKNOWN;
    t_out = t_max;
    normalize_sweep(sa);
    normalize_sweep(sb);
    float total_radius = pa.radius + pb.radius;
    float target = bmax(kLinearSlop, total_radius - 3.0f * kLinearSlop);
    float tolerance = 0.25f * kLinearSlop;
    float t1 = 0.0f;
    const int kMaxIterations = 20;
    int iter = 0;
    SimplexCache cache;
    for (;;) {
        Xf xf_a = get_transform(sa, t1), xf_b = get_transform(sb, t1);
        float dist = distance(pa, xf_a, pb, xf_b, cache);
        if (dist <= 0.0f) {
            state = B2G_TOI_OVERLAPPED;
            t_out = 0.0f;
            break;
        }
        if (dist < target + tolerance) {
            state = B2G_TOI_TOUCHING;
            t_out = t1;
            break;
        }
        SeparationFunction fcn;
        fcn.initialize(cache, pa, sa, pb, sb, t1);
        bool done = false;
        float t2 = t_max;
        int push_back_iter = 0;
        for (;;) {
            int index_a = 0, index_b = 0;
            float s2 = fcn.find_min_separation(index_a, index_b, t2);
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
            float s1 = fcn.evaluate(index_a, index_b, t1);
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
            int root_iter_count = 0;
            float a1 = t1, a2 = t2;
            for (;;) {
                float t;
                if ((root_iter_count & 1) == 1) t = a1 + (target - s1) * (a2 - a1) / (s2 - s1);
                else t = 0.5f * (a1 + a2);
                ++root_iter_count;
                float s = fcn.evaluate(index_a, index_b, t);
                if (std::fabs(s - target) < tolerance) {
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
                if (root_iter_count == 50) break;
            }
            ++push_back_iter;
            if (push_back_iter == kMaxPolygonVertices) break;
        }
        ++iter;
        if (done) break;
        if (iter == kMaxIterations) {
            state = B2G_TOI_FAILED;
            t_out = t1;
            break;
        }
    }
}

Sweep sweep_of(const b2g_sweep& s) {
    Sweep w;
    w.local_center = Vec2{s.local_center.x, s.local_center.y};
    w.c0 = Vec2{s.c0.x, s.c0.y};
    w.c = Vec2{s.c.x, s.c.y};
    w.a0 = s.a0;
    w.a = s.a;
    w.alpha0 = s.alpha0;
    return w;
}

}  // namespace

/* the time of impact of two shapes (child 0) on their sweeps, for the world's solve_toi */
void time_of_impact_shapes(const Shape& a, const Sweep& sa, const Shape& b, const Sweep& sb, float t_max, int& state,
                           float& t) {
    const Proxy pa = proxy_of(a), pb = proxy_of(b);
    time_of_impact(pa, sa, pb, sb, t_max, state, t);
}

}  // namespace ora

extern "C" int ora_time_of_impact(const b2g_fixture_def* da, const b2g_sweep* sa, const b2g_fixture_def* db,
                                  const b2g_sweep* sb, const float* t_max, int n, b2g_toi_output* out) {
    for (int i = 0; i < n; ++i) {
        ora::Shape a, b;
        ora::shape_from_def(da[i], a);
        ora::shape_from_def(db[i], b);
        const ora::Proxy pa = ora::proxy_of(a), pb = ora::proxy_of(b);
        int state;
        float t;
        ora::time_of_impact(pa, ora::sweep_of(sa[i]), pb, ora::sweep_of(sb[i]), t_max ? t_max[i] : 1.0f, state, t);
        out[i].state = state;
        out[i].t = t;
    }
    return 0;
}
