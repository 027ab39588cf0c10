/*
 * b2g_collide.cuh — shape records and contact manifolds for the GPU narrowphase.
 *
 * Each routine produces the manifold of the matching box2d-rs routine, with the same
 * feature ids and the same f32 operation order (so points/normals are bit-identical):
 *   collide_circles            src/private/collision/b2_collide_circle.rs:7-34
 *   collide_polygon_circle     src/private/collision/b2_collide_circle.rs:36-133
 *   collide_polygons           src/private/collision/b2_collide_polygon.rs:8-225
 *   collide_edge_circle        src/private/collision/b2_collide_edge.rs:11-123
 *   collide_edge_polygon       src/private/collision/b2_collide_edge.rs:172-475
 *   clip_segment               src/private/collision/b2_collision.rs:171-214
 *   shape_aabb                 b2_polygon_shape.rs:292-312, b2_circle_shape.rs:64-77, b2_edge_shape.rs:104-124
 * The routines read a shape through accessors (sh_v, sh_n, sh_radius, ...), from a flat 144-byte
 * ShapeRec or from a fixture's rows of the world's structure-of-arrays shape tables (ShapeRows), with
 * the same values either way. collide_polygons_group is collide_polygons spread over the 8 lanes of a
 * warp segment (lane k holds vertex k of both polygons), for warps that collide four polygon pairs
 * at a time; its results equal collide_polygons' bit for bit.
 */
#ifndef B2G_COLLIDE_CUH
#define B2G_COLLIDE_CUH

#include "b2g_math.cuh"

namespace b2g {

enum { SHAPE_CIRCLE = 0, SHAPE_EDGE = 1, SHAPE_POLYGON = 2 };
enum { MANIFOLD_CIRCLES = 0, MANIFOLD_FACE_A = 1, MANIFOLD_FACE_B = 2 };
enum { FEATURE_VERTEX = 0, FEATURE_FACE = 1 };
/* contact kinds: which routine a contact uses (A is the primary type, b2_contact_registers.rs:67-103) */
enum { KIND_CIRCLES = 0, KIND_POLYGON_CIRCLE = 1, KIND_POLYGONS = 2, KIND_EDGE_CIRCLE = 3, KIND_EDGE_POLYGON = 4 };

struct __align__(16) ShapeRec {
    V2 v[kMaxPolygonVertices];  /* polygon vertices | circle centre in v[0] | edge vertex0..3 in v[0..3] */
    V2 n[kMaxPolygonVertices];  /* polygon normals */
    V2 centroid;
    float radius;
    int32_t meta;               /* type | count << 8 | one_sided << 16 */
};
static_assert(sizeof(ShapeRec) == 144, "ShapeRec layout");

B2G_HD int shape_type(const ShapeRec& s) { return s.meta & 0xff; }
B2G_HD int shape_count(const ShapeRec& s) { return (s.meta >> 8) & 0xff; }
B2G_HD bool shape_one_sided(const ShapeRec& s) { return ((s.meta >> 16) & 1) != 0; }

/* A fixture's rows of the structure-of-arrays shape tables: kMaxPolygonVertices rows of
 * (v.x, v.y, n.x, n.y) (polygon vertex k and the normal of edge k; a circle's centre in row 0; an
 * edge's vertex0..3 in rows 0-3) and the header fields (centroid, radius, meta word). */
struct ShapeRows {
    const float4* vn;
    V2 centroid;
    float radius;
    int32_t meta;
};

B2G_HD V2 sh_v(const ShapeRec& s, int i) { return s.v[i]; }
B2G_HD V2 sh_n(const ShapeRec& s, int i) { return s.n[i]; }
B2G_HD float sh_radius(const ShapeRec& s) { return s.radius; }
B2G_HD int32_t sh_meta(const ShapeRec& s) { return s.meta; }
B2G_HD V2 sh_centroid(const ShapeRec& s) { return s.centroid; }
B2G_HD V2 sh_v(const ShapeRows& s, int i) { const float4 r = s.vn[i]; return mk(r.x, r.y); }
B2G_HD V2 sh_n(const ShapeRows& s, int i) { const float4 r = s.vn[i]; return mk(r.z, r.w); }
B2G_HD float sh_radius(const ShapeRows& s) { return s.radius; }
B2G_HD int32_t sh_meta(const ShapeRows& s) { return s.meta; }
B2G_HD V2 sh_centroid(const ShapeRows& s) { return s.centroid; }
template <class S> B2G_HD int sh_count(const S& s) { return (sh_meta(s) >> 8) & 0xff; }
template <class S> B2G_HD bool sh_one_sided(const S& s) { return ((sh_meta(s) >> 16) & 1) != 0; }

B2G_HD uint32_t feature(uint32_t ia, uint32_t ib, uint32_t ta, uint32_t tb) {
    return (ia & 0xffu) | ((ib & 0xffu) << 8) | ((ta & 0xffu) << 16) | ((tb & 0xffu) << 24);
}
B2G_HD uint32_t feature_swap(uint32_t id) {
    return feature((id >> 8) & 0xffu, id & 0xffu, (id >> 24) & 0xffu, (id >> 16) & 0xffu);
}

struct Manifold {
    V2 ln, lp;       /* local normal, local point */
    V2 p[2];         /* point local positions */
    uint32_t id[2];
    int type, count;
};

struct ClipV {
    V2 v;
    uint32_t id;
};

B2G_HD void shape_aabb(const ShapeRec& s, const Xf& xf, AABB& out) {
    int t = shape_type(s);
    if (t == SHAPE_CIRCLE) {
        V2 p = add(xf.p, mul(xf.q, s.v[0]));
        out.lo = mk(p.x - s.radius, p.y - s.radius);
        out.hi = mk(p.x + s.radius, p.y + s.radius);
    } else if (t == SHAPE_EDGE) {
        V2 a = mul(xf, s.v[1]);
        V2 b = mul(xf, s.v[2]);
        V2 r = mk(s.radius, s.radius);
        out.lo = sub(vmin(a, b), r);
        out.hi = add(vmax(a, b), r);
    } else {
        int n = shape_count(s);
        V2 lo = mul(xf, s.v[0]);
        V2 hi = lo;
        for (int i = 1; i < n; ++i) {
            V2 v = mul(xf, s.v[i]);
            lo = vmin(lo, v);
            hi = vmax(hi, v);
        }
        V2 r = mk(s.radius, s.radius);
        out.lo = sub(lo, r);
        out.hi = add(hi, r);
    }
}

B2G_HD int clip_segment(ClipV out[2], const ClipV in[2], V2 normal, float offset, int vertex_index_a) {
    int count = 0;
    float d0 = dot(normal, in[0].v) - offset;
    float d1 = dot(normal, in[1].v) - offset;
    if (d0 <= 0.0f) out[count++] = in[0];
    if (d1 <= 0.0f) out[count++] = in[1];
    if (d0 * d1 < 0.0f) {
        float interp = fdiv(d0, d0 - d1);
        out[count].v = add(in[0].v, scale(interp, sub(in[1].v, in[0].v)));
        out[count].id = feature((uint32_t)vertex_index_a, (in[0].id >> 8) & 0xffu, FEATURE_VERTEX, FEATURE_FACE);
        ++count;
    }
    return count;
}

template <class S>
B2G_HD void collide_circles(Manifold& m, const S& a, const Xf& xfA, const S& b, const Xf& xfB) {
    m.count = 0;
    V2 pA = mul(xfA, sh_v(a, 0));
    V2 pB = mul(xfB, sh_v(b, 0));
    V2 d = sub(pB, pA);
    float distSqr = dot(d, d);
    float radius = sh_radius(a) + sh_radius(b);
    if (distSqr > radius * radius) return;
    m.type = MANIFOLD_CIRCLES;
    m.lp = sh_v(a, 0);
    m.ln = mk(0.0f, 0.0f);
    m.count = 1;
    m.p[0] = sh_v(b, 0);
    m.id[0] = 0;
}

template <class S>
B2G_HD void collide_polygon_circle(Manifold& m, const S& poly, const Xf& xfA, const S& circ, const Xf& xfB) {
    m.count = 0;
    V2 c = mul(xfB, sh_v(circ, 0));
    V2 cLocal = mul_t(xfA, c);
    int normalIndex = 0;
    float separation = -kMaxFloat;
    float radius = sh_radius(poly) + sh_radius(circ);
    int n = sh_count(poly);
    for (int i = 0; i < n; ++i) {
        float s = dot(sh_n(poly, i), sub(cLocal, sh_v(poly, i)));
        if (s > radius) return;
        if (s > separation) {
            separation = s;
            normalIndex = i;
        }
    }
    int i1 = normalIndex;
    int i2 = (i1 + 1 < n) ? i1 + 1 : 0;
    V2 v1 = sh_v(poly, i1);
    V2 v2 = sh_v(poly, i2);
    m.type = MANIFOLD_FACE_A;
    m.p[0] = sh_v(circ, 0);
    m.id[0] = 0;
    if (separation < kEpsilon) {
        m.count = 1;
        m.ln = sh_n(poly, normalIndex);
        m.lp = scale(0.5f, add(v1, v2));
        return;
    }
    float u1 = dot(sub(cLocal, v1), sub(v2, v1));
    float u2 = dot(sub(cLocal, v2), sub(v1, v2));
    if (u1 <= 0.0f) {
        if (dist_sq(cLocal, v1) > radius * radius) return;
        m.count = 1;
        m.ln = sub(cLocal, v1);
        normalize(m.ln);
        m.lp = v1;
    } else if (u2 <= 0.0f) {
        if (dist_sq(cLocal, v2) > radius * radius) return;
        m.count = 1;
        m.ln = sub(cLocal, v2);
        normalize(m.ln);
        m.lp = v2;
    } else {
        V2 faceCenter = scale(0.5f, add(v1, v2));
        float s = dot(sub(cLocal, faceCenter), sh_n(poly, i1));
        if (s > radius) return;
        m.count = 1;
        m.ln = sh_n(poly, i1);
        m.lp = faceCenter;
    }
}

template <class S>
B2G_HD float find_max_separation(int& edgeIndex, const S& p1, const Xf& xf1, const S& p2, const Xf& xf2) {
    Xf xf = mul_t(xf2, xf1);
    int n1 = sh_count(p1), n2 = sh_count(p2);
    int best = 0;
    float maxSep = -kMaxFloat;
    for (int i = 0; i < n1; ++i) {
        V2 n = mul(xf.q, sh_n(p1, i));
        V2 v1 = mul(xf, sh_v(p1, i));
        float si = kMaxFloat;
        for (int j = 0; j < n2; ++j) {
            float sij = dot(n, sub(sh_v(p2, j), v1));
            if (sij < si) si = sij;
        }
        if (si > maxSep) {
            maxSep = si;
            best = i;
        }
    }
    edgeIndex = best;
    return maxSep;
}

template <class S>
B2G_HD void collide_polygons(Manifold& m, const S& A, const Xf& xfA, const S& B, const Xf& xfB) {
    m.count = 0;
    float totalRadius = sh_radius(A) + sh_radius(B);
    int edgeA = 0;
    float sepA = find_max_separation(edgeA, A, xfA, B, xfB);
    if (sepA > totalRadius) return;
    int edgeB = 0;
    float sepB = find_max_separation(edgeB, B, xfB, A, xfA);
    if (sepB > totalRadius) return;
    const float kTol = 0.1f * kLinearSlop;
    const bool flip = sepB > sepA + kTol;
    const S& poly1 = flip ? B : A;
    const S& poly2 = flip ? A : B;
    const Xf xf1 = flip ? xfB : xfA;
    const Xf xf2 = flip ? xfA : xfB;
    const int edge1 = flip ? edgeB : edgeA;
    m.type = flip ? MANIFOLD_FACE_B : MANIFOLD_FACE_A;
    /* incident edge: b2_find_incident_edge, b2_collide_polygon.rs:48-93 */
    ClipV incident[2];
    {
        V2 normal1 = mul_t(xf2.q, mul(xf1.q, sh_n(poly1, edge1)));
        int n2 = sh_count(poly2);
        int index = 0;
        float minDot = kMaxFloat;
        for (int i = 0; i < n2; ++i) {
            float d = dot(normal1, sh_n(poly2, i));
            if (d < minDot) {
                minDot = d;
                index = i;
            }
        }
        int i1 = index;
        int i2 = (i1 + 1 < n2) ? i1 + 1 : 0;
        incident[0].v = mul(xf2, sh_v(poly2, i1));
        incident[0].id = feature((uint32_t)edge1, (uint32_t)i1, FEATURE_FACE, FEATURE_VERTEX);
        incident[1].v = mul(xf2, sh_v(poly2, i2));
        incident[1].id = feature((uint32_t)edge1, (uint32_t)i2, FEATURE_FACE, FEATURE_VERTEX);
    }
    int count1 = sh_count(poly1);
    int iv1 = edge1;
    int iv2 = (edge1 + 1 < count1) ? edge1 + 1 : 0;
    V2 v11 = sh_v(poly1, iv1);
    V2 v12 = sh_v(poly1, iv2);
    V2 localTangent = sub(v12, v11);
    normalize(localTangent);
    V2 localNormal = cross_vs(localTangent, 1.0f);
    V2 planePoint = scale(0.5f, add(v11, v12));
    V2 tangent = mul(xf1.q, localTangent);
    V2 normal = cross_vs(tangent, 1.0f);
    v11 = mul(xf1, v11);
    v12 = mul(xf1, v12);
    float frontOffset = dot(normal, v11);
    float sideOffset1 = -dot(tangent, v11) + totalRadius;
    float sideOffset2 = dot(tangent, v12) + totalRadius;
    ClipV cp1[2], cp2[2];
    if (clip_segment(cp1, incident, neg(tangent), sideOffset1, iv1) < 2) return;
    if (clip_segment(cp2, cp1, tangent, sideOffset2, iv2) < 2) return;
    m.ln = localNormal;
    m.lp = planePoint;
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = dot(normal, cp2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            m.p[pc] = mul_t(xf2, cp2[i].v);
            m.id[pc] = flip ? feature_swap(cp2[i].id) : cp2[i].id;
            ++pc;
        }
    }
    m.count = pc;
}

template <class S>
B2G_HD void collide_edge_circle(Manifold& m, const S& edge, const Xf& xfA, const S& circ, const Xf& xfB) {
    m.count = 0;
    V2 Q = mul_t(xfA, mul(xfB, sh_v(circ, 0)));
    V2 A = sh_v(edge, 1), B = sh_v(edge, 2);
    V2 e = sub(B, A);
    V2 n = mk(e.y, -e.x);
    float offset = dot(n, sub(Q, A));
    bool oneSided = sh_one_sided(edge);
    if (oneSided && offset < 0.0f) return;
    float u = dot(e, sub(B, Q));
    float v = dot(e, sub(Q, A));
    float radius = sh_radius(edge) + sh_radius(circ);
    m.p[0] = sh_v(circ, 0);
    if (v <= 0.0f) {
        V2 d = sub(Q, A);
        if (dot(d, d) > radius * radius) return;
        if (oneSided) {
            V2 e1 = sub(A, sh_v(edge, 0));
            if (dot(e1, sub(A, Q)) > 0.0f) return;
        }
        m.count = 1;
        m.type = MANIFOLD_CIRCLES;
        m.ln = mk(0.0f, 0.0f);
        m.lp = A;
        m.id[0] = feature(0, 0, FEATURE_VERTEX, FEATURE_VERTEX);
        return;
    }
    if (u <= 0.0f) {
        V2 d = sub(Q, B);
        if (dot(d, d) > radius * radius) return;
        if (oneSided) {
            V2 e2 = sub(sh_v(edge, 3), B);
            if (dot(e2, sub(Q, B)) > 0.0f) return;
        }
        m.count = 1;
        m.type = MANIFOLD_CIRCLES;
        m.ln = mk(0.0f, 0.0f);
        m.lp = B;
        m.id[0] = feature(1, 0, FEATURE_VERTEX, FEATURE_VERTEX);
        return;
    }
    float den = dot(e, e);
    V2 P = scale(fdiv(1.0f, den), add(scale(u, A), scale(v, B)));
    V2 d = sub(Q, P);
    if (dot(d, d) > radius * radius) return;
    if (offset < 0.0f) n = mk(-n.x, -n.y);
    normalize(n);
    m.count = 1;
    m.type = MANIFOLD_FACE_A;
    m.ln = n;
    m.lp = A;
    m.id[0] = feature(0, 0, FEATURE_FACE, FEATURE_VERTEX);
}

template <class S>
B2G_HD void collide_edge_polygon(Manifold& m, const S& edge, const Xf& xfA, const S& poly, const Xf& xfB) {
    m.count = 0;
    Xf xf = mul_t(xfA, xfB);
    V2 centroidB = mul(xf, sh_centroid(poly));
    V2 v1 = sh_v(edge, 1);
    V2 v2 = sh_v(edge, 2);
    V2 edge1 = sub(v2, v1);
    normalize(edge1);
    V2 normal1 = mk(edge1.y, -edge1.x);
    float offset1 = dot(normal1, sub(centroidB, v1));
    bool oneSided = sh_one_sided(edge);
    if (oneSided && offset1 < 0.0f) return;
    const int nb = sh_count(poly);
    V2 tv[kMaxPolygonVertices], tn[kMaxPolygonVertices];
    for (int i = 0; i < nb; ++i) {
        tv[i] = mul(xf, sh_v(poly, i));
        tn[i] = mul(xf.q, sh_n(poly, i));
    }
    float radius = sh_radius(poly) + sh_radius(edge);
    /* b2_compute_edge_separation: axis EdgeA over {normal1, -normal1} */
    V2 eNormal = mk(0.0f, 0.0f);
    float eSep = -kMaxFloat;
    {
        V2 axes[2] = {normal1, neg(normal1)};
        for (int j = 0; j < 2; ++j) {
            float sj = kMaxFloat;
            for (int i = 0; i < nb; ++i) {
                float si = dot(axes[j], sub(tv[i], v1));
                if (si < sj) sj = si;
            }
            if (sj > eSep) {
                eSep = sj;
                eNormal = axes[j];
            }
        }
    }
    if (eSep > radius) return;
    /* b2_compute_polygon_separation: axis EdgeB over the polygon's normals */
    int pIndex = -1;
    bool pFound = false;
    V2 pNormal = mk(0.0f, 0.0f);
    float pSep = -kMaxFloat;
    for (int i = 0; i < nb; ++i) {
        V2 n = neg(tn[i]);
        float s1 = dot(n, sub(tv[i], v1));
        float s2 = dot(n, sub(tv[i], v2));
        float s = fminr(s1, s2);
        if (s > pSep) {
            pFound = true;
            pIndex = i;
            pSep = s;
            pNormal = n;
        }
    }
    if (pSep > radius) return;
    /* primary axis: 0 = edge A, 1 = polygon (EdgeB). The reference indexes out of
     * bounds (and panics) if no polygon axis was found, which needs NaN input; here
     * that case keeps the edge axis. */
    int primaryType;
    int primaryIndex;
    V2 primaryNormal;
    const float kRelativeTol = 0.98f;
    const float kAbsoluteTol = 0.001f;
    if (pFound && pSep - radius > kRelativeTol * (eSep - radius) + kAbsoluteTol) {
        primaryType = 1;
        primaryIndex = pIndex;
        primaryNormal = pNormal;
    } else {
        primaryType = 0;
        primaryIndex = 0;
        primaryNormal = eNormal;
    }
    if (oneSided) {
        V2 edge0 = sub(v1, sh_v(edge, 0));
        normalize(edge0);
        V2 normal0 = mk(edge0.y, -edge0.x);
        bool convex1 = cross(edge0, edge1) >= 0.0f;
        V2 edge2 = sub(sh_v(edge, 3), v2);
        normalize(edge2);
        V2 normal2 = mk(edge2.y, -edge2.x);
        bool convex2 = cross(edge1, edge2) >= 0.0f;
        const float sinTol = 0.1f;
        bool side1 = dot(primaryNormal, edge1) <= 0.0f;
        if (side1) {
            if (convex1) {
                if (cross(primaryNormal, normal0) > sinTol) return;
            } else {
                primaryType = 0;
                primaryIndex = 0;
                primaryNormal = eNormal;
            }
        } else {
            if (convex2) {
                if (cross(normal2, primaryNormal) > sinTol) return;
            } else {
                primaryType = 0;
                primaryIndex = 0;
                primaryNormal = eNormal;
            }
        }
    }
    ClipV clip[2];
    int ri1, ri2;
    V2 rv1, rv2, rnormal, sn1, sn2;
    if (primaryType == 0) {
        m.type = MANIFOLD_FACE_A;
        int best = 0;
        float bestValue = dot(primaryNormal, tn[0]);
        for (int i = 1; i < nb; ++i) {
            float value = dot(primaryNormal, tn[i]);
            if (value < bestValue) {
                bestValue = value;
                best = i;
            }
        }
        int i1 = best;
        int i2 = (i1 + 1 < nb) ? i1 + 1 : 0;
        clip[0].v = tv[i1];
        clip[0].id = feature(0, (uint32_t)i1, FEATURE_FACE, FEATURE_VERTEX);
        clip[1].v = tv[i2];
        clip[1].id = feature(0, (uint32_t)i2, FEATURE_FACE, FEATURE_VERTEX);
        ri1 = 0;
        ri2 = 1;
        rv1 = v1;
        rv2 = v2;
        rnormal = primaryNormal;
        sn1 = neg(edge1);
        sn2 = edge1;
    } else {
        m.type = MANIFOLD_FACE_B;
        clip[0].v = v2;
        clip[0].id = feature(1, (uint32_t)primaryIndex, FEATURE_VERTEX, FEATURE_FACE);
        clip[1].v = v1;
        clip[1].id = feature(0, (uint32_t)primaryIndex, FEATURE_VERTEX, FEATURE_FACE);
        ri1 = primaryIndex;
        ri2 = (ri1 + 1 < nb) ? ri1 + 1 : 0;
        rv1 = tv[ri1];
        rv2 = tv[ri2];
        rnormal = tn[ri1];
        sn1 = mk(rnormal.y, -rnormal.x);
        sn2 = neg(sn1);
    }
    float so1 = dot(sn1, rv1);
    float so2 = dot(sn2, rv2);
    ClipV cp1[2], cp2[2];
    if (clip_segment(cp1, clip, sn1, so1, ri1) < 2) return;
    if (clip_segment(cp2, cp1, sn2, so2, ri2) < 2) return;
    if (primaryType == 0) {
        m.ln = rnormal;
        m.lp = rv1;
    } else {
        m.ln = sh_n(poly, ri1);
        m.lp = sh_v(poly, ri1);
    }
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = dot(rnormal, sub(cp2[i].v, rv1));
        if (separation <= radius) {
            if (primaryType == 0) {
                m.p[pc] = mul_t(xf, cp2[i].v);
                m.id[pc] = cp2[i].id;
            } else {
                m.p[pc] = cp2[i].v;
                m.id[pc] = feature_swap(cp2[i].id);
            }
            ++pc;
        }
    }
    m.count = pc;
}

template <class S>
B2G_HD void evaluate(int kind, Manifold& m, const S& a, const Xf& xfA, const S& b, const Xf& xfB) {
    switch (kind) {
        case KIND_CIRCLES: collide_circles(m, a, xfA, b, xfB); break;
        case KIND_POLYGON_CIRCLE: collide_polygon_circle(m, a, xfA, b, xfB); break;
        case KIND_POLYGONS: collide_polygons(m, a, xfA, b, xfB); break;
        case KIND_EDGE_CIRCLE: collide_edge_circle(m, a, xfA, b, xfB); break;
        default: collide_edge_polygon(m, a, xfA, b, xfB); break;
    }
}

#ifdef __CUDACC__
/* ---- collide_polygons over an 8-lane segment of a warp ------------------------------------------
 * Four polygon pairs per warp: lanes 8g..8g+7 take pair g, lane k of the segment holding row k of
 * both polygons (vertex k and the normal of edge k, zeros past the count). Every lane of the warp
 * calls collide_polygons_group together (the shuffles name the whole warp); a segment without a pair
 * passes zero rows and counts. The per-edge scans of b2_find_max_separation and b2_find_incident_edge
 * run one edge per lane, each lane computing the sequential routine's expression for its edge, and
 * the lanes' results are combined so that the pick is the sequential scan's: the first index of the
 * best value among the values that scan would accept (a value > -kMaxFloat for the maximum, < kMaxFloat
 * for the minimum; NaN never). The rest of the routine runs on every lane of the segment alike. */
constexpr unsigned kFullWarp = 0xffffffffu;

__device__ __forceinline__ float seg_shfl(float x, int k) { return __shfl_sync(kFullWarp, x, k, 8); }

/* b2_find_max_separation (b2_collide_polygon.rs:8-46) with edge `lane` of poly1: p1 / p2 are this
 * lane's rows of poly1 / poly2 */
__device__ __forceinline__ float seg_max_separation(int& edgeIndex, int lane, float4 p1, int n1, const Xf& xf1,
                                                    float4 p2, int n2, const Xf& xf2) {
    const Xf xf = mul_t(xf2, xf1);
    const V2 n = mul(xf.q, mk(p1.z, p1.w));
    const V2 v1 = mul(xf, mk(p1.x, p1.y));
    float si = kMaxFloat;
#pragma unroll
    for (int j = 0; j < kMaxPolygonVertices; ++j) {
        const V2 v2 = mk(seg_shfl(p2.x, j), seg_shfl(p2.y, j));
        const float sij = dot(n, sub(v2, v1));
        if (j < n2 && sij < si) si = sij;
    }
    const bool ok = lane < n1 && si > -kMaxFloat;
    float best = ok ? si : -kMaxFloat;
    int at = ok ? lane : kMaxPolygonVertices;
#pragma unroll
    for (int off = 1; off < 8; off <<= 1) {
        const float ob = __shfl_xor_sync(kFullWarp, best, off, 8);
        const int oa = __shfl_xor_sync(kFullWarp, at, off, 8);
        if (ob > best || (ob == best && oa < at)) {
            best = ob;
            at = oa;
        }
    }
    edgeIndex = at < kMaxPolygonVertices ? at : 0;
    return best;
}

/* collide_polygons (b2_collide_polygon.rs:102-225) for the pair of this lane's segment: la / lb are
 * the lane's rows of A / B, na / nb their vertex counts, ra / rb their radii */
__device__ __forceinline__ void collide_polygons_group(Manifold& m, int lane, float4 la, int na, float ra, const Xf& xfA,
                                                       float4 lb, int nb, float rb, const Xf& xfB) {
    m.count = 0;
    const float totalRadius = ra + rb;
    int edgeA = 0, edgeB = 0;
    const float sepA = seg_max_separation(edgeA, lane, la, na, xfA, lb, nb, xfB);
    const float sepB = seg_max_separation(edgeB, lane, lb, nb, xfB, la, na, xfA);
    const bool separated = sepA > totalRadius || sepB > totalRadius;
    const float kTol = 0.1f * kLinearSlop;
    const bool flip = sepB > sepA + kTol;
    const float4 p1 = flip ? lb : la;
    const float4 p2 = flip ? la : lb;
    const int count1 = flip ? nb : na;
    const int n2 = flip ? na : nb;
    const Xf xf1 = flip ? xfB : xfA;
    const Xf xf2 = flip ? xfA : xfB;
    const int edge1 = flip ? edgeB : edgeA;
    /* b2_find_incident_edge (b2_collide_polygon.rs:48-93): the first poly2 normal of least dot */
    const V2 normal1 = mul_t(xf2.q, mul(xf1.q, mk(seg_shfl(p1.z, edge1), seg_shfl(p1.w, edge1))));
    const float d = dot(normal1, mk(p2.z, p2.w));
    const bool ok = lane < n2 && d < kMaxFloat;
    float minDot = ok ? d : kMaxFloat;
    int at = ok ? lane : kMaxPolygonVertices;
#pragma unroll
    for (int off = 1; off < 8; off <<= 1) {
        const float od = __shfl_xor_sync(kFullWarp, minDot, off, 8);
        const int oa = __shfl_xor_sync(kFullWarp, at, off, 8);
        if (od < minDot || (od == minDot && oa < at)) {
            minDot = od;
            at = oa;
        }
    }
    const int i1 = at < kMaxPolygonVertices ? at : 0;
    const int i2 = (i1 + 1 < n2) ? i1 + 1 : 0;
    const V2 w1 = mk(seg_shfl(p2.x, i1), seg_shfl(p2.y, i1));
    const V2 w2 = mk(seg_shfl(p2.x, i2), seg_shfl(p2.y, i2));
    const int iv1 = edge1;
    const int iv2 = (edge1 + 1 < count1) ? edge1 + 1 : 0;
    V2 v11 = mk(seg_shfl(p1.x, iv1), seg_shfl(p1.y, iv1));
    V2 v12 = mk(seg_shfl(p1.x, iv2), seg_shfl(p1.y, iv2));
    /* no shuffles below: the segments may part ways */
    if (separated) return;
    m.type = flip ? MANIFOLD_FACE_B : MANIFOLD_FACE_A;
    ClipV incident[2];
    incident[0].v = mul(xf2, w1);
    incident[0].id = feature((uint32_t)edge1, (uint32_t)i1, FEATURE_FACE, FEATURE_VERTEX);
    incident[1].v = mul(xf2, w2);
    incident[1].id = feature((uint32_t)edge1, (uint32_t)i2, FEATURE_FACE, FEATURE_VERTEX);
    V2 localTangent = sub(v12, v11);
    normalize(localTangent);
    V2 localNormal = cross_vs(localTangent, 1.0f);
    V2 planePoint = scale(0.5f, add(v11, v12));
    V2 tangent = mul(xf1.q, localTangent);
    V2 normal = cross_vs(tangent, 1.0f);
    v11 = mul(xf1, v11);
    v12 = mul(xf1, v12);
    float frontOffset = dot(normal, v11);
    float sideOffset1 = -dot(tangent, v11) + totalRadius;
    float sideOffset2 = dot(tangent, v12) + totalRadius;
    ClipV cp1[2], cp2[2];
    if (clip_segment(cp1, incident, neg(tangent), sideOffset1, iv1) < 2) return;
    if (clip_segment(cp2, cp1, tangent, sideOffset2, iv2) < 2) return;
    m.ln = localNormal;
    m.lp = planePoint;
    int pc = 0;
    for (int i = 0; i < 2; ++i) {
        float separation = dot(normal, cp2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            m.p[pc] = mul_t(xf2, cp2[i].v);
            m.id[pc] = flip ? feature_swap(cp2[i].id) : cp2[i].id;
            ++pc;
        }
    }
    m.count = pc;
}

/* Which pair of a batch this lane's segment takes: of the lanes in `todo` (a warp-uniform mask of
 * lanes with a polygon pair), segment g takes the g-th; returns that lane, or -1. */
__device__ __forceinline__ int seg_source(unsigned todo, int segment) {
    for (int k = 0; k < segment; ++k) todo &= todo - 1u;
    return todo ? __ffs((int)todo) - 1 : -1;
}
/* todo without its first four lanes (the ones a batch took) */
__device__ __forceinline__ unsigned seg_rest(unsigned todo) {
#pragma unroll
    for (int k = 0; k < 4; ++k) todo &= todo - 1u;
    return todo;
}
#endif

}  // namespace b2g
#endif
