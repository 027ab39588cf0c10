/*
 * Oracle shapes and narrowphase — TEST INFRASTRUCTURE ONLY (the checker).
 * See b2_oracle_collide.h for the reference file:line of each routine.
 * Compile with -ffp-contract=off.
 */
#include "b2_oracle_collide.h"

namespace ora {

bool g_trig_libm = true;

/* set_as_box, private/collision/b2_polygon_shape.rs:12-23 */
void polygon_set_as_box(Shape& s, float hx, float hy) {
    s.type = SHAPE_POLYGON;
    s.count = 4;
    s.verts[0] = v2(-hx, -hy);
    s.verts[1] = v2(hx, -hy);
    s.verts[2] = v2(hx, hy);
    s.verts[3] = v2(-hx, hy);
    s.normals[0] = v2(0.0f, -1.0f);
    s.normals[1] = v2(1.0f, 0.0f);
    s.normals[2] = v2(0.0f, 1.0f);
    s.normals[3] = v2(-1.0f, 0.0f);
    s.centroid = v2(0.0f, 0.0f);
}

/* set_as_box_angle, :25-50 */
void polygon_set_as_box_oriented(Shape& s, float hx, float hy, Vec2 c, float angle) {
    polygon_set_as_box(s, hx, hy);
    s.centroid = c;
    Xf xf{c, rot(angle)};
    for (int i = 0; i < s.count; ++i) {
        s.verts[i] = mul(xf, s.verts[i]);
        s.normals[i] = mul(xf.q, s.normals[i]);
    }
}

/* compute_centroid, :53-77 */
static Vec2 compute_centroid(const Vec2* vs, int count) {
    Vec2 c{0.0f, 0.0f};
    float area = 0.0f;
    const Vec2 s = vs[0];
    const float inv3 = 1.0f / 3.0f;
    for (int i = 0; i < count; ++i) {
        Vec2 p1 = vs[0] - s;
        Vec2 p2 = vs[i] - s;
        Vec2 p3 = (i + 1 < count) ? vs[i + 1] - s : vs[0] - s;
        Vec2 e1 = p2 - p1;
        Vec2 e2 = p3 - p1;
        float d = cross(e1, e2);
        float tri = 0.5f * d;
        area += tri;
        c += (tri * inv3) * ((p1 + p2) + p3);
    }
    c = (1.0f / area) * c + s;
    return c;
}

/* set (gift-wrapping hull), :96-211. Returns false where the reference falls back to a unit box. */
bool polygon_set_hull(Shape& s, const Vec2* vertices, int count) {
    s.type = SHAPE_POLYGON;
    if (count < 3) {
        polygon_set_as_box(s, 1.0f, 1.0f);
        return false;
    }
    int n = bmin(count, kMaxPolygonVertices);
    Vec2 ps[kMaxPolygonVertices];
    int temp = 0;
    for (int i = 0; i < n; ++i) {
        Vec2 v = vertices[i];
        bool unique = true;
        for (int j = 0; j < temp; ++j) {
            if (dist_sq(v, ps[j]) < ((0.5f * kLinearSlop) * (0.5f * kLinearSlop))) {
                unique = false;
                break;
            }
        }
        if (unique) ps[temp++] = v;
    }
    n = temp;
    if (n < 3) {
        polygon_set_as_box(s, 1.0f, 1.0f);
        return false;
    }
    int i0 = 0;
    float x0 = ps[0].x;
    for (int i = 1; i < n; ++i) {
        float x = ps[i].x;
        if (x > x0 || (x == x0 && ps[i].y < ps[i0].y)) {
            i0 = i;
            x0 = x;
        }
    }
    int hull[kMaxPolygonVertices];
    int m = 0;
    int ih = i0;
    for (;;) {
        if (m >= kMaxPolygonVertices) {  /* reference asserts here */
            polygon_set_as_box(s, 1.0f, 1.0f);
            return false;
        }
        hull[m] = ih;
        int ie = 0;
        for (int j = 1; j < n; ++j) {
            if (ie == ih) {
                ie = j;
                continue;
            }
            Vec2 r = ps[ie] - ps[hull[m]];
            Vec2 v = ps[j] - ps[hull[m]];
            float c = cross(r, v);
            if (c < 0.0f) ie = j;
            if (c == 0.0f && length_sq(v) > length_sq(r)) ie = j;
        }
        ++m;
        ih = ie;
        if (ie == i0) break;
    }
    if (m < 3) {
        polygon_set_as_box(s, 1.0f, 1.0f);
        return false;
    }
    s.count = m;
    for (int i = 0; i < m; ++i) s.verts[i] = ps[hull[i]];
    for (int i = 0; i < m; ++i) {
        int i2 = (i + 1 < m) ? i + 1 : 0;
        Vec2 edge = s.verts[i2] - s.verts[i];
        s.normals[i] = cross_vs(edge, 1.0f);
        normalize(s.normals[i]);
    }
    s.centroid = compute_centroid(s.verts, m);
    return true;
}

void compute_aabb(const Shape& s, const Xf& xf, AABB& out) {
    if (s.type == SHAPE_CIRCLE) {
        /* b2_circle_shape.rs:64-77: p = xf.p + R*m_p */
        Vec2 p = xf.p + mul(xf.q, s.p);
        out.lo = v2(p.x - s.radius, p.y - s.radius);
        out.hi = v2(p.x + s.radius, p.y + s.radius);
    } else if (s.type == SHAPE_EDGE) {
        /* b2_edge_shape.rs:104-124 */
        Vec2 a = mul(xf, s.v1);
        Vec2 b = mul(xf, s.v2);
        Vec2 lo = vmin(a, b), hi = vmax(a, b);
        Vec2 r{s.radius, s.radius};
        out.lo = lo - r;
        out.hi = hi + r;
    } else {
        /* b2_polygon_shape.rs:292-312 */
        Vec2 lo = mul(xf, s.verts[0]);
        Vec2 hi = lo;
        for (int i = 1; i < s.count; ++i) {
            Vec2 v = mul(xf, s.verts[i]);
            lo = vmin(lo, v);
            hi = vmax(hi, v);
        }
        Vec2 r{s.radius, s.radius};
        out.lo = lo - r;
        out.hi = hi + r;
    }
}

void compute_mass(const Shape& s, float density, MassData& md) {
    if (s.type == SHAPE_CIRCLE) {
        /* b2_circle_shape.rs:79-86 */
        md.mass = density * kPi * s.radius * s.radius;
        md.center = s.p;
        md.I = md.mass * (0.5f * s.radius * s.radius + dot(s.p, s.p));
    } else if (s.type == SHAPE_EDGE) {
        md.mass = 0.0f;
        md.center = 0.5f * (s.v1 + s.v2);
        md.I = 0.0f;
    } else {
        /* b2_polygon_shape.rs:314-390 */
        Vec2 c{0.0f, 0.0f};
        float area = 0.0f, inert = 0.0f;
        const Vec2 o = s.verts[0];
        const float inv3 = 1.0f / 3.0f;
        for (int i = 0; i < s.count; ++i) {
            Vec2 e1 = s.verts[i] - o;
            Vec2 e2 = (i + 1 < s.count) ? s.verts[i + 1] - o : s.verts[0] - o;
            float d = cross(e1, e2);
            float tri = 0.5f * d;
            area += tri;
            c += (tri * inv3) * (e1 + e2);
            float intx2 = e1.x * e1.x + e2.x * e1.x + e2.x * e2.x;
            float inty2 = e1.y * e1.y + e2.y * e1.y + e2.y * e2.y;
            inert += ((0.25f * inv3) * d) * (intx2 + inty2);
        }
        md.mass = density * area;
        c *= 1.0f / area;
        md.center = c + o;
        md.I = density * inert;
        md.I += md.mass * (dot(md.center, md.center) - dot(c, c));
    }
}

/* b2_world_manifold_initialize, private/collision/b2_collision.rs:7-68 */
void world_manifold(WorldManifold& wm, const Manifold& m, const Xf& xfA, float rA, const Xf& xfB, float rB) {
    if (m.point_count == 0) return;
    if (m.type == MANIFOLD_CIRCLES) {
        wm.normal = v2(1.0f, 0.0f);
        Vec2 pa = mul(xfA, m.local_point);
        Vec2 pb = mul(xfB, m.points[0].local_point);
        if (dist_sq(pa, pb) > kEpsilon * kEpsilon) {
            wm.normal = pb - pa;
            normalize(wm.normal);
        }
        Vec2 ca = pa + rA * wm.normal;
        Vec2 cb = pb - rB * wm.normal;
        wm.points[0] = 0.5f * (ca + cb);
        wm.separations[0] = dot(cb - ca, wm.normal);
    } else if (m.type == MANIFOLD_FACE_A) {
        wm.normal = mul(xfA.q, m.local_normal);
        Vec2 plane = mul(xfA, m.local_point);
        for (int i = 0; i < m.point_count; ++i) {
            Vec2 clip = mul(xfB, m.points[i].local_point);
            Vec2 ca = clip + (rA - dot(clip - plane, wm.normal)) * wm.normal;
            Vec2 cb = clip - rB * wm.normal;
            wm.points[i] = 0.5f * (ca + cb);
            wm.separations[i] = dot(cb - ca, wm.normal);
        }
    } else {
        wm.normal = mul(xfB.q, m.local_normal);
        Vec2 plane = mul(xfB, m.local_point);
        for (int i = 0; i < m.point_count; ++i) {
            Vec2 clip = mul(xfA, m.points[i].local_point);
            Vec2 cb = clip + (rB - dot(clip - plane, wm.normal)) * wm.normal;
            Vec2 ca = clip - rA * wm.normal;
            wm.points[i] = 0.5f * (ca + cb);
            wm.separations[i] = dot(ca - cb, wm.normal);
        }
        wm.normal = -wm.normal;
    }
}

/* b2_clip_segment_to_line, private/collision/b2_collision.rs:171-214 */
static int clip_segment(ClipVertex out[2], const ClipVertex in[2], Vec2 normal, float offset, int vertex_index_a) {
    int count = 0;
    float d0 = dot(normal, in[0].v) - offset;
    float d1 = dot(normal, in[1].v) - offset;
    if (d0 <= 0.0f) out[count++] = in[0];
    if (d1 <= 0.0f) out[count++] = in[1];
    if (d0 * d1 < 0.0f) {
        float interp = d0 / (d0 - d1);
        out[count].v = in[0].v + interp * (in[1].v - in[0].v);
        out[count].id = feature((uint32_t)vertex_index_a, (in[0].id >> 8) & 0xffu, FEATURE_VERTEX, FEATURE_FACE);
        ++count;
    }
    return count;
}

/* b2_collide_circles, b2_collide_circle.rs:7-34 */
void collide_circles(Manifold& m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB) {
    m.point_count = 0;
    Vec2 pA = mul(xfA, a.p);
    Vec2 pB = mul(xfB, b.p);
    Vec2 d = pB - pA;
    float distSqr = dot(d, d);
    float radius = a.radius + b.radius;
    if (distSqr > radius * radius) return;
    m.type = MANIFOLD_CIRCLES;
    m.local_point = a.p;
    m.local_normal = v2(0.0f, 0.0f);
    m.point_count = 1;
    m.points[0].local_point = b.p;
    m.points[0].id = 0;
}

/* b2_collide_polygon_and_circle, b2_collide_circle.rs:36-133 */
void collide_polygon_circle(Manifold& m, const Shape& poly, const Xf& xfA, const Shape& circ, const Xf& xfB) {
    m.point_count = 0;
    Vec2 c = mul(xfB, circ.p);
    Vec2 cLocal = mul_t(xfA, c);
    int normalIndex = 0;
    float separation = -kMaxFloat;
    float radius = poly.radius + circ.radius;
    int n = poly.count;
    for (int i = 0; i < n; ++i) {
        float s = dot(poly.normals[i], cLocal - poly.verts[i]);
        if (s > radius) return;
        if (s > separation) {
            separation = s;
            normalIndex = i;
        }
    }
    int i1 = normalIndex;
    int i2 = (i1 + 1 < n) ? i1 + 1 : 0;
    Vec2 v1 = poly.verts[i1];
    Vec2 v2_ = poly.verts[i2];
    if (separation < kEpsilon) {
        m.point_count = 1;
        m.type = MANIFOLD_FACE_A;
        m.local_normal = poly.normals[normalIndex];
        m.local_point = 0.5f * (v1 + v2_);
        m.points[0].local_point = circ.p;
        m.points[0].id = 0;
        return;
    }
    float u1 = dot(cLocal - v1, v2_ - v1);
    float u2 = dot(cLocal - v2_, v1 - v2_);
    if (u1 <= 0.0f) {
        if (dist_sq(cLocal, v1) > radius * radius) return;
        m.point_count = 1;
        m.type = MANIFOLD_FACE_A;
        m.local_normal = cLocal - v1;
        normalize(m.local_normal);
        m.local_point = v1;
        m.points[0].local_point = circ.p;
        m.points[0].id = 0;
    } else if (u2 <= 0.0f) {
        if (dist_sq(cLocal, v2_) > radius * radius) return;
        m.point_count = 1;
        m.type = MANIFOLD_FACE_A;
        m.local_normal = cLocal - v2_;
        normalize(m.local_normal);
        m.local_point = v2_;
        m.points[0].local_point = circ.p;
        m.points[0].id = 0;
    } else {
        Vec2 faceCenter = 0.5f * (v1 + v2_);
        float s = dot(cLocal - faceCenter, poly.normals[i1]);
        if (s > radius) return;
        m.point_count = 1;
        m.type = MANIFOLD_FACE_A;
        m.local_normal = poly.normals[i1];
        m.local_point = faceCenter;
        m.points[0].local_point = circ.p;
        m.points[0].id = 0;
    }
}

/* b2_find_max_separation, b2_collide_polygon.rs:8-46 */
static float find_max_separation(int& edgeIndex, const Shape& p1, const Xf& xf1, const Shape& p2, const Xf& xf2) {
    Xf xf = mul_t(xf2, xf1);
    int best = 0;
    float maxSep = -kMaxFloat;
    for (int i = 0; i < p1.count; ++i) {
        Vec2 n = mul(xf.q, p1.normals[i]);
        Vec2 v1 = mul(xf, p1.verts[i]);
        float si = kMaxFloat;
        for (int j = 0; j < p2.count; ++j) {
            float sij = dot(n, p2.verts[j] - v1);
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

/* b2_find_incident_edge, b2_collide_polygon.rs:48-93 */
static void find_incident_edge(ClipVertex c[2], const Shape& p1, const Xf& xf1, int edge1, const Shape& p2, const Xf& xf2) {
    Vec2 normal1 = mul_t(xf2.q, mul(xf1.q, p1.normals[edge1]));
    int index = 0;
    float minDot = kMaxFloat;
    for (int i = 0; i < p2.count; ++i) {
        float d = dot(normal1, p2.normals[i]);
        if (d < minDot) {
            minDot = d;
            index = i;
        }
    }
    int i1 = index;
    int i2 = (i1 + 1 < p2.count) ? i1 + 1 : 0;
    c[0].v = mul(xf2, p2.verts[i1]);
    c[0].id = feature((uint32_t)edge1, (uint32_t)i1, FEATURE_FACE, FEATURE_VERTEX);
    c[1].v = mul(xf2, p2.verts[i2]);
    c[1].id = feature((uint32_t)edge1, (uint32_t)i2, FEATURE_FACE, FEATURE_VERTEX);
}

/* b2_collide_polygons, b2_collide_polygon.rs:102-225 */
void collide_polygons(Manifold& m, const Shape& A, const Xf& xfA, const Shape& B, const Xf& xfB) {
    m.point_count = 0;
    float totalRadius = A.radius + B.radius;
    int edgeA = 0;
    float sepA = find_max_separation(edgeA, A, xfA, B, xfB);
    if (sepA > totalRadius) return;
    int edgeB = 0;
    float sepB = find_max_separation(edgeB, B, xfB, A, xfA);
    if (sepB > totalRadius) return;
    const Shape* poly1;
    const Shape* poly2;
    Xf xf1, xf2;
    int edge1;
    bool flip;
    const float kTol = 0.1f * kLinearSlop;
    if (sepB > sepA + kTol) {
        poly1 = &B; poly2 = &A; xf1 = xfB; xf2 = xfA; edge1 = edgeB;
        m.type = MANIFOLD_FACE_B;
        flip = true;
    } else {
        poly1 = &A; poly2 = &B; xf1 = xfA; xf2 = xfB; edge1 = edgeA;
        m.type = MANIFOLD_FACE_A;
        flip = false;
    }
    ClipVertex incident[2];
    find_incident_edge(incident, *poly1, xf1, edge1, *poly2, xf2);
    int count1 = poly1->count;
    int iv1 = edge1;
    int iv2 = (edge1 + 1 < count1) ? edge1 + 1 : 0;
    Vec2 v11 = poly1->verts[iv1];
    Vec2 v12 = poly1->verts[iv2];
    Vec2 localTangent = v12 - v11;
    normalize(localTangent);
    Vec2 localNormal = cross_vs(localTangent, 1.0f);
    Vec2 planePoint = 0.5f * (v11 + v12);
    Vec2 tangent = mul(xf1.q, localTangent);
    Vec2 normal = cross_vs(tangent, 1.0f);
    v11 = mul(xf1, v11);
    v12 = mul(xf1, v12);
    float frontOffset = dot(normal, v11);
    float sideOffset1 = -dot(tangent, v11) + totalRadius;
    float sideOffset2 = dot(tangent, v12) + totalRadius;
    ClipVertex cp1[2], cp2[2];
    int np = clip_segment(cp1, incident, -tangent, sideOffset1, iv1);
    if (np < 2) return;
    np = clip_segment(cp2, cp1, tangent, sideOffset2, iv2);
    if (np < 2) return;
    m.local_normal = localNormal;
    m.local_point = planePoint;
    int pointCount = 0;
    for (int i = 0; i < kMaxManifoldPoints; ++i) {
        float separation = dot(normal, cp2[i].v) - frontOffset;
        if (separation <= totalRadius) {
            ManifoldPoint& p = m.points[pointCount];
            p.local_point = mul_t(xf2, cp2[i].v);
            p.id = flip ? feature_swap(cp2[i].id) : cp2[i].id;
            ++pointCount;
        }
    }
    m.point_count = pointCount;
}

/* b2_collide_edge_and_circle, b2_collide_edge.rs:11-123 */
void collide_edge_circle(Manifold& m, const Shape& edge, const Xf& xfA, const Shape& circ, const Xf& xfB) {
    m.point_count = 0;
    Vec2 Q = mul_t(xfA, mul(xfB, circ.p));
    Vec2 A = edge.v1, B = edge.v2;
    Vec2 e = B - A;
    Vec2 n{e.y, -e.x};
    float offset = dot(n, Q - A);
    bool oneSided = edge.one_sided;
    if (oneSided && offset < 0.0f) return;
    float u = dot(e, B - Q);
    float v = dot(e, Q - A);
    float radius = edge.radius + circ.radius;
    /* cf.index_b = 0, cf.type_b = vertex */
    if (v <= 0.0f) {
        Vec2 P = A;
        Vec2 d = Q - P;
        float dd = dot(d, d);
        if (dd > radius * radius) return;
        if (edge.one_sided) {
            Vec2 A1 = edge.v0;
            Vec2 B1 = A;
            Vec2 e1 = B1 - A1;
            float u1 = dot(e1, B1 - Q);
            if (u1 > 0.0f) return;
        }
        m.point_count = 1;
        m.type = MANIFOLD_CIRCLES;
        m.local_normal = v2(0.0f, 0.0f);
        m.local_point = P;
        m.points[0].id = feature(0, 0, FEATURE_VERTEX, FEATURE_VERTEX);
        m.points[0].local_point = circ.p;
        return;
    }
    if (u <= 0.0f) {
        Vec2 P = B;
        Vec2 d = Q - P;
        float dd = dot(d, d);
        if (dd > radius * radius) return;
        if (edge.one_sided) {
            Vec2 B2 = edge.v3;
            Vec2 A2 = B;
            Vec2 e2 = B2 - A2;
            float v2_ = dot(e2, Q - A2);
            if (v2_ > 0.0f) return;
        }
        m.point_count = 1;
        m.type = MANIFOLD_CIRCLES;
        m.local_normal = v2(0.0f, 0.0f);
        m.local_point = P;
        m.points[0].id = feature(1, 0, FEATURE_VERTEX, FEATURE_VERTEX);
        m.points[0].local_point = circ.p;
        return;
    }
    float den = dot(e, e);
    Vec2 P = (1.0f / den) * (u * A + v * B);
    Vec2 d = Q - P;
    float dd = dot(d, d);
    if (dd > radius * radius) return;
    if (offset < 0.0f) n = v2(-n.x, -n.y);
    normalize(n);
    m.point_count = 1;
    m.type = MANIFOLD_FACE_A;
    m.local_normal = n;
    m.local_point = A;
    m.points[0].id = feature(0, 0, FEATURE_FACE, FEATURE_VERTEX);
    m.points[0].local_point = circ.p;
}

namespace {
enum { AXIS_UNKNOWN = 0, AXIS_EDGE_A = 1, AXIS_EDGE_B = 2 };
struct EPAxis {
    Vec2 normal;
    int type;
    int index;
    float separation;
};
struct TempPolygon {
    Vec2 verts[kMaxPolygonVertices];
    Vec2 normals[kMaxPolygonVertices];
    int count;
};
struct ReferenceFace {
    int i1, i2;
    Vec2 v1, v2, normal, sideNormal1, sideNormal2;
    float sideOffset1, sideOffset2;
};

/* b2_compute_edge_separation, b2_collide_edge.rs:172-202 */
EPAxis edge_separation(const TempPolygon& pb, Vec2 v1, Vec2 normal1) {
    EPAxis axis{v2(0.0f, 0.0f), AXIS_EDGE_A, -1, -kMaxFloat};
    Vec2 axes[2] = {normal1, -normal1};
    for (int j = 0; j < 2; ++j) {
        float sj = kMaxFloat;
        for (int i = 0; i < pb.count; ++i) {
            float si = dot(axes[j], pb.verts[i] - v1);
            if (si < sj) sj = si;
        }
        if (sj > axis.separation) {
            axis.index = j;
            axis.separation = sj;
            axis.normal = axes[j];
        }
    }
    return axis;
}

/* b2_compute_polygon_separation, :204-228 */
EPAxis polygon_separation(const TempPolygon& pb, Vec2 v1, Vec2 v2_) {
    EPAxis axis{v2(0.0f, 0.0f), AXIS_UNKNOWN, -1, -kMaxFloat};
    for (int i = 0; i < pb.count; ++i) {
        Vec2 n = -pb.normals[i];
        float s1 = dot(n, pb.verts[i] - v1);
        float s2 = dot(n, pb.verts[i] - v2_);
        float s = bmin(s1, s2);
        if (s > axis.separation) {
            axis.type = AXIS_EDGE_B;
            axis.index = i;
            axis.separation = s;
            axis.normal = n;
        }
    }
    return axis;
}
}  // namespace

/* b2_collide_edge_and_polygon, b2_collide_edge.rs:230-475 */
void collide_edge_polygon(Manifold& m, const Shape& edge, const Xf& xfA, const Shape& poly, const Xf& xfB) {
    m.point_count = 0;
    Xf xf = mul_t(xfA, xfB);
    Vec2 centroidB = mul(xf, poly.centroid);
    Vec2 v1 = edge.v1;
    Vec2 v2_ = edge.v2;
    Vec2 edge1 = v2_ - v1;
    normalize(edge1);
    Vec2 normal1{edge1.y, -edge1.x};
    float offset1 = dot(normal1, centroidB - v1);
    bool oneSided = edge.one_sided;
    if (oneSided && offset1 < 0.0f) return;
    TempPolygon tp;
    tp.count = poly.count;
    for (int i = 0; i < poly.count; ++i) {
        tp.verts[i] = mul(xf, poly.verts[i]);
        tp.normals[i] = mul(xf.q, poly.normals[i]);
    }
    float radius = poly.radius + edge.radius;
    EPAxis edgeAxis = edge_separation(tp, v1, normal1);
    if (edgeAxis.separation > radius) return;
    EPAxis polygonAxis = polygon_separation(tp, v1, v2_);
    if (polygonAxis.separation > radius) return;
    const float kRelativeTol = 0.98f;
    const float kAbsoluteTol = 0.001f;
    EPAxis primary;
    if (polygonAxis.separation - radius > kRelativeTol * (edgeAxis.separation - radius) + kAbsoluteTol)
        primary = polygonAxis;
    else
        primary = edgeAxis;
    if (oneSided) {
        Vec2 edge0 = v1 - edge.v0;
        normalize(edge0);
        Vec2 normal0{edge0.y, -edge0.x};
        bool convex1 = cross(edge0, edge1) >= 0.0f;
        Vec2 edge2 = edge.v3 - v2_;
        normalize(edge2);
        Vec2 normal2{edge2.y, -edge2.x};
        bool convex2 = cross(edge1, edge2) >= 0.0f;
        const float sinTol = 0.1f;
        bool side1 = dot(primary.normal, edge1) <= 0.0f;
        if (side1) {
            if (convex1) {
                if (cross(primary.normal, normal0) > sinTol) return;
            } else {
                primary = edgeAxis;
            }
        } else {
            if (convex2) {
                if (cross(normal2, primary.normal) > sinTol) return;
            } else {
                primary = edgeAxis;
            }
        }
    }
    ClipVertex clip[2];
    ReferenceFace rf;
    if (primary.type == AXIS_EDGE_A) {
        m.type = MANIFOLD_FACE_A;
        int best = 0;
        float bestValue = dot(primary.normal, tp.normals[0]);
        for (int i = 1; i < tp.count; ++i) {
            float value = dot(primary.normal, tp.normals[i]);
            if (value < bestValue) {
                bestValue = value;
                best = i;
            }
        }
        int i1 = best;
        int i2 = (i1 + 1 < tp.count) ? i1 + 1 : 0;
        clip[0].v = tp.verts[i1];
        clip[0].id = feature(0, (uint32_t)i1, FEATURE_FACE, FEATURE_VERTEX);
        clip[1].v = tp.verts[i2];
        clip[1].id = feature(0, (uint32_t)i2, FEATURE_FACE, FEATURE_VERTEX);
        rf.i1 = 0;
        rf.i2 = 1;
        rf.v1 = v1;
        rf.v2 = v2_;
        rf.normal = primary.normal;
        rf.sideNormal1 = -edge1;
        rf.sideNormal2 = edge1;
    } else {
        m.type = MANIFOLD_FACE_B;
        clip[0].v = v2_;
        clip[0].id = feature(1, (uint32_t)primary.index, FEATURE_VERTEX, FEATURE_FACE);
        clip[1].v = v1;
        clip[1].id = feature(0, (uint32_t)primary.index, FEATURE_VERTEX, FEATURE_FACE);
        rf.i1 = primary.index;
        rf.i2 = (rf.i1 + 1 < tp.count) ? rf.i1 + 1 : 0;
        rf.v1 = tp.verts[rf.i1];
        rf.v2 = tp.verts[rf.i2];
        rf.normal = tp.normals[rf.i1];
        rf.sideNormal1 = v2(rf.normal.y, -rf.normal.x);
        rf.sideNormal2 = -rf.sideNormal1;
    }
    rf.sideOffset1 = dot(rf.sideNormal1, rf.v1);
    rf.sideOffset2 = dot(rf.sideNormal2, rf.v2);
    ClipVertex cp1[2], cp2[2];
    int np = clip_segment(cp1, clip, rf.sideNormal1, rf.sideOffset1, rf.i1);
    if (np < kMaxManifoldPoints) return;
    np = clip_segment(cp2, cp1, rf.sideNormal2, rf.sideOffset2, rf.i2);
    if (np < kMaxManifoldPoints) return;
    if (primary.type == AXIS_EDGE_A) {
        m.local_normal = rf.normal;
        m.local_point = rf.v1;
    } else {
        m.local_normal = poly.normals[rf.i1];
        m.local_point = poly.verts[rf.i1];
    }
    int pointCount = 0;
    for (int i = 0; i < kMaxManifoldPoints; ++i) {
        float separation = dot(rf.normal, cp2[i].v - rf.v1);
        if (separation <= radius) {
            ManifoldPoint& p = m.points[pointCount];
            if (primary.type == AXIS_EDGE_A) {
                p.local_point = mul_t(xf, cp2[i].v);
                p.id = cp2[i].id;
            } else {
                p.local_point = cp2[i].v;
                p.id = feature_swap(cp2[i].id);
            }
            ++pointCount;
        }
    }
    m.point_count = pointCount;
}

}  // namespace ora
