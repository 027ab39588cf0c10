/*
 * Oracle shapes and narrowphase — TEST INFRASTRUCTURE ONLY (the checker).
 *
 * CPU restatement of the box2d-rs 0.0.4 manifold routines and shape helpers:
 *   polygon set / set_as_box / set_as_box_angle / compute_aabb / compute_mass
 *       src/private/collision/b2_polygon_shape.rs:12-50, 96-211, 292-390
 *   circle compute_aabb / compute_mass   src/private/collision/b2_circle_shape.rs:64-86
 *   edge compute_aabb                    src/private/collision/b2_edge_shape.rs:104-124
 *   b2_collide_circles / polygon_and_circle   src/private/collision/b2_collide_circle.rs:7-133
 *   b2_collide_polygons (+ find_max_separation, find_incident_edge)
 *                                        src/private/collision/b2_collide_polygon.rs:8-225
 *   b2_collide_edge_and_circle / edge_and_polygon
 *                                        src/private/collision/b2_collide_edge.rs:11-475
 *   b2_clip_segment_to_line, world manifold
 *                                        src/private/collision/b2_collision.rs:7-68, 171-214
 */
#ifndef B2_ORACLE_COLLIDE_H
#define B2_ORACLE_COLLIDE_H

#include "b2_oracle_math.h"

struct b2g_fixture_def;

namespace ora {

enum { SHAPE_CIRCLE = 0, SHAPE_EDGE = 1, SHAPE_POLYGON = 2 };
enum { MANIFOLD_CIRCLES = 0, MANIFOLD_FACE_A = 1, MANIFOLD_FACE_B = 2 };
enum { FEATURE_VERTEX = 0, FEATURE_FACE = 1 };

/* B2contactFeature packed into 32 bits: index_a | index_b<<8 | type_a<<16 | type_b<<24 */
inline uint32_t feature(uint32_t ia, uint32_t ib, uint32_t ta, uint32_t tb) {
    return (ia & 0xffu) | ((ib & 0xffu) << 8) | ((ta & 0xffu) << 16) | ((tb & 0xffu) << 24);
}
inline uint32_t feature_swap(uint32_t id) {
    uint32_t ia = id & 0xffu, ib = (id >> 8) & 0xffu, ta = (id >> 16) & 0xffu, tb = (id >> 24) & 0xffu;
    return feature(ib, ia, tb, ta);
}

struct Shape {
    int type = SHAPE_CIRCLE;
    float radius = 0.0f;
    Vec2 p{0.0f, 0.0f};                        /* circle centre */
    Vec2 v0{0, 0}, v1{0, 0}, v2{0, 0}, v3{0, 0};  /* edge */
    bool one_sided = false;
    int count = 0;                             /* polygon */
    Vec2 verts[kMaxPolygonVertices];
    Vec2 normals[kMaxPolygonVertices];
    Vec2 centroid{0, 0};
};

/* the shape of a fixture definition (b2_oracle_world.cpp) */
void shape_from_def(const ::b2g_fixture_def& d, Shape& s);

struct MassData {
    float mass;
    Vec2 center;
    float I;
};

struct ManifoldPoint {
    Vec2 local_point{0, 0};
    float normal_impulse = 0.0f;
    float tangent_impulse = 0.0f;
    uint32_t id = 0;
};

struct Manifold {
    ManifoldPoint points[kMaxManifoldPoints];
    Vec2 local_normal{0, 0};
    Vec2 local_point{0, 0};
    int type = MANIFOLD_CIRCLES;
    int point_count = 0;
};

struct WorldManifold {
    Vec2 normal{0, 0};
    Vec2 points[kMaxManifoldPoints];
    float separations[kMaxManifoldPoints];
};

struct ClipVertex {
    Vec2 v{0, 0};
    uint32_t id = 0;
};

void polygon_set_as_box(Shape& s, float hx, float hy);
void polygon_set_as_box_oriented(Shape& s, float hx, float hy, Vec2 center, float angle);
bool polygon_set_hull(Shape& s, const Vec2* pts, int count);
void compute_aabb(const Shape& s, const Xf& xf, AABB& out);
void compute_mass(const Shape& s, float density, MassData& out);

void world_manifold(WorldManifold& wm, const Manifold& m, const Xf& xfA, float rA, const Xf& xfB, float rB);

void collide_circles(Manifold& m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void collide_polygon_circle(Manifold& m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void collide_polygons(Manifold& m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void collide_edge_circle(Manifold& m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);
void collide_edge_polygon(Manifold& m, const Shape& a, const Xf& xfA, const Shape& b, const Xf& xfB);

/* b2_time_of_impact of two shapes (child 0) on their sweeps; state as B2G_TOI_* (b2_oracle_toi.cpp) */
void time_of_impact_shapes(const Shape& a, const Sweep& sa, const Shape& b, const Sweep& sb, float t_max, int& state,
                           float& t);

}  // namespace ora
#endif
