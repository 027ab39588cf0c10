/*
 * Oracle math — TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * CPU restatement of the f32 vector algebra of box2d-rs 0.0.4, src/b2_math.rs.
 * Every expression keeps the reference's operand order, and the file must be
 * compiled with -ffp-contract=off so no a*b+c is fused (Rust never fuses).
 */
#ifndef B2_ORACLE_MATH_H
#define B2_ORACLE_MATH_H

#include <cmath>
#include <cfloat>
#include <cstdint>
#include "../box2d-rs_gb300/csrc/b2g_trig.h"

namespace ora {

/* Constants, src/b2_common.rs and src/b2_settings.rs (evaluated in f32 as rustc does). */
constexpr float kMaxFloat = FLT_MAX;
constexpr float kEpsilon = FLT_EPSILON;
constexpr float kPi = 3.14159265358979323846f;
constexpr float kAabbExtension = 0.1f;
constexpr float kAabbMultiplier = 4.0f;
constexpr float kLinearSlop = 0.005f;
constexpr float kPolygonRadius = 2.0f * kLinearSlop;
constexpr float kMaxLinearCorrection = 0.2f;
constexpr float kMaxTranslation = 2.0f;
constexpr float kMaxTranslationSquared = kMaxTranslation * kMaxTranslation;
constexpr float kMaxRotation = 0.5f * kPi;
constexpr float kMaxRotationSquared = kMaxRotation * kMaxRotation;
constexpr float kBaumgarte = 0.2f;
constexpr float kToiBaumgarte = 0.75f;
constexpr float kAngularSlop = 2.0f / 180.0f * kPi;
constexpr float kMaxAngularCorrection = 8.0f / 180.0f * kPi;
constexpr int kMaxSubSteps = 8;
constexpr int kMaxToiContacts = 32;
constexpr float kTimeToSleep = 0.5f;
constexpr float kLinearSleepTolerance = 0.01f;
constexpr float kAngularSleepTolerance = 2.0f / 180.0f * kPi;
constexpr int kMaxPolygonVertices = 8;
constexpr int kMaxManifoldPoints = 2;

/* Which sin/cos B2Rot::set uses: the platform libm (what `f32::sin` calls on Linux)
 * or the project's correctly rounded b2g_sincosf, which the GPU uses too. */
extern bool g_trig_libm;

struct Vec2 {
    float x, y;
};
inline Vec2 v2(float x, float y) { return Vec2{x, y}; }
inline Vec2 operator+(Vec2 a, Vec2 b) { return Vec2{a.x + b.x, a.y + b.y}; }
inline Vec2 operator-(Vec2 a, Vec2 b) { return Vec2{a.x - b.x, a.y - b.y}; }
inline Vec2 operator-(Vec2 a) { return Vec2{-a.x, -a.y}; }
inline Vec2 operator*(float s, Vec2 a) { return Vec2{s * a.x, s * a.y}; }
inline Vec2& operator+=(Vec2& a, Vec2 b) { a.x += b.x; a.y += b.y; return a; }
inline Vec2& operator-=(Vec2& a, Vec2 b) { a.x -= b.x; a.y -= b.y; return a; }
inline Vec2& operator*=(Vec2& a, float s) { a.x *= s; a.y *= s; return a; }
inline float dot(Vec2 a, Vec2 b) { return a.x * b.x + a.y * b.y; }
inline float cross(Vec2 a, Vec2 b) { return a.x * b.y - a.y * b.x; }
inline Vec2 cross_vs(Vec2 a, float s) { return Vec2{s * a.y, -s * a.x}; }
inline Vec2 cross_sv(float s, Vec2 a) { return Vec2{-s * a.y, s * a.x}; }
inline float length(Vec2 a) { return std::sqrt(a.x * a.x + a.y * a.y); }
inline float length_sq(Vec2 a) { return a.x * a.x + a.y * a.y; }
inline float dist_sq(Vec2 a, Vec2 b) { Vec2 c = a - b; return dot(c, c); }
/* B2vec2::normalize, src/b2_math.rs:82-93 */
inline float normalize(Vec2& a) {
    float len = length(a);
    if (len < kEpsilon) return 0.0f;
    float inv = 1.0f / len;
    a.x *= inv;
    a.y *= inv;
    return len;
}
template <class T> inline T bmin(T a, T b) { return a < b ? a : b; }
template <class T> inline T bmax(T a, T b) { return a > b ? a : b; }
template <class T> inline T bclamp(T a, T lo, T hi) { return bmax(lo, bmin(a, hi)); }
inline Vec2 vmin(Vec2 a, Vec2 b) { return Vec2{bmin(a.x, b.x), bmin(a.y, b.y)}; }
inline Vec2 vmax(Vec2 a, Vec2 b) { return Vec2{bmax(a.x, b.x), bmax(a.y, b.y)}; }

struct Rot {
    float s, c;
};
inline Rot rot(float angle) {
    Rot q;
    if (g_trig_libm) {
        q.s = std::sin(angle);
        q.c = std::cos(angle);
    } else {
        b2g_sincosf(angle, &q.s, &q.c);
    }
    return q;
}
inline Rot rot_identity() { return Rot{0.0f, 1.0f}; }
/* b2_mul_rot_by_vec2 / b2_mul_t_rot_by_vec2, src/b2_math.rs:620-630 */
inline Vec2 mul(Rot q, Vec2 v) { return Vec2{q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y}; }
inline Vec2 mul_t(Rot q, Vec2 v) { return Vec2{q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y}; }
inline Rot mul_t(Rot q, Rot r) { return Rot{q.c * r.s - q.s * r.c, q.c * r.c + q.s * r.s}; }

struct Xf {
    Vec2 p;
    Rot q;
};
/* b2_mul_transform_by_vec2, src/b2_math.rs:646-651 */
inline Vec2 mul(const Xf& t, Vec2 v) {
    float x = (t.q.c * v.x - t.q.s * v.y) + t.p.x;
    float y = (t.q.s * v.x + t.q.c * v.y) + t.p.y;
    return Vec2{x, y};
}
/* b2_mul_t_transform_by_vec2, :653-660 */
inline Vec2 mul_t(const Xf& t, Vec2 v) {
    float px = v.x - t.p.x;
    float py = v.y - t.p.y;
    return Vec2{t.q.c * px + t.q.s * py, -t.q.s * px + t.q.c * py};
}
/* b2_mul_t_transform, :674-680 */
inline Xf mul_t(const Xf& a, const Xf& b) {
    Xf c;
    c.q = mul_t(a.q, b.q);
    c.p = mul_t(a.q, b.p - a.p);
    return c;
}

struct Mat22 {
    Vec2 ex, ey;
};
inline Vec2 mul(const Mat22& a, Vec2 v) { return Vec2{a.ex.x * v.x + a.ey.x * v.y, a.ex.y * v.x + a.ey.y * v.y}; }
/* B2Mat22::solve, src/b2_math.rs:278-293 */
inline Vec2 solve(const Mat22& m, Vec2 b) {
    float a11 = m.ex.x, a12 = m.ey.x, a21 = m.ex.y, a22 = m.ey.y;
    float det = a11 * a22 - a12 * a21;
    if (det != 0.0f) det = 1.0f / det;
    return Vec2{det * (a22 * b.x - a12 * b.y), det * (a11 * b.y - a21 * b.x)};
}
/* B2Mat22::get_inverse, src/b2_math.rs:261-276 */
inline Mat22 inverse(const Mat22& m) {
    float a = m.ex.x, b = m.ey.x, c = m.ex.y, d = m.ey.y;
    float det = a * d - b * c;
    if (det != 0.0f) det = 1.0f / det;
    Mat22 r;
    r.ex = Vec2{det * d, -det * c};
    r.ey = Vec2{-det * b, det * a};
    return r;
}

struct Sweep {
    Vec2 local_center, c0, c;
    float a0, a, alpha0;
};

struct AABB {
    Vec2 lo, hi;
};
inline Vec2 center(const AABB& b) { return 0.5f * (b.lo + b.hi); }
inline float perimeter(const AABB& b) {
    float wx = b.hi.x - b.lo.x;
    float wy = b.hi.y - b.lo.y;
    return 2.0f * (wx + wy);
}
inline AABB combine(const AABB& a, const AABB& b) { return AABB{vmin(a.lo, b.lo), vmax(a.hi, b.hi)}; }
inline bool contains(const AABB& outer, const AABB& inner) {
    bool r = true;
    r = r && outer.lo.x <= inner.lo.x;
    r = r && outer.lo.y <= inner.lo.y;
    r = r && inner.hi.x <= outer.hi.x;
    r = r && inner.hi.y <= outer.hi.y;
    return r;
}
/* b2_test_overlap, src/b2_collision.rs:355-368 */
inline bool overlap(const AABB& a, const AABB& b) {
    Vec2 d1 = b.lo - a.hi;
    Vec2 d2 = a.lo - b.hi;
    if (d1.x > 0.0f || d1.y > 0.0f) return false;
    if (d2.x > 0.0f || d2.y > 0.0f) return false;
    return true;
}

}  // namespace ora
#endif
