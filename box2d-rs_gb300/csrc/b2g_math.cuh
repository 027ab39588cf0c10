/*
 * b2g_math.cuh — f32 vector algebra for the GPU step (and its host-side creation code).
 *
 * The reference (box2d-rs src/b2_math.rs) evaluates every expression as separately
 * rounded IEEE f32 operations. Device code is compiled with --fmad=false and host
 * code with -ffp-contract=off, and every helper below keeps the reference's operand
 * order (e.g. b2_mul_transform_by_vec2 is (c*x - s*y) + p.x, src/b2_math.rs:646-651),
 * so results are bit-identical to the CPU restatement.
 */
#ifndef B2G_MATH_CUH
#define B2G_MATH_CUH

#include <stdint.h>
#include "b2g_trig.h"

#if defined(__CUDACC__)
#define B2G_D __device__ __forceinline__
#else
#define B2G_D inline
#endif

namespace b2g {

constexpr float kMaxFloat = 3.402823466e+38f;
constexpr float kEpsilon = 1.192092896e-07f;
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
constexpr float kTimeToSleep = 0.5f;
constexpr float kLinearSleepTolerance = 0.01f;
constexpr float kAngularSleepTolerance = 2.0f / 180.0f * kPi;
constexpr int kMaxPolygonVertices = 8;

struct V2 {
    float x, y;
};
B2G_HD V2 mk(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
B2G_HD V2 add(V2 a, V2 b) { return mk(a.x + b.x, a.y + b.y); }
B2G_HD V2 sub(V2 a, V2 b) { return mk(a.x - b.x, a.y - b.y); }
B2G_HD V2 neg(V2 a) { return mk(-a.x, -a.y); }
B2G_HD V2 scale(float s, V2 a) { return mk(s * a.x, s * a.y); }
B2G_HD float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
B2G_HD float cross(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
B2G_HD V2 cross_vs(V2 a, float s) { return mk(s * a.y, -s * a.x); }
B2G_HD V2 cross_sv(float s, V2 a) { return mk(-s * a.y, s * a.x); }
B2G_HD float length_sq(V2 a) { return a.x * a.x + a.y * a.y; }
B2G_HD float dist_sq(V2 a, V2 b) { V2 c = sub(a, b); return dot(c, c); }
B2G_HD float fsqrt(float x) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(x);
#else
    return __builtin_sqrtf(x);
#endif
}
B2G_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
B2G_HD float length(V2 a) { return fsqrt(a.x * a.x + a.y * a.y); }
/* B2vec2::normalize: zero-length guard at f32 epsilon (src/b2_math.rs:82-93) */
B2G_HD float normalize(V2& a) {
    float len = length(a);
    if (len < kEpsilon) return 0.0f;
    float inv = fdiv(1.0f, len);
    a.x *= inv;
    a.y *= inv;
    return len;
}
B2G_HD float fminr(float a, float b) { return a < b ? a : b; }  /* b2_min: if a < b {a} else {b} */
B2G_HD float fmaxr(float a, float b) { return a > b ? a : b; }  /* b2_max: if a > b {a} else {b} */
B2G_HD float fclampr(float a, float lo, float hi) { return fmaxr(lo, fminr(a, hi)); }
B2G_HD V2 vmin(V2 a, V2 b) { return mk(fminr(a.x, b.x), fminr(a.y, b.y)); }
B2G_HD V2 vmax(V2 a, V2 b) { return mk(fmaxr(a.x, b.x), fmaxr(a.y, b.y)); }
B2G_HD float fabsr(float a) { return a < 0.0f ? -a : a; }

struct Rot {
    float s, c;
};
B2G_HD Rot rot(float angle) {
    Rot q;
    b2g_sincosf(angle, &q.s, &q.c);
    return q;
}
B2G_HD V2 mul(Rot q, V2 v) { return mk(q.c * v.x - q.s * v.y, q.s * v.x + q.c * v.y); }
B2G_HD V2 mul_t(Rot q, V2 v) { return mk(q.c * v.x + q.s * v.y, -q.s * v.x + q.c * v.y); }
B2G_HD Rot mul_t(Rot q, Rot r) { Rot o; o.s = q.c * r.s - q.s * r.c; o.c = q.c * r.c + q.s * r.s; return o; }

struct Xf {
    V2 p;
    Rot q;
};
B2G_HD V2 mul(const Xf& t, V2 v) {
    float x = (t.q.c * v.x - t.q.s * v.y) + t.p.x;
    float y = (t.q.s * v.x + t.q.c * v.y) + t.p.y;
    return mk(x, y);
}
B2G_HD V2 mul_t(const Xf& t, V2 v) {
    float px = v.x - t.p.x;
    float py = v.y - t.p.y;
    return mk(t.q.c * px + t.q.s * py, -t.q.s * px + t.q.c * py);
}
B2G_HD Xf mul_t(const Xf& a, const Xf& b) {
    Xf c;
    c.q = mul_t(a.q, b.q);
    c.p = mul_t(a.q, sub(b.p, a.p));
    return c;
}

struct AABB {
    V2 lo, hi;
};
B2G_HD V2 center(const AABB& b) { return scale(0.5f, add(b.lo, b.hi)); }
B2G_HD AABB combine(const AABB& a, const AABB& b) { AABB r; r.lo = vmin(a.lo, b.lo); r.hi = vmax(a.hi, b.hi); return r; }
B2G_HD bool contains(const AABB& outer, const AABB& inner) {
    return outer.lo.x <= inner.lo.x && outer.lo.y <= inner.lo.y && inner.hi.x <= outer.hi.x && inner.hi.y <= outer.hi.y;
}
/* b2_test_overlap (src/b2_collision.rs:355-368): closed intervals; d > 0 separates.
 * For finite IEEE values (b - a > 0) == (b > a), so comparisons are used directly. */
B2G_HD bool overlap4(float alx, float aly, float ahx, float ahy, float blx, float bly, float bhx, float bhy) {
    return !(blx > ahx || bly > ahy || alx > bhx || aly > bhy);
}

}  // namespace b2g
#endif
