/*
 * b2g_trig.h — sine and cosine of an f32 angle, identical on host and device.
 *
 * The reference builds every rotation with `f32::sin` / `f32::cos`
 * (B2Rot::set, src/b2_math.rs:363-376), which on Linux is the platform libm's
 * sinf/cosf. CUDA's sinf/cosf give different last bits, so this project uses
 * one function of its own on both sides, evaluated in IEEE double and rounded
 * once to f32 (so it is correctly rounded except in astronomically rare ties):
 *
 *   1. Cody–Waite reduction: k = nearest integer to x·2/π, r = x − k·π/2 with
 *      π/2 split into three doubles; the first two carry 33 significant bits so
 *      k·P1 and k·P2 are exact for |k| < 2^20 (|x| < ~1.6e6 rad).
 *   2. Taylor series of sin and cos about 0 on |r| ≤ π/4, through r^19 and
 *      r^18, evaluated by Horner's rule (truncation error < 1e-21).
 *   3. Quadrant selection by k mod 4, then one rounding to f32.
 *
 * Every operation is a separately rounded IEEE double operation. Host code must
 * be compiled with -ffp-contract=off and device code with --fmad=false so that
 * no multiply-add is fused; then host and device results are bit-identical.
 *
 * b2g_sincosf returns exactly the same bits, faster: GB300's FP64 rate is a small fraction of
 * its FP32 rate, so for |x| <= 8192 the value is first computed in float pairs (hi + lo, about
 * 46 significant bits, with explicit fused multiply-adds for the exact products):
 *   1. the same reduction r = x - k*pi/2 with pi/2 in five float parts (the first four with at
 *      most 11 significant bits, so k*P1..k*P4 are exact for |k| < 2^13);
 *   2. r = j/32 + d with |d| <= 1/64 and a table of sin(j/32), cos(j/32) as float pairs;
 *   3. sin d and cos d - 1 by their Taylor series (through d^5 and d^6), then the angle-sum
 *      formulas.
 * The float result is the pair's high part. It is returned only when the pair lies farther than
 * an error bound (2^-42 relative, far above the actual error of either computation) from the
 * midpoint between two floats; then the true value and the double evaluation round to the same
 * float. Otherwise (about one call in 2^17), and for |x| > 8192, zero, inf and NaN, the double
 * routine runs. tests/trig_check.cpp compares the two on every float in the fast range.
 */
#ifndef B2G_TRIG_H
#define B2G_TRIG_H

#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define B2G_HD __host__ __device__ __forceinline__
#else
#define B2G_HD inline
#endif

/* π/2 = B2G_PIO2_1 + B2G_PIO2_2 + B2G_PIO2_3 (first two terms: 33 significant bits). */
#define B2G_PIO2_1 0x1.921fb54400000p+0
#define B2G_PIO2_2 0x1.0b4611a600000p-34
#define B2G_PIO2_3 0x1.3198a2e037073p-69
#define B2G_2_OVER_PI 0x1.45f306dc9c883p-1

/* 1/n! rounded to double */
#define B2G_INV_F2 0x1.0000000000000p-1
#define B2G_INV_F3 0x1.5555555555555p-3
#define B2G_INV_F4 0x1.5555555555555p-5
#define B2G_INV_F5 0x1.1111111111111p-7
#define B2G_INV_F6 0x1.6c16c16c16c17p-10
#define B2G_INV_F7 0x1.a01a01a01a01ap-13
#define B2G_INV_F8 0x1.a01a01a01a01ap-16
#define B2G_INV_F9 0x1.71de3a556c734p-19
#define B2G_INV_F10 0x1.27e4fb7789f5cp-22
#define B2G_INV_F11 0x1.ae64567f544e4p-26
#define B2G_INV_F12 0x1.1eed8eff8d898p-29
#define B2G_INV_F13 0x1.6124613a86d09p-33
#define B2G_INV_F14 0x1.93974a8c07c9dp-37
#define B2G_INV_F15 0x1.ae7f3e733b81fp-41
#define B2G_INV_F16 0x1.ae7f3e733b81fp-45
#define B2G_INV_F17 0x1.952c77030ad4ap-49
#define B2G_INV_F18 0x1.6827863b97d97p-53
#define B2G_INV_F19 0x1.2f49b46814157p-57

/* sin(x), cos(x) for f32 x evaluated in double (the definition of the results). NaN/inf inputs
 * give NaN. */
B2G_HD void b2g_sincosf_ref(float x, float* out_s, float* out_c)
{
    const double xd = (double)x;
    if (!(xd - xd == 0.0)) { /* inf or nan */
        const double nan = xd - xd;
        *out_s = (float)nan;
        *out_c = (float)nan;
        return;
    }
    /* nearest integer by the 1.5·2^52 shift (|t| < 2^51 always holds for f32 input / (π/2)) */
    const double shifter = 0x1.8p52;
    const double t = xd * B2G_2_OVER_PI;
    const double kd = (t + shifter) - shifter;
    double r = xd - kd * B2G_PIO2_1;
    r = r - kd * B2G_PIO2_2;
    r = r - kd * B2G_PIO2_3;
    const double z = r * r;
    /* sin r = r + r*z*(-1/3! + z*(1/5! - z*(...))) */
    double ps = -B2G_INV_F19;
    ps = ps * z + B2G_INV_F17;
    ps = ps * z - B2G_INV_F15;
    ps = ps * z + B2G_INV_F13;
    ps = ps * z - B2G_INV_F11;
    ps = ps * z + B2G_INV_F9;
    ps = ps * z - B2G_INV_F7;
    ps = ps * z + B2G_INV_F5;
    ps = ps * z - B2G_INV_F3;
    const double sr = r + (r * z) * ps;
    /* cos r = 1 - z/2 + z*z*(1/4! - z/6! + ... - z^7/18!) */
    double pc = -B2G_INV_F18;
    pc = pc * z + B2G_INV_F16;
    pc = pc * z - B2G_INV_F14;
    pc = pc * z + B2G_INV_F12;
    pc = pc * z - B2G_INV_F10;
    pc = pc * z + B2G_INV_F8;
    pc = pc * z - B2G_INV_F6;
    pc = pc * z + B2G_INV_F4;
    const double cr = (1.0 - z * B2G_INV_F2) + (z * z) * pc;
    /* quadrant: k mod 4 (two's complement of a small integer) */
    const long long k = (long long)kd;
    const int q = (int)(k & 3);
    double s, c;
    if (q == 0) { s = sr; c = cr; }
    else if (q == 1) { s = cr; c = -sr; }
    else if (q == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
    *out_s = (float)s;
    *out_c = (float)c;
}

/* ---- the float fast path (see the file comment) ---- */
#define B2G_SC_TABLE_VALUES                                                                              \
    0.0f, 0.0f, 0x1.0p+0f, 0.0f,                                                                         \
    0x1.ffeaaap-6f, 0x1.dddd0ep-31f, 0x1.ffc002p-1f, -0x1.555b06p-26f,                                   \
    0x1.ffaaaep-5f, 0x1.dda9dcp-30f, 0x1.ff0016p-1f, -0x1.56c166p-26f,                                   \
    0x1.7f701p-4f, 0x1.92a872p-31f, 0x1.fdc06cp-1f, -0x1.0328cap-30f,                                    \
    0x1.feaaeep-4f, 0x1.d0ddc6p-29f, 0x1.fc0156p-1f, -0x1.b05486p-26f,                                   \
    0x1.3eb312p-3f, 0x1.8bacdap-28f, 0x1.f9c34p-1f, 0x1.4f9886p-26f,                                     \
    0x1.7dc102p-3f, 0x1.f75e56p-28f, 0x1.f706bep-1f, -0x1.84c792p-31f,                                   \
    0x1.bc6f84p-3f, 0x1.db8c34p-28f, 0x1.f3cc7cp-1f, 0x1.d9e8b6p-28f,                                    \
    0x1.faaeeep-3f, -0x1.619d52p-28f, 0x1.f0154ap-1f, -0x1.0422bep-30f,                                  \
    0x1.1c37d6p-2f, 0x1.31ae1ep-28f, 0x1.ebe214p-1f, 0x1.eeddf4p-26f,                                    \
    0x1.3ad12ap-2f, -0x1.12c584p-27f, 0x1.e733eap-1f, 0x1.93d3fap-33f,                                   \
    0x1.591bcap-2f, -0x1.7429a4p-32f, 0x1.e20bf4p-1f, 0x1.359ad8p-26f,                                   \
    0x1.771026p-2f, -0x1.5137bep-27f, 0x1.dc6b7ep-1f, 0x1.732b22p-26f,                                   \
    0x1.94a6bep-2f, 0x1.3ea8d8p-27f, 0x1.d653fp-1f, 0x1.cf901p-27f,                                      \
    0x1.b1d83p-2f, 0x1.4c8586p-28f, 0x1.cfc6dp-1f, -0x1.6b5498p-27f,                                     \
    0x1.ce9d2ep-2f, 0x1.ea529p-29f, 0x1.c8c5cp-1f, -0x1.cc795ep-27f,                                     \
    0x1.eaee88p-2f, -0x1.769f42p-27f, 0x1.c1528p-1f, 0x1.96df54p-27f,                                    \
    0x1.036294p-1f, -0x1.8e59aap-27f, 0x1.b96eeep-1f, 0x1.eb1082p-26f,                                   \
    0x1.110d0cp-1f, 0x1.2da70ep-27f, 0x1.b11d04p-1f, 0x1.62a4c6p-29f,                                    \
    0x1.1e7344p-1f, -0x1.b93516p-26f, 0x1.a85ed4p-1f, 0x1.b9f016p-28f,                                   \
    0x1.2b91dep-1f, 0x1.510844p-26f, 0x1.9f368ep-1f, 0x1.b225fp-26f,                                     \
    0x1.386598p-1f, -0x1.753afap-26f, 0x1.95a67ep-1f, 0x1.963f98p-34f,                                   \
    0x1.44eb38p-1f, 0x1.cf386ap-29f, 0x1.8bb106p-1f, -0x1.688dcp-27f,                                    \
    0x1.511fap-1f, -0x1.426572p-28f, 0x1.8158a4p-1f, -0x1.cdd254p-26f,                                   \
    0x1.5cffc2p-1f, -0x1.280e1ep-26f, 0x1.769fecp-1f, 0x1.954848p-27f,                                   \
    0x1.6888a4p-1f, 0x1.c26966p-26f, 0x1.6b899p-1f, -0x1.584128p-27f,                                    \
    0x1.73b768p-1f, 0x1.bd4afp-30f, 0x1.601852p-1f, 0x1.bd58f8p-27f

/* sin(j/32) hi, lo, cos(j/32) hi, lo for j = 0..26 (hi + lo within 2^-47 relative) */
#if defined(__CUDACC__)
__device__ static const float b2g_sc_table_dev[27 * 4] = {B2G_SC_TABLE_VALUES};
#endif
static const float b2g_sc_table_host[27 * 4] = {B2G_SC_TABLE_VALUES};

B2G_HD float b2g_fmaf_(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
B2G_HD unsigned b2g_f2u_(float v) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(v);
#else
    unsigned u;
    memcpy(&u, &v, 4);
    return u;
#endif
}
B2G_HD float b2g_u2f_(unsigned u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float v;
    memcpy(&v, &u, 4);
    return v;
#endif
}
/* s + e = a + b exactly */
B2G_HD void b2g_two_sum_(float a, float b, float* s, float* e) {
    const float t = a + b;
    const float bb = t - a;
    *e = (a - (t - bb)) + (b - bb);
    *s = t;
}
/* the float the pair (vh, vl) rounds to is certainly vh, for both the pair's true value and the
 * double evaluation, when |vl| + bound stays below the half-spacing towards vl's side */
B2G_HD bool b2g_rounds_to_hi_(float vh, float vl) {
    const unsigned bits = b2g_f2u_(vh) & 0x7fffffffu;
    const unsigned ex = bits >> 23;
    if (ex < 40u) return false;                          /* |vh| < 2^-87: leave it to the double path */
    const float ulp = b2g_u2f_((ex - 23u) << 23);
    const float avh = b2g_u2f_(bits), avl = vl < 0.0f ? -vl : vl;
    const bool toward_zero = (vl < 0.0f) != (vh < 0.0f) && vl != 0.0f;
    const float half = (toward_zero && (bits & 0x7fffffu) == 0u) ? 0.25f * ulp : 0.5f * ulp;
    const float bound = 0x1.0p-42f * avh + 0x1.0p-62f;
    return avl + bound < half;
}

/* sin(x), cos(x) for f32 x: the same results as b2g_sincosf_ref. */
B2G_HD void b2g_sincosf(float x, float* out_s, float* out_c)
{
    const float ax = x < 0.0f ? -x : x;
    if (!(ax <= 8192.0f) || x == 0.0f) {
        b2g_sincosf_ref(x, out_s, out_c);
        return;
    }
#if defined(__CUDA_ARCH__)
    const float* tab = b2g_sc_table_dev;
    const float kf = rintf(x * 0x1.45f306p-1f);
#else
    const float* tab = b2g_sc_table_host;
    const float kf = rintf(x * 0x1.45f306p-1f);
#endif
    /* r = x - k*pi/2 as rh + rl; k*P1..k*P4 are exact, x - k*P1 is exact (Sterbenz) */
    float s_, e_, t_;
    const float a = x - kf * 0x1.92p+0f;
    b2g_two_sum_(a, -(kf * 0x1.fb4p-12f), &s_, &e_);
    b2g_two_sum_(s_, -(kf * 0x1.444p-24f), &s_, &t_);
    e_ = e_ + t_;
    b2g_two_sum_(s_, -(kf * 0x1.68cp-39f), &s_, &t_);
    e_ = e_ + t_;
    const float p5 = kf * 0x1.1a6264p-54f;
    const float q5 = b2g_fmaf_(kf, 0x1.1a6264p-54f, -p5);
    b2g_two_sum_(s_, -p5, &s_, &t_);
    e_ = (e_ + t_) - q5;
    float rh, rl;
    b2g_two_sum_(s_, e_, &rh, &rl);
    /* r = j/32 + d */
    const float jf = rintf(rh * 32.0f);
    float dh, dl;
    b2g_two_sum_(rh - jf * 0.03125f, rl, &dh, &dl);
    const int j = (int)jf;
    const int aj = j < 0 ? -j : j;
    float sth = tab[4 * aj], stl = tab[4 * aj + 1];
    const float cth = tab[4 * aj + 2], ctl = tab[4 * aj + 3];
    if (j < 0) {
        sth = -sth;
        stl = -stl;
    }
    /* d^2 */
    const float d2h = dh * dh;
    const float d2l = b2g_fmaf_(dh, dh, -d2h) + 2.0f * dh * dl;
    /* sin d = d + d*c, c = d^2 * (-1/6 + d^2/120 - d^4/5040) */
    const float u = d2h * (0x1.111112p-7f - d2h * 0x1.a01a02p-13f);
    float ih, il;
    b2g_two_sum_(-0x1.555556p-3f, u, &ih, &il);
    il = il + 0x1.555556p-28f;
    const float ch = d2h * ih;
    const float cl = b2g_fmaf_(d2h, ih, -ch) + (d2h * il + d2l * ih);
    const float ph = dh * ch;
    const float pl = b2g_fmaf_(dh, ch, -ph) + (dh * cl + dl * ch);
    float sdh, sdl;
    b2g_two_sum_(dh, ph, &sdh, &sdl);
    sdl = sdl + (dl + pl);
    /* cos d - 1 = -d^2/2 + d^4 * (1/24 - d^2/720) */
    const float v = (d2h * d2h) * (0x1.555556p-5f - d2h * 0x1.6c16c2p-10f);
    float mh, ml;
    b2g_two_sum_(-0.5f * d2h, v, &mh, &ml);
    ml = ml - 0.5f * d2l;
    /* sin r = st + (st*(cos d - 1) + ct*sin d), cos r = ct + (ct*(cos d - 1) - st*sin d) */
    float sr_h, sr_l, cr_h, cr_l;
    {
        const float ah = sth * mh, al = b2g_fmaf_(sth, mh, -ah) + (sth * ml + stl * mh);
        const float bh = cth * sdh, bl = b2g_fmaf_(cth, sdh, -bh) + (cth * sdl + ctl * sdh);
        float abh, abl;
        b2g_two_sum_(ah, bh, &abh, &abl);
        abl = abl + (al + bl);
        float th, tl;
        b2g_two_sum_(sth, abh, &th, &tl);
        tl = tl + (stl + abl);
        b2g_two_sum_(th, tl, &sr_h, &sr_l);
    }
    {
        const float ah = cth * mh, al = b2g_fmaf_(cth, mh, -ah) + (cth * ml + ctl * mh);
        const float bh = sth * sdh, bl = b2g_fmaf_(sth, sdh, -bh) + (sth * sdl + stl * sdh);
        float abh, abl;
        b2g_two_sum_(ah, -bh, &abh, &abl);
        abl = abl + (al - bl);
        float th, tl;
        b2g_two_sum_(cth, abh, &th, &tl);
        tl = tl + (ctl + abl);
        b2g_two_sum_(th, tl, &cr_h, &cr_l);
    }
    /* quadrant k mod 4 */
    const int q = ((int)kf) & 3;
    float sh, sl, chh, cll;
    if (q == 0) { sh = sr_h; sl = sr_l; chh = cr_h; cll = cr_l; }
    else if (q == 1) { sh = cr_h; sl = cr_l; chh = -sr_h; cll = -sr_l; }
    else if (q == 2) { sh = -sr_h; sl = -sr_l; chh = -cr_h; cll = -cr_l; }
    else { sh = -cr_h; sl = -cr_l; chh = sr_h; cll = sr_l; }
    if (!b2g_rounds_to_hi_(sh, sl) || !b2g_rounds_to_hi_(chh, cll)) {
        b2g_sincosf_ref(x, out_s, out_c);
        return;
    }
    *out_s = sh;
    *out_c = chh;
}

#endif /* B2G_TRIG_H */
