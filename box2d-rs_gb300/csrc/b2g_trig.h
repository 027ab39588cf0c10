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
 */
#ifndef B2G_TRIG_H
#define B2G_TRIG_H

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

/* sin(x), cos(x) for f32 x. NaN/inf inputs give NaN. */
B2G_HD void b2g_sincosf(float x, float* out_s, float* out_c)
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

#endif /* B2G_TRIG_H */
