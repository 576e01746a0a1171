/*
 * Elementary functions in fp32 built only from correctly rounded operations
 * (add, subtract, multiply, divide, square root, floor, rint), so that the
 * tessellation kernel and its C restatement evaluate them to the same bits on
 * any machine.
 *
 * The reference's tessellation shader (renderer/src/shaders/tessellate.glsl)
 * calls the shading language's acos, cos and sin, whose precision the language
 * leaves to each GPU; these are one precise choice among the allowed ones.
 * Methods (textbook, coefficients derived here from the series):
 *   sin/cos  Cody-Waite reduction by pi/2 with a three-part constant
 *            (pi/2 = P1 + P2 + P3, P1 and P2 short enough that k * P1 and
 *            k * P2 are exact for |k| < 4096), then the Taylor series of sin
 *            and cos on |r| <= pi/4, through r^11 and r^12;
 *   acos     acos(x) = pi/2 - asin(x) for |x| <= 1/2, and
 *            acos(+-x) = 2 asin(sqrt((1 - x) / 2)) (or pi minus it) otherwise,
 *            with the Taylor series of asin on [0, 1/2] through x^25;
 *   cbrt     exponent split y = m * 2^(3q), a linear first guess on
 *            m in [1/2, 4), then four Newton steps t -= (t - m / t^2) / 3.
 * tests/test_fp32_math.py measures the error of each against double-precision
 * libm over dense sweeps.
 *
 * Compiled as CUDA device code (the operations are the explicit round-to-
 * nearest intrinsics, never contracted) or as C (the caller builds with
 * -ffp-contract=off).
 */
#ifndef RIVE_FP32_MATH_H
#define RIVE_FP32_MATH_H

#include <stdint.h>

#if defined(__CUDACC__)
#define RC_FN __device__ __forceinline__
#define RC_ADD(a, b) __fadd_rn((a), (b))
#define RC_SUB(a, b) __fsub_rn((a), (b))
#define RC_MUL(a, b) __fmul_rn((a), (b))
#define RC_DIV(a, b) __fdiv_rn((a), (b))
#define RC_SQRT(a) __fsqrt_rn(a)
#define RC_RINT(a) rintf(a)
#define RC_F2U(a) __float_as_uint(a)
#define RC_U2F(a) __uint_as_float(a)
#else
#include <math.h>
#include <string.h>
#define RC_FN static inline
#define RC_ADD(a, b) ((a) + (b))
#define RC_SUB(a, b) ((a) - (b))
#define RC_MUL(a, b) ((a) * (b))
#define RC_DIV(a, b) ((a) / (b))
#define RC_SQRT(a) sqrtf(a)
#define RC_RINT(a) rintf(a)
static inline uint32_t rc_f2u_(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static inline float rc_u2f_(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}
#define RC_F2U(a) rc_f2u_(a)
#define RC_U2F(a) rc_u2f_(a)
#endif

/* pi/2 split for the reduction: 0x1.92p+0 + 0x1.fb6p-12 + -0x1.777a5cp-25. */
#define RC_PIO2_1 1.5703125f
#define RC_PIO2_2 4.838705062866211e-4f
#define RC_PIO2_3 -4.371138828673793e-8f
#define RC_TWO_OVER_PI 0.6366197466850281f
/* pi/2 and pi as a float plus the float nearest the remainder. */
#define RC_PIO2_HI 1.5707963705062866f
#define RC_PIO2_LO -4.371138828673793e-8f
#define RC_PI_HI 3.1415927410125732f
#define RC_PI_LO -8.742277657347586e-8f

/* sin(r) and cos(r) for |r| <= pi/4 (a little beyond is harmless): Taylor
 * series, Horner in r^2. */
RC_FN void rc_sincos_kernel(float r, float* s, float* c)
{
    const float z = RC_MUL(r, r);
    /* 1/3!, 1/5!, ..., 1/11! with alternating signs */
    float ps = -2.5052108385441720e-8f;                 /* -1/11! */
    ps = RC_ADD(RC_MUL(ps, z), 2.7557319223985893e-6f); /* 1/9! */
    ps = RC_ADD(RC_MUL(ps, z), -1.9841269841269841e-4f); /* -1/7! */
    ps = RC_ADD(RC_MUL(ps, z), 8.3333333333333333e-3f);  /* 1/5! */
    ps = RC_ADD(RC_MUL(ps, z), -1.6666666666666667e-1f); /* -1/3! */
    *s = RC_ADD(r, RC_MUL(RC_MUL(r, z), ps));
    /* 1/4!, ..., 1/12! */
    float pc = 2.0876756987868099e-9f;                   /* 1/12! */
    pc = RC_ADD(RC_MUL(pc, z), -2.7557319223985891e-7f); /* -1/10! */
    pc = RC_ADD(RC_MUL(pc, z), 2.4801587301587302e-5f);  /* 1/8! */
    pc = RC_ADD(RC_MUL(pc, z), -1.3888888888888889e-3f); /* -1/6! */
    pc = RC_ADD(RC_MUL(pc, z), 4.1666666666666667e-2f);  /* 1/4! */
    /* 1 - z/2 + z^2 * pc */
    *c = RC_ADD(RC_SUB(1.f, RC_MUL(z, .5f)), RC_MUL(RC_MUL(z, z), pc));
}

/* sin(x) and cos(x); NaN for NaN and infinite x. Accurate for |x| < 6400
 * (the reduction's exact range), which covers every angle the tessellation
 * forms (a few turns at most). */
RC_FN void rc_sincosf(float x, float* s, float* c)
{
    const float k = RC_RINT(RC_MUL(x, RC_TWO_OVER_PI));
    float r = RC_SUB(x, RC_MUL(k, RC_PIO2_1));
    r = RC_SUB(r, RC_MUL(k, RC_PIO2_2));
    r = RC_SUB(r, RC_MUL(k, RC_PIO2_3));
    float sr, cr;
    rc_sincos_kernel(r, &sr, &cr);
    /* quadrant = k mod 4 (k is an exact small integer here) */
    const float q4 = RC_SUB(k, RC_MUL(4.f, floorf(RC_MUL(k, .25f))));
    const int q = (q4 == q4) ? (int)q4 : 0;
    switch (q)
    {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
    if (!(x == x) || x - x != 0.f)
    {
        *s = RC_SUB(x, x);
        *c = *s;
    }
}

RC_FN float rc_cosf(float x)
{
    float s, c;
    rc_sincosf(x, &s, &c);
    return c;
}

RC_FN float rc_sinf(float x)
{
    float s, c;
    rc_sincosf(x, &s, &c);
    return s;
}

/* asin(x) for 0 <= x <= 1/2: x + x^3 * P(x^2), P the Taylor series
 * coefficients (2n)! / (4^n (n!)^2 (2n + 1)) for n = 1..12. */
RC_FN float rc_asin_kernel(float x)
{
    const float z = RC_MUL(x, x);
    float p = 6.4472103118896484e-3f;          /* n = 12 */
    p = RC_ADD(RC_MUL(p, z), 7.3125258735988454e-3f); /* 11 */
    p = RC_ADD(RC_MUL(p, z), 8.3903358096168150e-3f); /* 10 */
    p = RC_ADD(RC_MUL(p, z), 9.7616095291940780e-3f); /* 9 */
    p = RC_ADD(RC_MUL(p, z), 1.1551800896139705e-2f); /* 8 */
    p = RC_ADD(RC_MUL(p, z), 1.3964843750000000e-2f); /* 7 */
    p = RC_ADD(RC_MUL(p, z), 1.7352764423076924e-2f); /* 6 */
    p = RC_ADD(RC_MUL(p, z), 2.2372159090909092e-2f); /* 5 */
    p = RC_ADD(RC_MUL(p, z), 3.0381944444444444e-2f); /* 4 */
    p = RC_ADD(RC_MUL(p, z), 4.4642857142857144e-2f); /* 3 */
    p = RC_ADD(RC_MUL(p, z), 7.5000000000000000e-2f); /* 2 */
    p = RC_ADD(RC_MUL(p, z), 1.6666666666666666e-1f); /* 1 */
    return RC_ADD(x, RC_MUL(RC_MUL(x, z), p));
}

/* acos(x) in [0, pi] for x in [-1, 1]; NaN outside. */
RC_FN float rc_acosf(float x)
{
    const float ax = x < 0.f ? -x : x;
    if (ax <= .5f)
    {
        /* pi/2 - asin(x) */
        const float a = rc_asin_kernel(ax);
        return RC_SUB(RC_PIO2_HI, RC_SUB(x < 0.f ? -a : a, RC_PIO2_LO));
    }
    if (!(ax <= 1.f))
        return RC_SUB(x, x) / 0.f; /* NaN */
    const float s = RC_SQRT(RC_MUL(RC_SUB(1.f, ax), .5f));
    const float a2 = RC_MUL(2.f, rc_asin_kernel(s));
    if (x > 0.f)
        return a2;
    /* pi - 2 asin(s) */
    return RC_ADD(RC_SUB(RC_PI_HI, a2), RC_PI_LO);
}

/* Real cube root of y >= 0 (what powf(y, 1/3) approximates); y = 0 and
 * y = +inf return themselves, NaN returns NaN. */
RC_FN float rc_cbrtf(float y)
{
    if (!(y > 0.f) || RC_SUB(y, y) != 0.f)
        return y;
    uint32_t u = RC_F2U(y);
    int e = (int)((u >> 23) & 0xffu);
    float m;
    if (e == 0)
    {
        /* subnormal: scale by 2^24 (exact) and fold it into the exponent */
        const float ys = RC_MUL(y, 16777216.f);
        u = RC_F2U(ys);
        e = (int)((u >> 23) & 0xffu) - 24;
    }
    /* y = m * 2^(e - 126) with m in [1/2, 1); make the exponent a multiple
     * of 3 by moving up to two factors of 2 into m (m in [1/2, 4)). */
    int ex = e - 126;
    int r = ex % 3;
    if (r < 0)
        r += 3;
    const int q = (ex - r) / 3;
    m = RC_U2F((u & 0x007fffffu) | 0x3f000000u); /* [1/2, 1) */
    if (r == 1)
        m = RC_MUL(m, 2.f);
    else if (r == 2)
        m = RC_MUL(m, 4.f);
    /* m in [1/2, 4): first guess on the line through (1/2, cbrt(1/2)) and
     * (4, cbrt(4)), within 10%; each Newton step squares the error. */
    float t = RC_ADD(RC_MUL(m, .2267716f), .6803147f);
    for (int i = 0; i < 4; ++i)
        t = RC_SUB(t, RC_DIV(RC_SUB(t, RC_DIV(m, RC_MUL(t, t))), 3.f));
    /* times 2^q, q in [-50, 43]: build the power of two in two exact steps */
    const int q1 = q / 2, q2 = q - q / 2;
    t = RC_MUL(t, RC_U2F((uint32_t)(127 + q1) << 23));
    return RC_MUL(t, RC_U2F((uint32_t)(127 + q2) << 23));
}

#endif /* RIVE_FP32_MATH_H */
