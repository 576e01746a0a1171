/*
 * passes.c -- TEST INFRASTRUCTURE (the oracle). A plain, unoptimised C
 * restatement of rive-runtime's rasterOrdering GPU passes. Only tests, the
 * smoke check and the benchmark's CPU-baseline leg may load it, and only as
 * the checker. See passes.h for what each function restates.
 *
 * Arithmetic follows the GLSL statement by statement in fp32 (built with
 * -ffp-contract=off). The tessellation pass takes acos, sin, cos and the cube
 * root from rive_fp32_math.h, the same correctly-rounded-operation
 * implementations the tessellation kernel compiles, so the two agree bit for
 * bit; the other passes use libm. `half` values of the
 * shaders are computed in fp32 (desktop mediump) and rounded to fp16 exactly
 * where the shaders pack them into pixel local storage (packHalf2x16).
 *
 * What pins it: its inputs are the reference front end's own records
 * (captured from the compiled reference, byte for byte); the advanced blend
 * functions reproduce the known answers of the reference's
 * advanced_blend_test.cpp; tessellated vertices agree with an FP64 twin of
 * the same segment parameters. The composed pixels themselves have no
 * reference output to compare with (the reference ships no pixel goldens and
 * its GPU backends need a graphics API, which none of the machines this runs
 * on provides): for the final images this oracle is "parity unpinned".
 */
#include "passes.h"
#include "rive_fp32_math.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- constants (renderer/src/shaders/constants.glsl) --------------------- */
#define TESS_TEXTURE_WIDTH 2048
#define GRAD_TEXTURE_WIDTH 512
#define PI_F 3.14159265359f
#define TWO_PI_F 6.28318530718f
#define AA_RADIUS 0.5f
#define GRAD_SPAN_FLAG_LEFT_BORDER 0x80000000u
#define GRAD_SPAN_FLAG_RIGHT_BORDER 0x40000000u
#define GRAD_SPAN_FLAG_COMPLEX_BORDER 0x20000000u
#define GRAD_SPAN_FLAGS_MASK 0xe0000000u
#define RETROFIT_TRI_STRIP_CONTOUR_FLAG (1u << 31)
#define CULL_EXCESS_TESSELLATION_SEGMENTS_CONTOUR_FLAG (1u << 29)
#define JOIN_TYPE_MASK (7u << 26)
#define MITER_CLIP_JOIN_CONTOUR_FLAG (5u << 26)
#define MITER_REVERT_JOIN_CONTOUR_FLAG (4u << 26)
#define BEVEL_JOIN_CONTOUR_FLAG (3u << 26)
#define ROUND_JOIN_CONTOUR_FLAG (2u << 26)
#define FEATHER_JOIN_CONTOUR_FLAG (1u << 26)
#define EMULATED_STROKE_CAP_CONTOUR_FLAG (1u << 25)
#define NEGATE_PATH_FILL_COVERAGE_FLAG (1u << 24)
#define MIRRORED_CONTOUR_CONTOUR_FLAG (1u << 23)
#define JOIN_TANGENT_0_CONTOUR_FLAG (1u << 22)
#define JOIN_TANGENT_INNER_CONTOUR_FLAG (1u << 21)
#define LEFT_JOIN_CONTOUR_FLAG (1u << 20)
#define RIGHT_JOIN_CONTOUR_FLAG (1u << 19)
#define CONTOUR_ID_MASK 0xffffu
#define STROKE_VERTEX 0
#define FAN_VERTEX 1
#define FAN_MIDPOINT_VERTEX 2
#define CLIP_UPDATE_PAINT_TYPE 0u
#define SOLID_COLOR_PAINT_TYPE 1u
#define LINEAR_GRADIENT_PAINT_TYPE 2u
#define RADIAL_GRADIENT_PAINT_TYPE 3u
#define PAINT_FLAG_EVEN_ODD_FILL 0x200u
#define PAINT_FLAG_HAS_CLIP_RECT 0x400u
#define MAX_DENORM_F16 1023u
#define EPSILON_FP16_NON_DENORM 6.2e-5f
#define BLEND_SRC_OVER 0
#define BLEND_MODE_SCREEN 1
#define BLEND_MODE_OVERLAY 2
#define BLEND_MODE_DARKEN 3
#define BLEND_MODE_LIGHTEN 4
#define BLEND_MODE_COLORDODGE 5
#define BLEND_MODE_COLORBURN 6
#define BLEND_MODE_HARDLIGHT 7
#define BLEND_MODE_SOFTLIGHT 8
#define BLEND_MODE_DIFFERENCE 9
#define BLEND_MODE_EXCLUSION 10
#define BLEND_MODE_MULTIPLY 11
#define BLEND_MODE_HUE 12
#define BLEND_MODE_SATURATION 13
#define BLEND_MODE_COLOR 14
#define BLEND_MODE_LUMINOSITY 15

/* gpu::ShaderFeatures (gpu.hpp:840-856). */
#define SF_CLIPPING (1u << 0)
#define SF_CLIP_RECT (1u << 1)
#define SF_ADVANCED_BLEND (1u << 2)
#define SF_FEATHER (1u << 3)
/* Feathering (constants.glsl:19-43, draw_path_common.glsl:7-13). */
#define GAUSSIAN_TABLE_SIZE 512
#define GAUSSIAN_INTEGRAL_TEXTURE_STDDEVS 3.f
#define FEATHER_COVERAGE_BIAS -2.f
#define FEATHER_COVERAGE_THRESHOLD -1.5f
#define FEATHER_X_COORD_BIAS .25f
#define HORIZONTAL_COTANGENT_THRESHOLD 1e3f
#define HORIZONTAL_COTANGENT_VALUE (HORIZONTAL_COTANGENT_THRESHOLD * HORIZONTAL_COTANGENT_THRESHOLD)
#define FEATHER_JOIN_HELPER_VERTEX_COUNT 3.f
/* midpointFanCenterAAPatches (gpu.hpp:591-640): both AA ramps of an 8-segment
 * span, a middle-out fan and the midpoint triangle. */
#define CENTER_VERTEX_COUNT (PATCH_SEGMENT_SPAN * 8 + PATCH_SEGMENT_SPAN + 2)
#define CENTER_INDEX_COUNT (PATCH_SEGMENT_SPAN * 12 + 7 * 3 + 3)
#define DRAW_TYPE_MIDPOINT_FAN_CENTER_AA_PATCHES 1u
static float feather_lut(float x);
static float inverse_feather_lut(float x);
static void build_feather_table(void);
static void build_inverse_feather_table(void);
#define SF_EVEN_ODD (1u << 4)
/* gpu::ShaderMiscFlags::clockwiseFill of a draw batch (gpu.hpp:917), carried
 * with each triangle's shader features in a bit ShaderFeatures leaves free. */
#define MISC_CLOCKWISE_FILL (1u << 1)
#define FEATURE_CLOCKWISE_FILL (1u << 15)
#define SF_NESTED_CLIPPING (1u << 5)
#define SF_HSL_BLEND_MODES (1u << 6)
#define SF_DITHER (1u << 7)
#define SF_MODULATED_IMAGE (1u << 8)
#define PAINT_FLAG_HAS_IMAGE 0x800u

/* Patch geometry (gpu.hpp:591-640). */
#define PATCH_SEGMENT_SPAN 8
#define PATCH_VERTEX_COUNT 42
#define PATCH_INDEX_COUNT 72
/* Outer-curve patches (gpu.hpp:591-646): 16 curve segments plus a zero-length
 * bowtie join; AA ramps on both sides of the curve, a middle-out fan over the
 * 16 curve segments, no midpoint triangle. */
#define OUTER_SEGMENT_SPAN 17
#define OUTER_VERTEX_COUNT (OUTER_SEGMENT_SPAN * 8 + OUTER_SEGMENT_SPAN)
#define OUTER_INDEX_COUNT (OUTER_SEGMENT_SPAN * 12 + 15 * 3)
#define DRAW_TYPE_OUTER_CURVE_PATCHES 2u
#define DRAW_TYPE_INTERIOR_TRIANGULATION 3u
#define DRAW_TYPE_FEATHER_ATLAS_BLIT 4u
#define DRAW_TYPE_IMAGE_MESH 6u

/* Sub-pixel precision of the rasteriser (Vulkan minimum is 4 bits; desktop
 * parts use 8). */
#define SUBPIXEL_BITS 8
#define SUBPIXEL_ONE (1 << SUBPIXEL_BITS)

typedef struct
{
    float x, y;
} f2;

static uint64_t g_stat_triangles, g_stat_fragments;

/* ---- half floats --------------------------------------------------------- */
uint16_t oracle_f32_to_f16(float f)
{
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t e = (x >> 23) & 0xffu;
    uint32_t m = x & 0x7fffffu;
    if (e == 0xffu) /* inf / nan */
        return (uint16_t)(sign | 0x7c00u | (m ? 0x200u : 0));
    int32_t he = (int32_t)e - 127 + 15;
    if (he >= 31)
        return (uint16_t)(sign | 0x7c00u);
    if (he <= 0)
    {
        if (he < -10)
            return (uint16_t)sign;
        m |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - he);
        uint32_t hm = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1);
        uint32_t half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u)))
            ++hm;
        return (uint16_t)(sign | hm);
    }
    uint32_t hm = m >> 13;
    uint32_t rem = m & 0x1fffu;
    uint32_t h = ((uint32_t)he << 10) | hm;
    if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u)))
        ++h; /* may carry into the exponent, which is correct */
    return (uint16_t)(sign | h);
}

float oracle_f16_to_f32(uint16_t h)
{
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    uint32_t x;
    if (e == 0)
    {
        if (m == 0)
            x = sign;
        else
        {
            int32_t ee = -1;
            do
            {
                ++ee;
                m <<= 1;
            } while ((m & 0x400u) == 0);
            x = sign | ((uint32_t)(127 - 15 - ee) << 23) | ((m & 0x3ffu) << 13);
        }
    }
    else if (e == 31)
        x = sign | 0x7f800000u | (m << 13);
    else
        x = sign | ((e - 15 + 127) << 23) | (m << 13);
    float f;
    memcpy(&f, &x, 4);
    return f;
}

static inline float u2f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static inline uint32_t f2u(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
/* GLSL clamp as GPUs evaluate it, min(max(x, lo), hi) with IEEE minNum and
 * maxNum: a NaN x gives lo (the kernels' fminf(fmaxf(x, lo), hi)). */
static inline float clampf(float x, float lo, float hi)
{
    return fminf(fmaxf(x, lo), hi);
}
/* min and max as the kernels take them (IEEE minNum/maxNum: a NaN operand
 * yields the other one). */
static inline float minf(float a, float b) { return fminf(a, b); }
static inline float maxf(float a, float b) { return fmaxf(a, b); }
static inline float signf(float x)
{
    return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f);
}
static inline float fractf(float x) { return x - floorf(x); }
/* GLSL mod(x, y) = x - y * floor(x / y). */
static inline float glsl_mod(float x, float y) { return x - y * floorf(x / y); }
static inline float dot2(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
static inline f2 sub2(f2 a, f2 b) { return (f2){a.x - b.x, a.y - b.y}; }
static inline f2 add2(f2 a, f2 b) { return (f2){a.x + b.x, a.y + b.y}; }
static inline f2 mul2(f2 a, float s) { return (f2){a.x * s, a.y * s}; }
static inline f2 normalize2(f2 v)
{
    float inv = 1.f / sqrtf(dot2(v, v));
    return (f2){v.x * inv, v.y * inv};
}
static inline float det2(f2 c0, f2 c1) { return c0.x * c1.y - c1.x * c0.y; }
static inline int neq2(f2 a, f2 b) { return a.x != b.x || a.y != b.y; }

/* bezier_utils.glsl:24-32 */
static float cosine_between_vectors(f2 a, f2 b)
{
    float ab_cosTheta = dot2(a, b);
    float ab_pow2 = dot2(a, a) * dot2(b, b);
    return (ab_pow2 == 0.f) ? 1.f
                            : clampf(ab_cosTheta * (1.f / sqrtf(ab_pow2)),
                                     -1.f,
                                     1.f);
}

/* bezier_utils.glsl:65-71 */
static void find_cubic_tangents(f2 p0, f2 p1, f2 p2, f2 p3, f2* t0, f2* t1)
{
    *t0 = sub2(neq2(p0, p1) ? p1 : neq2(p1, p2) ? p2 : p3, p0);
    *t1 = sub2(p3, neq2(p3, p2) ? p2 : neq2(p2, p1) ? p1 : p0);
}

/* common.glsl atan2 */
static float rive_atan2(f2 v)
{
    v = normalize2(v);
    float theta = rc_acosf(clampf(v.x, -1.f, 1.f));
    return v.y >= 0.f ? theta : -theta;
}

/* ---- pass 1: color ramps (color_ramp.glsl:40-107) ------------------------ */
static void unpack_color_int(uint32_t c, float out[4])
{
    out[0] = (float)((c >> 16) & 0xffu) / 255.f;
    out[1] = (float)((c >> 8) & 0xffu) / 255.f;
    out[2] = (float)((c >> 0) & 0xffu) / 255.f;
    out[3] = (float)((c >> 24) & 0xffu) / 255.f;
}

static inline uint8_t unorm8(float x)
{
    x = clampf(x, 0.f, 1.f);
    return (uint8_t)floorf(x * 255.f + 0.5f);
}

int oracle_color_ramps(const rive_cuda_flush_desc* d,
                       const oracle_buffers* b,
                       uint8_t* grad)
{
    const uint32_t H = d->grad_data_height;
    memset(grad, 0, (size_t)GRAD_TEXTURE_WIDTH * H * 4);
    if (d->grad_span_count == 0)
        return 0;
    if ((size_t)(d->first_grad_span + d->grad_span_count) * 16 >
        b->grad_spans_bytes)
        return -1;
    const uint32_t* spans = (const uint32_t*)b->grad_spans;
    for (uint32_t s = 0; s < d->grad_span_count; ++s)
    {
        const uint32_t* sp = spans + 4 * (size_t)(d->first_grad_span + s);
        uint32_t yWithFlags = sp[1];
        uint32_t y = yWithFlags & ~GRAD_SPAN_FLAGS_MASK;
        if (y >= H)
            continue;
        /* Column x positions of the 8-vertex strip, in texels. */
        float cx[4];
        cx[0] = cx[1] = (float)(sp[0] & 0xffffu) / 65536.f;
        cx[2] = cx[3] = (float)(sp[0] >> 16) / 65536.f;
        if (yWithFlags & GRAD_SPAN_FLAG_LEFT_BORDER)
            cx[0] = (yWithFlags & GRAD_SPAN_FLAG_COMPLEX_BORDER)
                        ? 0.f
                        : cx[0] - 1.f / GRAD_TEXTURE_WIDTH;
        if (yWithFlags & GRAD_SPAN_FLAG_RIGHT_BORDER)
            cx[3] = (yWithFlags & GRAD_SPAN_FLAG_COMPLEX_BORDER)
                        ? 1.f
                        : cx[3] + 1.f / GRAD_TEXTURE_WIDTH;
        float c0[4], c1[4];
        unpack_color_int(sp[2], c0);
        unpack_color_int(sp[3], c1);
        for (int q = 0; q < 3; ++q)
        {
            float xa = cx[q] * GRAD_TEXTURE_WIDTH;
            float xb = cx[q + 1] * GRAD_TEXTURE_WIDTH;
            if (!(xb > xa))
                continue;
            for (int i = 0; i < GRAD_TEXTURE_WIDTH; ++i)
            {
                float pc = (float)i + .5f;
                /* Left edge inclusive, right edge exclusive (top-left). */
                if (pc < xa || pc >= xb)
                    continue;
                float col[4];
                if (q == 0)
                    memcpy(col, c0, sizeof(col));
                else if (q == 2)
                    memcpy(col, c1, sizeof(col));
                else
                {
                    float t = (pc - xa) / (xb - xa);
                    for (int k = 0; k < 4; ++k)
                        col[k] = c0[k] + (c1[k] - c0[k]) * t;
                }
                uint8_t* px = grad + ((size_t)y * GRAD_TEXTURE_WIDTH + i) * 4;
                for (int k = 0; k < 4; ++k)
                    px[k] = unorm8(col[k]);
            }
        }
    }
    return 0;
}

/* ---- pass 2: tessellation (tessellate.glsl:61-567) ------------------------ */
typedef struct
{
    f2 p0, p1, p2, p3;
    float totalVertexCount;
    float parametricSegmentCount;
    float joinSegmentCount;
    float radsPerPolarSegment;
    f2 joinTangent;
    float radsPerJoinSegment;
    uint32_t contourIDWithFlags;
} tess_varyings;

static const float* path_record(const rive_cuda_flush_desc* d,
                                const oracle_buffers* b,
                                uint32_t pathID)
{
    size_t idx = (size_t)d->first_path + pathID;
    if ((idx + 1) * 64 > b->paths_bytes)
        return NULL;
    return (const float*)b->paths + idx * 16;
}

static const uint32_t* contour_record(const rive_cuda_flush_desc* d,
                                      const oracle_buffers* b,
                                      uint32_t contourID)
{
    size_t idx = (size_t)d->first_contour + contourID - 1;
    if ((idx + 1) * 16 > b->contours_bytes)
        return NULL;
    return (const uint32_t*)b->contours + idx * 4;
}

/* GLSL mix(): x * (1 - a) + y * a. */
static inline f2 glsl_mix2(f2 x, f2 y, float a)
{
    return (f2){x.x * (1.f - a) + y.x * a, x.y * (1.f - a) + y.y * a};
}

/* clamped_divide (bezier_utils.glsl:164-169): clamp(a/b, 0, 1). */
static float clamped_divide(float a, float b)
{
    a = b < 0.f ? -a : a;
    b = fabsf(b);
    return a > 0.f ? (a < b ? a / b : 1.f) : 0.f;
}

/* find_cubic_max_height (bezier_utils.glsl:173-245): three Newton steps from
 * t = 1/2 on the height above the chord. */
static float find_cubic_max_height(f2 p0, f2 p1, f2 p2, f2 p3, float* outT)
{
    f2 base = sub2(p3, p0);
    float lengthBase = sqrtf(dot2(base, base));
    if (lengthBase == 0.f)
    {
        *outT = .5f;
        return 0.f;
    }
    f2 norm = {-base.y / lengthBase, base.x / lengthBase};
    float h2 = dot2(norm, sub2(p2, p0));
    float h1 = dot2(norm, sub2(p1, p0));
    float dh = h1 - h2;
    float _3A = 3.f * dh;
    float B = -h1 - dh;
    float C = h1;
    float t = .5f;
    for (int i = 0; i < 3; ++i)
    {
        float _3At = _3A * t;
        t = clamped_divide(_3At * t - C, 2.f * (_3At + B));
    }
    *outT = t;
    return fabsf(t * (t * (t * _3A + 3.f * B) + 3.f * C));
}

/* measure_cubic_local_curvature (bezier_utils.glsl:77-153): the turn, in
 * radians, across a spread of `desiredSpread` centred at T. */
static float measure_cubic_local_curvature(f2 p0, f2 p1, f2 p2, f2 p3, float T,
                                           float desiredSpread)
{
    f2 C = sub2(p1, p0);
    f2 D = sub2(p2, p1);
    f2 E = sub2(p3, p0);
    f2 B = sub2(D, C);
    f2 A = add2(mul2(D, -3.f), E);
    f2 tangent = mul2(add2(mul2(add2(mul2(A, T), mul2(B, 2.f)), T), C), 3.f);
    float lengthTan = sqrtf(dot2(tangent, tangent));
    if (lengthTan == 0.f)
        return 0.f;
    tangent = mul2(tangent, 1.f / lengthTan);
    float A_ = 2.f * dot2(A, tangent);
    float C_ = 3.f * (A_ * T + 4.f * dot2(B, tangent)) * T + 6.f * dot2(C, tangent);
    float maxDT = minf(T, 1.f - T);
    float maxSpread = (A_ * maxDT * maxDT + C_) * maxDT;
    float targetSpread = minf(desiredSpread, maxSpread * .9999f);
    float dt;
    if (A_ == 0.f)
    {
        dt = targetSpread / C_;
    }
    else
    {
        float r = 1.f / A_;
        float b = C_ * r, c = -targetSpread * r;
        float Q = (-1.f / 3.f) * b, R = .5f * c;
        float discr = R * R - Q * Q * Q;
        if (discr < 0.f)
        {
            float sqrtQ = sqrtf(Q);
            float th = rc_acosf(R / (sqrtQ * sqrtQ * sqrtQ));
            dt = -2.f * sqrtQ * rc_cosf(th * (1.f / 3.f) + (-PI_F * 2.f / 3.f));
        }
        else
        {
            float Aq = rc_cbrtf(fabsf(R) + sqrtf(discr));
            if (R < 0.f)
                Aq = -Aq;
            dt = Aq != 0.f ? Aq + Q / Aq : 0.f;
        }
    }
    dt = fabsf(dt);
    float t0 = T - dt, t1 = T + dt;
    f2 dir0 = add2(mul2(add2(mul2(A, t0), mul2(B, 2.f)), t0), C);
    f2 dir1 = add2(mul2(add2(mul2(A, t1), mul2(B, 2.f)), t1), C);
    f2 e0, e1;
    find_cubic_tangents(p0, p1, p2, p3, &e0, &e1);
    f2 tan0 = t0 < 1e-3f ? e0 : dir0;
    f2 tan1 = t1 > 1.f - 1e-3f ? e1 : dir1;
    return rc_acosf(cosine_between_vectors(tan0, tan1));
}

/* Compensated De Casteljau (Graillat, Langlois and Louvet's compensated
 * evaluation): every mix (b - a) * t + a is computed with its exact rounding
 * errors (TwoSum for the sums, a fused multiply-subtract for the product),
 * the errors are carried through the levels with the values, and the point
 * is value + error rounded once: as if evaluated in twice the precision, so
 * the fp32 point is within about half an ulp of the exact point at T. */
static inline float two_sum_err(float a, float b, float s)
{
    const float bb = s - a;
    return (a - (s - bb)) + (b - bb);
}

typedef struct
{
    float v, e; /* value and its (first-order) error term */
} cfloat;

static inline cfloat cmix(cfloat a, cfloat b, float t)
{
    const float d = b.v - a.v;
    const float ed = two_sum_err(b.v, -a.v, d);
    const float p = d * t;
    const float ep = fmaf(d, t, -p);
    const float r = a.v + p;
    const float er = two_sum_err(a.v, p, r);
    /* a + (b - a) t = r + er + ep + ed t, plus the inputs' errors mixed. */
    const float e = ((er + ep) + ed * t) + fmaf(b.e - a.e, t, a.e);
    return (cfloat){r, e};
}

static float eval_cubic_c(float a0, float a1, float a2, float a3, float t, float* t0, float* t1)
{
    const cfloat p0 = {a0, 0.f}, p1 = {a1, 0.f}, p2 = {a2, 0.f}, p3 = {a3, 0.f};
    const cfloat ab = cmix(p0, p1, t), bc = cmix(p1, p2, t), cd = cmix(p2, p3, t);
    const cfloat abc = cmix(ab, bc, t), bcd = cmix(bc, cd, t);
    const cfloat r = cmix(abc, bcd, t);
    *t0 = abc.v;
    *t1 = bcd.v;
    return r.v + r.e;
}

/* The tessellated point at T by De Casteljau (tessellate.glsl:535-540),
 * compensated as above. *abc and *bcd are the last level's pair, whose
 * difference is the tangent. */
static f2 eval_cubic_mix(f2 p0, f2 p1, f2 p2, f2 p3, float T, f2* abc, f2* bcd)
{
    f2 q;
    q.x = eval_cubic_c(p0.x, p1.x, p2.x, p3.x, T, &abc->x, &bcd->x);
    q.y = eval_cubic_c(p0.y, p1.y, p2.y, p3.y, T, &abc->y, &bcd->y);
    return q;
}

/* The parametric segment count of a cubic in pixel space under the path's
 * 2x2 matrix m (columns (m0, m1), (m2, m3)): Wang's formula at precision 4,
 * as the CULL_EXCESS_TESSELLATION_SEGMENTS recount (tessellate.glsl:195-211)
 * evaluates it. */
static float wang_cubic_segments(f2 p0, f2 p1, f2 p2, f2 p3, const float* m)
{
    f2 a = {-2.f * p1.x + p2.x + p0.x, -2.f * p1.y + p2.y + p0.y};
    f2 c = {-2.f * p2.x + p3.x + p1.x, -2.f * p2.y + p3.y + p1.y};
    f2 d0 = {m[0] * a.x + m[2] * a.y, m[1] * a.x + m[3] * a.y};
    f2 d1 = {m[0] * c.x + m[2] * c.y, m[1] * c.x + m[3] * c.y};
    float mm = maxf(dot2(d0, d0), dot2(d1, d1));
    return maxf(ceilf(sqrtf(.75f * 4.f * sqrtf(mm))), 1.f);
}

/* Vertex-shader half of pass 2, evaluated once per span rectangle. */
static int tess_setup(const rive_cuda_flush_desc* d,
                      const oracle_buffers* b,
                      const uint32_t* sp,
                      int second,
                      tess_varyings* v,
                      int* out_x0,
                      int* out_x1,
                      float* out_y)
{
    const float* spf = (const float*)sp;
    f2 p0 = {spf[0], spf[1]}, p1 = {spf[2], spf[3]};
    f2 p2 = {spf[4], spf[5]}, p3 = {spf[6], spf[7]};
    float y = second ? spf[11] : spf[10];
    int32_t x0x1 = (int32_t)(second ? sp[13] : sp[12]);
    int x0 = (int32_t)((uint32_t)x0x1 << 16) >> 16;
    int x1 = x0x1 >> 16;
    uint32_t args_z = sp[14];
    uint32_t parametricSegmentCount = args_z & 0x3ffu;
    uint32_t polarSegmentCount = (args_z >> 10) & 0x3ffu;
    uint32_t joinSegmentCount = args_z >> 20;
    uint32_t contourIDWithFlags = sp[15];
    uint32_t contourID = contourIDWithFlags & CONTOUR_ID_MASK;
    uint32_t pathID = 0;
    if (contourID > 0)
    {
        const uint32_t* c = contour_record(d, b, contourID);
        if (!c)
            return -1;
        pathID = c[2];
    }
    float strokeRadius = 0, featherRadius = 0;
    const float* path = NULL;
    if (pathID != 0)
    {
        path = path_record(d, b, pathID);
        if (!path)
            return -1;
        strokeRadius = path[6];
        featherRadius = path[7];
    }
    if (featherRadius != 0.f && strokeRadius == 0.f)
    {
        /* tessellate.glsl:141-190: a cubic of a feathered fill is flattened
         * toward its chord, more where it curves, to mimic the softening a
         * feather gets from curvature. */
        float maxHeightT;
        float height = find_cubic_max_height(p0, p1, p2, p3, &maxHeightT);
        float oneStddev = featherRadius * (1.f / GAUSSIAN_INTEGRAL_TEXTURE_STDDEVS);
        float curvature = measure_cubic_local_curvature(p0, p1, p2, p3, maxHeightT, oneStddev);
        float dimming = 1.f - curvature * (1.f / PI_F);
        f2 base = sub2(p3, p0);
        float stddevsPow2 = dot2(base, base) / (oneStddev * oneStddev);
        float dimmingByStddevs = (stddevsPow2 - 1.f) * .5f;
        dimming = minf(dimming, dimmingByStddevs);
        dimming = minf(dimming, .99f);
        float desiredOpacityOnCenter = .5f * dimming;
        float x = inverse_feather_lut(desiredOpacityOnCenter) * -2.f + 1.f;
        float softness = clamped_divide(x * featherRadius, height);
        f2 flat1 = glsl_mix2(p0, p3, 1.f / 3.f), flat2 = glsl_mix2(p0, p3, 2.f / 3.f);
        p1 = glsl_mix2(p1, flat1, softness);
        p2 = glsl_mix2(p2, flat2, softness);
    }
    if (contourIDWithFlags & CULL_EXCESS_TESSELLATION_SEGMENTS_CONTOUR_FLAG)
    {
        if (!path)
            path = path_record(d, b, pathID);
        if (!path)
            return -1;
        /* mat = [[m0, m1], [m2, m3]] columns; MUL(mat, v). */
        uint32_t un = (uint32_t)wang_cubic_segments(p0, p1, p2, p3, path);
        parametricSegmentCount =
            un < parametricSegmentCount ? un : parametricSegmentCount;
    }
    uint32_t totalVertexCount =
        parametricSegmentCount + polarSegmentCount + joinSegmentCount - 1u;
    f2 t0, t1;
    find_cubic_tangents(p0, p1, p2, p3, &t0, &t1);
    float theta = rc_acosf(cosine_between_vectors(t0, t1));
    float radsPerPolarSegment = theta / (float)polarSegmentCount;
    float turn = det2(sub2(p2, p0), sub2(p3, p1));
    if (turn == 0.f)
        turn = det2(t0, t1);
    if (turn < 0.f)
        radsPerPolarSegment = -radsPerPolarSegment;
    v->p0 = p0;
    v->p1 = p1;
    v->p2 = p2;
    v->p3 = p3;
    v->totalVertexCount = (float)totalVertexCount;
    v->parametricSegmentCount = (float)parametricSegmentCount;
    v->joinSegmentCount = (float)joinSegmentCount;
    v->radsPerPolarSegment = radsPerPolarSegment;
    v->joinTangent = (f2){spf[8], spf[9]};
    v->radsPerJoinSegment = 0.f;
    if (joinSegmentCount > 1u)
    {
        f2 jt = v->joinTangent;
        float joinTheta = rc_acosf(cosine_between_vectors(t1, jt));
        float joinSpan = (float)joinSegmentCount;
        if ((contourIDWithFlags &
             (JOIN_TYPE_MASK | EMULATED_STROKE_CAP_CONTOUR_FLAG)) ==
            (ROUND_JOIN_CONTOUR_FLAG | EMULATED_STROKE_CAP_CONTOUR_FLAG))
            joinSpan -= 2.f;
        float radsPerJoinSegment = joinTheta / joinSpan;
        if (det2(t1, jt) < 0.f)
            radsPerJoinSegment = -radsPerJoinSegment;
        v->radsPerJoinSegment = radsPerJoinSegment;
    }
    if (x1 < x0)
        contourIDWithFlags |= MIRRORED_CONTOUR_CONTOUR_FLAG;
    v->contourIDWithFlags = contourIDWithFlags;
    *out_x0 = x0;
    *out_x1 = x1;
    *out_y = y;
    return 0;
}

/* Fragment half of pass 2 (tessellate.glsl:294-567): one vertex. */
static void tess_fragment_t(const tess_varyings* v,
                            float vertexIdxIn,
                            uint32_t out[4],
                            float* outT,
                            f2 outPts[4])
{
    f2 p0 = v->p0, p1 = v->p1, p2 = v->p2, p3 = v->p3;
    f2 tan0, tan1;
    find_cubic_tangents(p0, p1, p2, p3, &tan0, &tan1);
    float vertexIdx = maxf(floorf(vertexIdxIn), 0.f);
    float totalVertexCount = v->totalVertexCount;
    float parametricSegmentCount = v->parametricSegmentCount;
    float joinSegmentCount = v->joinSegmentCount;
    float radsPerPolarSegment = v->radsPerPolarSegment;
    uint32_t contourIDWithFlags = v->contourIDWithFlags;

    float mergedSegmentCount = totalVertexCount - joinSegmentCount;
    float mergedVertexID = vertexIdx;
    if (mergedVertexID <= mergedSegmentCount)
    {
        contourIDWithFlags &= ~JOIN_TYPE_MASK;
    }
    else
    {
        p0 = p1 = p2 = p3;
        tan0 = tan1;
        tan1 = v->joinTangent;
        parametricSegmentCount = 1.f;
        mergedVertexID -= mergedSegmentCount;
        mergedSegmentCount = joinSegmentCount;
        radsPerPolarSegment = v->radsPerJoinSegment;
        if ((contourIDWithFlags & JOIN_TYPE_MASK) > ROUND_JOIN_CONTOUR_FLAG)
        {
            if (mergedVertexID < 2.5f)
                contourIDWithFlags |= JOIN_TANGENT_0_CONTOUR_FLAG;
            if (mergedVertexID > 1.5f && mergedVertexID < 3.5f)
                contourIDWithFlags |= JOIN_TANGENT_INNER_CONTOUR_FLAG;
        }
        else if ((contourIDWithFlags & EMULATED_STROKE_CAP_CONTOUR_FLAG) ||
                 (contourIDWithFlags & JOIN_TYPE_MASK) ==
                     FEATHER_JOIN_CONTOUR_FLAG)
        {
            mergedSegmentCount -= 2.f;
            mergedVertexID -= 1.f;
        }
        contourIDWithFlags |= radsPerPolarSegment < 0.f
                                  ? LEFT_JOIN_CONTOUR_FLAG
                                  : RIGHT_JOIN_CONTOUR_FLAG;
    }

    f2 tessCoord;
    float theta = 0.f;
    if (mergedVertexID == 0.f || mergedVertexID == mergedSegmentCount ||
        (contourIDWithFlags & JOIN_TYPE_MASK) > ROUND_JOIN_CONTOUR_FLAG)
    {
        int isTan0 = mergedVertexID < mergedSegmentCount * .5f;
        tessCoord = isTan0 ? p0 : p3;
        theta = rive_atan2(isTan0 ? tan0 : tan1);
    }
    else if (contourIDWithFlags & RETROFIT_TRI_STRIP_CONTOUR_FLAG)
    {
        tessCoord = p0;
        if (mergedVertexID >= 8.f)
            tessCoord = p1;
        if (mergedVertexID >= 12.f)
            tessCoord = p2;
        if (mergedVertexID >= 14.f)
            tessCoord = v->joinTangent;
    }
    else
    {
        float T, polarT;
        if (parametricSegmentCount == mergedSegmentCount)
        {
            T = mergedVertexID / parametricSegmentCount;
            polarT = 0.f;
        }
        else
        {
            f2 C = sub2(p1, p0);
            f2 D = sub2(p3, p0);
            f2 E = sub2(p2, p1);
            f2 B = sub2(E, C);
            f2 A = add2(mul2(E, -3.f), D);
            f2 B_ = mul2(B, parametricSegmentCount * 2.f);
            f2 C_ = mul2(C, parametricSegmentCount * parametricSegmentCount);
            float lastParametricVertexID = 0.f;
            float maxParametricVertexID =
                minf(parametricSegmentCount - 1.f, mergedVertexID);
            f2 tan0norm = normalize2(tan0);
            float negAbsRadsPerSegment = -fabsf(radsPerPolarSegment);
            float maxRotation0 = (1.f + mergedVertexID) * fabsf(radsPerPolarSegment);
            for (int p = 9; p >= 0; --p)
            {
                float testParametricID = lastParametricVertexID + exp2f((float)p);
                if (testParametricID <= maxParametricVertexID)
                {
                    f2 testTan = add2(mul2(A, testParametricID), B_);
                    testTan = add2(mul2(testTan, testParametricID), C_);
                    float cosRotation = dot2(normalize2(testTan), tan0norm);
                    float maxRotation =
                        testParametricID * negAbsRadsPerSegment + maxRotation0;
                    maxRotation = minf(maxRotation, PI_F);
                    if (cosRotation >= rc_cosf(maxRotation))
                        lastParametricVertexID = testParametricID;
                }
            }
            float parametricT = lastParametricVertexID / parametricSegmentCount;
            float lastPolarVertexID = mergedVertexID - lastParametricVertexID;
            float theta0 = rc_acosf(clampf(tan0norm.x, -1.f, 1.f));
            theta0 = tan0norm.y >= 0.f ? theta0 : -theta0;
            theta = lastPolarVertexID * radsPerPolarSegment + theta0;
            float sn, cs;
            rc_sincosf(theta, &sn, &cs);
            f2 norm = {sn, -cs};
            float a = dot2(norm, A), b_over_2 = dot2(norm, B), c = dot2(norm, C);
            float discr_over_4 = maxf(b_over_2 * b_over_2 - a * c, 0.f);
            float q = sqrtf(discr_over_4);
            if (b_over_2 > 0.f)
                q = -q;
            q -= b_over_2;
            float _5qa = -.5f * q * a;
            float rs, rt;
            if (fabsf(q * q + _5qa) < fabsf(a * c + _5qa))
            {
                rs = q;
                rt = a;
            }
            else
            {
                rs = c;
                rt = q;
            }
            polarT = (rt != 0.f) ? rs / rt : 0.f;
            polarT = clampf(polarT, 0.f, 1.f);
            if (lastPolarVertexID == 0.f)
                polarT = 0.f;
            T = maxf(parametricT, polarT);
        }
        f2 abc, bcd;
        tessCoord = eval_cubic_mix(p0, p1, p2, p3, T, &abc, &bcd);
        if (T != polarT)
            theta = rive_atan2(sub2(bcd, abc));
        if (outT)
        {
            *outT = T;
            outPts[0] = p0;
            outPts[1] = p1;
            outPts[2] = p2;
            outPts[3] = p3;
        }
    }
    out[0] = f2u(tessCoord.x);
    out[1] = f2u(tessCoord.y);
    if ((contourIDWithFlags & JOIN_TYPE_MASK) == FEATHER_JOIN_CONTOUR_FLAG)
    {
        /* tessellate.glsl:551-559: feather joins hand their stepping to the
         * draw pass. */
        out[2] = ((uint32_t)mergedSegmentCount << 16) | (uint32_t)mergedVertexID;
    }
    else
    {
        out[2] = f2u(glsl_mod(theta, TWO_PI_F));
    }
    out[3] = contourIDWithFlags;
}

static void tess_fragment(const tess_varyings* v, float vertexIdxIn, uint32_t out[4])
{
    tess_fragment_t(v, vertexIdxIn, out, NULL, NULL);
}

int oracle_tessellate(const rive_cuda_flush_desc* d,
                      const oracle_buffers* b,
                      uint32_t* tess)
{
    build_feather_table(); /* feathered fills soften through the inverse table */
    const uint32_t H = d->tess_data_height;
    memset(tess, 0, (size_t)TESS_TEXTURE_WIDTH * H * 16);
    if ((size_t)(d->first_tess_span + d->tess_span_count) * 64 >
        b->tess_spans_bytes)
        return -1;
    const uint32_t* spans = (const uint32_t*)b->tess_spans;
    for (uint32_t s = 0; s < d->tess_span_count; ++s)
    {
        const uint32_t* sp = spans + 16 * (size_t)(d->first_tess_span + s);
        for (int second = 0; second < 2; ++second)
        {
            tess_varyings v;
            int x0, x1;
            float y;
            int rc = tess_setup(d, b, sp, second, &v, &x0, &x1, &y);
            if (rc != 0)
                return rc;
            if (isnan(y) || x0 == x1)
                continue;
            if (y < 0.f || y >= (float)H)
                continue;
            int row = (int)y;
            int lo = x0 < x1 ? x0 : x1, hi = x0 < x1 ? x1 : x0;
            if (lo < 0)
                lo = 0;
            if (hi > TESS_TEXTURE_WIDTH)
                hi = TESS_TEXTURE_WIDTH;
            for (int px = lo; px < hi; ++px)
            {
                float vertexIdx =
                    v.totalVertexCount - fabsf((float)x1 - ((float)px + .5f));
                tess_fragment(&v, vertexIdx,
                              tess + ((size_t)row * TESS_TEXTURE_WIDTH + px) * 4);
            }
        }
    }
    return 0;
}

/* ---- FP64 twin of pass 2 --------------------------------------------------
 * For the tessellated-vertex tolerance: the same segment parameters (the
 * merged vertex's T, chosen by the fp32 algorithm above) evaluated in double
 * precision with De Casteljau. Endpoint and join vertices are exact copies of
 * control points in both and are returned as such.
 */
int oracle_tessellate_f64(const rive_cuda_flush_desc* d,
                          const oracle_buffers* b,
                          double* xy,
                          uint32_t* tess_flags)
{
    build_feather_table(); /* feathered fills soften through the inverse table */
    const uint32_t H = d->tess_data_height;
    const size_t N = (size_t)TESS_TEXTURE_WIDTH * H;
    memset(xy, 0, N * 2 * sizeof(double));
    memset(tess_flags, 0, N * sizeof(uint32_t));
    if ((size_t)(d->first_tess_span + d->tess_span_count) * 64 >
        b->tess_spans_bytes)
        return -1;
    const uint32_t* spans = (const uint32_t*)b->tess_spans;
    for (uint32_t s = 0; s < d->tess_span_count; ++s)
    {
        const uint32_t* sp = spans + 16 * (size_t)(d->first_tess_span + s);
        for (int second = 0; second < 2; ++second)
        {
            tess_varyings v;
            int x0, x1;
            float y;
            int rc = tess_setup(d, b, sp, second, &v, &x0, &x1, &y);
            if (rc != 0)
                return rc;
            if (isnan(y) || x0 == x1 || y < 0.f || y >= (float)H)
                continue;
            int row = (int)y;
            int lo = x0 < x1 ? x0 : x1, hi = x0 < x1 ? x1 : x0;
            if (lo < 0)
                lo = 0;
            if (hi > TESS_TEXTURE_WIDTH)
                hi = TESS_TEXTURE_WIDTH;
            for (int px = lo; px < hi; ++px)
            {
                size_t texel = (size_t)row * TESS_TEXTURE_WIDTH + px;
                uint32_t o[4];
                float T = -1.f;
                f2 q[4];
                float vertexIdx =
                    v.totalVertexCount - fabsf((float)x1 - ((float)px + .5f));
                tess_fragment_t(&v, vertexIdx, o, &T, q);
                tess_flags[texel] = o[3];
                if (T < 0.f)
                {
                    xy[texel * 2 + 0] = u2f(o[0]);
                    xy[texel * 2 + 1] = u2f(o[1]);
                    continue;
                }
                double t = T;
                double ax = q[0].x + (q[1].x - (double)q[0].x) * t;
                double ay = q[0].y + (q[1].y - (double)q[0].y) * t;
                double bx = q[1].x + (q[2].x - (double)q[1].x) * t;
                double by = q[1].y + (q[2].y - (double)q[1].y) * t;
                double cx = q[2].x + (q[3].x - (double)q[2].x) * t;
                double cy = q[2].y + (q[3].y - (double)q[2].y) * t;
                double abx = ax + (bx - ax) * t, aby = ay + (by - ay) * t;
                double bcx = bx + (cx - bx) * t, bcy = by + (cy - by) * t;
                xy[texel * 2 + 0] = abx + (bcx - abx) * t;
                xy[texel * 2 + 1] = aby + (bcy - aby) * t;
            }
        }
    }
    return 0;
}

/* ---- pass 3: draw + raster-ordered resolve -------------------------------- */

/* Patch vertex/index tables for PatchType::midpointFan (gpu.cpp:446-687). */
typedef struct
{
    float localVertexID, outset, fillCoverage;
    int32_t params;
    float mLocalVertexID, mOutset, mFillCoverage;
} patch_vertex;

static patch_vertex g_patch[PATCH_VERTEX_COUNT];
static uint16_t g_patch_idx[PATCH_INDEX_COUNT];
static patch_vertex g_outer[OUTER_VERTEX_COUNT];
static patch_vertex g_center[CENTER_VERTEX_COUNT];
static uint16_t g_center_idx[CENTER_INDEX_COUNT];
static uint16_t g_outer_idx[OUTER_INDEX_COUNT];
static int g_patch_ready = 0;

static void pv_set(patch_vertex* v, float l, float o, float c, int32_t params)
{
    v->localVertexID = l;
    v->outset = o;
    v->fillCoverage = c;
    v->params = params;
    v->mLocalVertexID = l;
    v->mOutset = o;
    v->mFillCoverage = c;
}
static void pv_mirror(patch_vertex* v, float l, float o, float c)
{
    v->mLocalVertexID = l;
    v->mOutset = o;
    v->mFillCoverage = c;
}

static void build_patch_tables(void)
{
    if (g_patch_ready)
        return;
    int n = 0;
    const int span = PATCH_SEGMENT_SPAN;
    int32_t strokeParams = (span << 2) | STROKE_VERTEX;
    for (int i = 0; i < span; ++i)
    {
        float l = (float)i, r = l + 1.f;
        pv_set(&g_patch[n + 0], l, -1.f, 1.f, strokeParams);
        pv_set(&g_patch[n + 1], l, +1.f, 0.f, strokeParams);
        pv_set(&g_patch[n + 2], r, -1.f, 1.f, strokeParams);
        pv_set(&g_patch[n + 3], r, +1.f, 0.f, strokeParams);
        pv_mirror(&g_patch[n + 0], r - 1.f, -1.f, 1.f);
        pv_mirror(&g_patch[n + 1], l - 1.f, -1.f, 1.f);
        pv_mirror(&g_patch[n + 2], r - 1.f, +1.f, 0.f);
        pv_mirror(&g_patch[n + 3], l - 1.f, +1.f, 0.f);
        n += 4;
    }
    int fanIdx = n;
    for (int i = 0; i <= span; ++i)
    {
        pv_set(&g_patch[n], (float)i, -1.f, 1.f, (span << 2) | FAN_VERTEX);
        pv_mirror(&g_patch[n], (float)i - 1.f, -1.f, 1.f);
        ++n;
    }
    int midIdx = n;
    pv_set(&g_patch[n++], 0.f, 0.f, 1.f, (span << 2) | FAN_MIDPOINT_VERTEX);
    static const uint16_t border[6] = {0, 1, 2, 2, 1, 3};
    int k = 0, e = 0;
    for (int s = 0; s < span; ++s)
    {
        for (int i = 0; i < 6; ++i)
            g_patch_idx[k++] = (uint16_t)(e + border[i]);
        e += 4;
    }
    for (int step = 1; step < span; step <<= 1)
        for (int i = 0; i < span; i += step * 2)
        {
            g_patch_idx[k++] = (uint16_t)(fanIdx + i);
            g_patch_idx[k++] = (uint16_t)(fanIdx + i + step);
            g_patch_idx[k++] = (uint16_t)(fanIdx + i + step * 2);
        }
    g_patch_idx[k++] = (uint16_t)fanIdx;
    g_patch_idx[k++] = (uint16_t)(fanIdx + span);
    g_patch_idx[k++] = (uint16_t)midIdx;
    (void)n;

    /* Outer-curve patch (gpu.cpp:446-687, PatchType::outerCurves). */
    const int ospan = OUTER_SEGMENT_SPAN;
    const int32_t oStroke = (ospan << 2) | STROKE_VERTEX;
    n = 0;
    for (int i = 0; i < ospan; ++i) /* top side of the centred AA ramp */
    {
        float l = (float)i, r = l + 1.f;
        pv_set(&g_outer[n + 0], l, 0.f, .5f, oStroke);
        pv_set(&g_outer[n + 1], l, 1.f, 0.f, oStroke);
        pv_set(&g_outer[n + 2], r, 0.f, .5f, oStroke);
        pv_set(&g_outer[n + 3], r, 1.f, 0.f, oStroke);
        pv_mirror(&g_outer[n + 0], r, 0.f, .5f);
        pv_mirror(&g_outer[n + 1], l, 0.f, .5f);
        pv_mirror(&g_outer[n + 2], r, 1.f, 0.f);
        pv_mirror(&g_outer[n + 3], l, 1.f, 0.f);
        n += 4;
    }
    for (int i = 0; i < ospan; ++i) /* bottom (negative coverage) side */
    {
        float l = (float)i, r = l + 1.f;
        pv_set(&g_outer[n + 0], l, -0.f, .5f, oStroke);
        pv_set(&g_outer[n + 1], r, -0.f, .5f, oStroke);
        pv_set(&g_outer[n + 2], l, -1.f, 0.f, oStroke);
        pv_set(&g_outer[n + 3], r, -1.f, 0.f, oStroke);
        pv_mirror(&g_outer[n + 0], r, -0.f, .5f);
        pv_mirror(&g_outer[n + 1], r, -1.f, 0.f);
        pv_mirror(&g_outer[n + 2], l, -0.f, .5f);
        pv_mirror(&g_outer[n + 3], l, -1.f, 0.f);
        n += 4;
    }
    const int ofan = n;
    for (int i = 0; i <= ospan - 1; ++i) /* fan over the 16 curve segments */
        pv_set(&g_outer[n++], (float)i, 0.f, 1.f, (ospan << 2) | FAN_VERTEX);
    static const uint16_t negBorder[6] = {0, 2, 1, 1, 2, 3};
    k = 0;
    e = 0;
    for (int sgm = 0; sgm < ospan; ++sgm)
    {
        for (int i = 0; i < 6; ++i)
            g_outer_idx[k++] = (uint16_t)(e + border[i]);
        e += 4;
    }
    for (int sgm = 0; sgm < ospan; ++sgm)
    {
        for (int i = 0; i < 6; ++i)
            g_outer_idx[k++] = (uint16_t)(e + negBorder[i]);
        e += 4;
    }
    for (int step = 1; step < ospan - 1; step <<= 1)
        for (int i = 0; i < ospan - 1; i += step * 2)
        {
            g_outer_idx[k++] = (uint16_t)(ofan + i);
            g_outer_idx[k++] = (uint16_t)(ofan + i + step);
            g_outer_idx[k++] = (uint16_t)(ofan + i + step * 2);
        }

    /* Center-AA midpoint fan (gpu.cpp:446-687, PatchType::midpointFanCenterAA):
     * the AA ramp centred on the curve (both sides), the middle-out fan and
     * the midpoint triangle; feathered fills draw with it. */
    n = 0;
    for (int i = 0; i < span; ++i) /* top side */
    {
        float l = (float)i, r = l + 1.f;
        pv_set(&g_center[n + 0], l, 0.f, .5f, strokeParams);
        pv_set(&g_center[n + 1], l, 1.f, 0.f, strokeParams);
        pv_set(&g_center[n + 2], r, 0.f, .5f, strokeParams);
        pv_set(&g_center[n + 3], r, 1.f, 0.f, strokeParams);
        pv_mirror(&g_center[n + 0], r - 1.f, 0.f, .5f);
        pv_mirror(&g_center[n + 1], l - 1.f, 0.f, .5f);
        pv_mirror(&g_center[n + 2], r - 1.f, 1.f, 0.f);
        pv_mirror(&g_center[n + 3], l - 1.f, 1.f, 0.f);
        n += 4;
    }
    for (int i = 0; i < span; ++i) /* bottom (negative coverage) side */
    {
        float l = (float)i, r = l + 1.f;
        pv_set(&g_center[n + 0], l, -0.f, .5f, strokeParams);
        pv_set(&g_center[n + 1], r, -0.f, .5f, strokeParams);
        pv_set(&g_center[n + 2], l, -1.f, 0.f, strokeParams);
        pv_set(&g_center[n + 3], r, -1.f, 0.f, strokeParams);
        pv_mirror(&g_center[n + 0], r - 1.f, -0.f, .5f);
        pv_mirror(&g_center[n + 1], r - 1.f, -1.f, 0.f);
        pv_mirror(&g_center[n + 2], l - 1.f, -0.f, .5f);
        pv_mirror(&g_center[n + 3], l - 1.f, -1.f, 0.f);
        n += 4;
    }
    const int cfan = n;
    for (int i = 0; i <= span; ++i)
    {
        pv_set(&g_center[n], (float)i, 0.f, 1.f, (span << 2) | FAN_VERTEX);
        pv_mirror(&g_center[n], (float)i - 1.f, 0.f, 1.f);
        ++n;
    }
    const int cmid = n;
    pv_set(&g_center[n++], 0.f, 0.f, 1.f, (span << 2) | FAN_MIDPOINT_VERTEX);
    k = 0;
    e = 0;
    for (int sgm = 0; sgm < span; ++sgm)
    {
        for (int i = 0; i < 6; ++i)
            g_center_idx[k++] = (uint16_t)(e + border[i]);
        e += 4;
    }
    for (int sgm = 0; sgm < span; ++sgm)
    {
        for (int i = 0; i < 6; ++i)
            g_center_idx[k++] = (uint16_t)(e + negBorder[i]);
        e += 4;
    }
    for (int step = 1; step < span; step <<= 1)
        for (int i = 0; i < span; i += step * 2)
        {
            g_center_idx[k++] = (uint16_t)(cfan + i);
            g_center_idx[k++] = (uint16_t)(cfan + i + step);
            g_center_idx[k++] = (uint16_t)(cfan + i + step * 2);
        }
    g_center_idx[k++] = (uint16_t)cfan;
    g_center_idx[k++] = (uint16_t)(cfan + span);
    g_center_idx[k++] = (uint16_t)cmid;
    g_patch_ready = 1;
}

/* float2x2 from 4 floats: columns (m0, m1) and (m2, m3). */
static inline f2 mat_mul(const float m[4], f2 v)
{
    return (f2){m[0] * v.x + m[2] * v.y, m[1] * v.x + m[3] * v.y};
}

/* draw_path_common.glsl:267-274 */
static float manhattan_pixel_width(const float M[4], f2 normalized)
{
    f2 v = mat_mul(M, normalized);
    return (fabsf(v.x) + fabsf(v.y)) * (1.f / dot2(v, v));
}

typedef struct
{
    f2 pos;
    float cov[4];
    uint32_t pathID;
    int discard;
} vtx_out;

/* unpack_tessellated_path_vertex (draw_path_common.glsl:275-789), for
 * midpointFan patches without feathering, rasterOrdering mode. */
/* pack_feathered_fill_coverages (draw_path_common.glsl:107-149). */
static void pack_feathered_fill_coverages(float cornerTheta, f2 spokeNorm, float outset,
                                          float cov[4])
{
    f2 cornerLocalCoord = {(1.f - spokeNorm.x * fabsf(outset)) * .5f,
                           (1.f - spokeNorm.y * fabsf(outset)) * .5f};
    float cotTheta, y0;
    if (fabsf(cornerTheta - PI_F * .5f) < 1.f / HORIZONTAL_COTANGENT_THRESHOLD)
    {
        cotTheta = 0.f;
        y0 = 0.f;
    }
    else
    {
        float tanTheta = tanf(cornerTheta);
        cotTheta = signf(PI_F * .5f - cornerTheta) /
                   maxf(fabsf(tanTheta), 1.f / HORIZONTAL_COTANGENT_VALUE);
        y0 = cotTheta >= 0.f ? cornerLocalCoord.y - (1.f - cornerLocalCoord.x) * tanTheta
                             : cornerLocalCoord.y + cornerLocalCoord.x * tanTheta;
    }
    cov[0] = maxf(cornerLocalCoord.x, 0.f) + FEATHER_X_COORD_BIAS;
    cov[1] = -cornerLocalCoord.y + FEATHER_COVERAGE_BIAS;
    cov[2] = cotTheta;
    cov[3] = y0;
}

static int patch_vertex_shader(const rive_cuda_flush_desc* d,
                               const oracle_buffers* b,
                               const uint32_t* tess,
                               size_t tessTexels,
                               const patch_vertex* pv,
                               uint32_t instanceID,
                               vtx_out* o)
{
    float localVertexID = pv->localVertexID;
    float outset = pv->outset;
    float fillCoverage = pv->fillCoverage;
    int patchSegmentSpan = pv->params >> 2;
    int vertexType = pv->params & 3;
    int lv = (int)localVertexID;
    int vertexIDOnContour = lv < patchSegmentSpan - 1 ? lv : patchSegmentSpan - 1;
    int64_t tessVertexIdx =
        (int64_t)instanceID * patchSegmentSpan + vertexIDOnContour;
    if (tessVertexIdx < 0 || (size_t)tessVertexIdx >= tessTexels)
        return -1;
    const uint32_t* tv = tess + (size_t)tessVertexIdx * 4;
    uint32_t contourIDWithFlags = tv[3];
    uint32_t contourID = contourIDWithFlags & CONTOUR_ID_MASK;
    if (contourID < 1)
        contourID = 1;
    const uint32_t* cd = contour_record(d, b, contourID);
    if (!cd)
        return -1;
    f2 midpoint = {u2f(cd[0]), u2f(cd[1])};
    uint32_t pathID = cd[2] & 0xffffu;
    uint32_t vertexIndex0 = cd[3];
    const float* path = path_record(d, b, pathID);
    if (!path)
        return -1;
    float M[4] = {path[0], path[1], path[2], path[3]};
    f2 translate = {path[4], path[5]};
    float strokeRadius = path[6];
    float featherRadius = path[7];
    uint32_t mirroredContourFlag =
        contourIDWithFlags & MIRRORED_CONTOUR_CONTOUR_FLAG;
    if (mirroredContourFlag)
    {
        localVertexID = pv->mLocalVertexID;
        outset = pv->mOutset;
        fillCoverage = pv->mFillCoverage;
        lv = (int)localVertexID;
    }
    if (lv != vertexIDOnContour)
    {
        int64_t repl = tessVertexIdx + lv - vertexIDOnContour;
        if (repl < 0 || (size_t)repl >= tessTexels)
            return -1;
        const uint32_t* rv = tess + (size_t)repl * 4;
        if ((rv[3] & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)) !=
            (contourIDWithFlags & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)))
        {
            int isClosed = strokeRadius == 0.f || midpoint.x != 0.f;
            if (isClosed)
            {
                if ((size_t)vertexIndex0 >= tessTexels)
                    return -1;
                tessVertexIdx = vertexIndex0;
                tv = tess + (size_t)vertexIndex0 * 4;
            }
        }
        else
        {
            tessVertexIdx = repl;
            tv = rv;
        }
        contourIDWithFlags =
            (tv[3] & ~MIRRORED_CONTOUR_CONTOUR_FLAG) | mirroredContourFlag;
    }
    float theta;
    float featherJoinEdge0Theta = 0.f, featherJoinCornerTheta = 0.f;
    if ((contourIDWithFlags & JOIN_TYPE_MASK) == FEATHER_JOIN_CONTOUR_FLAG &&
        vertexType == STROKE_VERTEX)
    {
        /* draw_path_common.glsl:372-468: a feather join steps between the
         * tangents of the tessellation vertices just before and after it,
         * backward segments first (to erase coverage outside the corner),
         * then forward ones. */
        uint32_t joinDataPacked = tv[2];
        float joinVertexID = (float)(joinDataPacked & 0xffffu);
        float joinSegmentCount = (float)(joinDataPacked >> 16);
        int off0 = (int)(-joinVertexID - 1.f), off1 = (int)(joinSegmentCount - joinVertexID + 1.f);
        if (contourIDWithFlags & MIRRORED_CONTOUR_CONTOUR_FLAG)
        {
            off0 = -off0;
            off1 = -off1;
        }
        int64_t ib = tessVertexIdx + off0, ia = tessVertexIdx + off1;
        if (ib < 0 || (size_t)ib >= tessTexels || ia < 0 || (size_t)ia >= tessTexels)
            return -1;
        const uint32_t* before = tess + (size_t)ib * 4;
        const uint32_t* after = tess + (size_t)ia * 4;
        if ((after[3] & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)) !=
            (before[3] & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)))
        {
            if ((size_t)vertexIndex0 >= tessTexels)
                return -1;
            after = tess + (size_t)vertexIndex0 * 4;
        }
        featherJoinEdge0Theta = u2f(before[2]);
        float featherJoinEdge1Theta = u2f(after[2]);
        featherJoinCornerTheta = featherJoinEdge1Theta - featherJoinEdge0Theta;
        if (fabsf(featherJoinCornerTheta) > PI_F)
            featherJoinCornerTheta -= TWO_PI_F * signf(featherJoinCornerTheta);
        float nonHelperSegmentCount =
            joinSegmentCount + 1.f - FEATHER_JOIN_HELPER_VERTEX_COUNT;
        float forwardSegmentCount =
            clampf(rintf(fabsf(featherJoinCornerTheta) / PI_F * nonHelperSegmentCount), 1.f,
                   nonHelperSegmentCount - 1.f);
        float backwardSegmentCount = nonHelperSegmentCount - forwardSegmentCount;
        if (joinVertexID <= backwardSegmentCount)
        {
            featherJoinCornerTheta =
                -(PI_F * signf(featherJoinCornerTheta) - featherJoinCornerTheta);
            joinSegmentCount = backwardSegmentCount;
            if (joinVertexID == backwardSegmentCount)
                outset = -outset;
        }
        else if (joinVertexID == backwardSegmentCount + 1.f)
        {
            joinVertexID = 0.f;
            joinSegmentCount = 0.f;
            outset = 0.f;
        }
        else
        {
            joinVertexID -= backwardSegmentCount + 2.f;
            joinSegmentCount = forwardSegmentCount;
        }
        if (joinVertexID == joinSegmentCount)
            theta = featherJoinEdge1Theta;
        else
            theta = featherJoinEdge0Theta +
                    featherJoinCornerTheta * (joinVertexID / joinSegmentCount);
    }
    else
    {
        theta = u2f(tv[2]);
    }
    /* sin and cos here, as everywhere in the passes, are the shared
     * correctly-rounded-operation forms (rive_fp32_math.h) the kernel uses. */
    float normS, normC;
    rc_sincosf(theta, &normS, &normC);
    f2 norm = {normS, -normC};
    f2 origin = {u2f(tv[0]), u2f(tv[1])};
    f2 postTransformVertexOffset = {0.f, 0.f};
    float cov[4] = {0.f, 0.f, 0.f, 0.f};
    o->discard = 0;

    if (featherRadius != 0.f)
    {
        /* draw_path_common.glsl:474-485: never feather harder than 1.5
         * standard deviations across half a pixel. */
        f2 mn = mat_mul(M, norm);
        featherRadius = maxf(featherRadius, (GAUSSIAN_INTEGRAL_TEXTURE_STDDEVS / 3.f) /
                                                sqrtf(dot2(mn, mn)));
    }

    if (strokeRadius != 0.f)
    {
        float detM = M[0] * M[3] - M[2] * M[1];
        outset *= signf(detM);
        if (contourIDWithFlags & LEFT_JOIN_CONTOUR_FLAG)
            outset = minf(outset, 0.f);
        if (contourIDWithFlags & RIGHT_JOIN_CONTOUR_FLAG)
            outset = maxf(outset, 0.f);
        float aaRadius = featherRadius != 0.f ? featherRadius
                                              : manhattan_pixel_width(M, norm) * AA_RADIUS;
        float globalCoverage = 1.f;
        if (aaRadius > strokeRadius && featherRadius == 0.f)
        {
            globalCoverage = strokeRadius / aaRadius;
            strokeRadius = aaRadius;
        }
        f2 vertexOffset = mul2(norm, strokeRadius + aaRadius);
        float x = outset * (strokeRadius + aaRadius);
        float k = 1.f / (aaRadius * 2.f);
        cov[0] = k * (x + strokeRadius) + .5f;
        cov[1] = k * (-x + strokeRadius) + .5f;
        uint32_t joinType = contourIDWithFlags & JOIN_TYPE_MASK;
        if (joinType > ROUND_JOIN_CONTOUR_FLAG)
        {
            int peekDir = 2;
            if (!(contourIDWithFlags & JOIN_TANGENT_0_CONTOUR_FLAG))
                peekDir = -peekDir;
            if (contourIDWithFlags & MIRRORED_CONTOUR_CONTOUR_FLAG)
                peekDir = -peekDir;
            int64_t other = tessVertexIdx + peekDir;
            if (other < 0 || (size_t)other >= tessTexels)
                return -1;
            float otherJoinTheta = u2f(tess[(size_t)other * 4 + 2]);
            float joinAngle = fabsf(otherJoinTheta - theta);
            if (joinAngle > PI_F)
                joinAngle = TWO_PI_F - joinAngle;
            int isTan0 = (contourIDWithFlags & JOIN_TANGENT_0_CONTOUR_FLAG) != 0;
            int isLeftJoin = (contourIDWithFlags & LEFT_JOIN_CONTOUR_FLAG) != 0;
            float bisectTheta =
                joinAngle * (isTan0 == isLeftJoin ? -.5f : .5f) + theta;
            float bisS, bisC;
            rc_sincosf(bisectTheta, &bisS, &bisC);
            f2 bisector = {bisS, -bisC};
            float bisectPixelWidth = manhattan_pixel_width(M, bisector);
            float miterRatio = rc_cosf(joinAngle * .5f);
            float clipRadius;
            if (joinType == MITER_CLIP_JOIN_CONTOUR_FLAG ||
                (joinType == MITER_REVERT_JOIN_CONTOUR_FLAG && miterRatio >= .25f))
            {
                float miterInverseLimit =
                    (contourIDWithFlags & EMULATED_STROKE_CAP_CONTOUR_FLAG) ? 1.f
                                                                             : .25f;
                clipRadius = strokeRadius * (1.f / maxf(miterRatio, miterInverseLimit));
            }
            else
            {
                clipRadius = strokeRadius * miterRatio + bisectPixelWidth * .5f;
            }
            float clipAARadius = clipRadius + bisectPixelWidth * AA_RADIUS;
            if (contourIDWithFlags & JOIN_TANGENT_INNER_CONTOUR_FLAG)
            {
                float strokeAARaidus = strokeRadius + aaRadius;
                float slop = aaRadius * .125f;
                if (strokeAARaidus <= clipAARadius * miterRatio + slop)
                {
                    float miterAARadius = strokeAARaidus * (1.f / miterRatio);
                    vertexOffset = mul2(bisector, miterAARadius);
                }
                else
                {
                    f2 bisectAAOffset = mul2(bisector, clipAARadius);
                    f2 kk = {dot2(vertexOffset, vertexOffset),
                             dot2(bisectAAOffset, bisectAAOffset)};
                    /* MUL(k, inverse(float2x2(vertexOffset, bisectAAOffset)))
                     * = row vector k times the inverse of the matrix whose
                     * columns are vertexOffset and bisectAAOffset. */
                    float a = vertexOffset.x, bb = vertexOffset.y;
                    float c = bisectAAOffset.x, dd = bisectAAOffset.y;
                    /* inverse() as the reference's own polyfills define it:
                     * the adjoint times 1 / determinant (hlsl.glsl:378-382,
                     * metal.glsl:509-514). */
                    float det = a * dd - c * bb;
                    float invDet = 1.f / det;
                    float inv00 = dd * invDet, inv01 = -bb * invDet; /* column 0 */
                    float inv10 = -c * invDet, inv11 = a * invDet;   /* column 1 */
                    vertexOffset.x = kk.x * inv00 + kk.y * inv01;
                    vertexOffset.y = kk.x * inv10 + kk.y * inv11;
                }
            }
            f2 pt = mul2(vertexOffset, fabsf(outset));
            float clipDistance = (clipAARadius - dot2(pt, bisector)) /
                                 (bisectPixelWidth * (AA_RADIUS * 2.f));
            if (contourIDWithFlags & LEFT_JOIN_CONTOUR_FLAG)
                cov[1] = clipDistance;
            else
                cov[0] = clipDistance;
        }
        cov[0] *= globalCoverage;
        cov[1] *= globalCoverage;
        cov[1] = maxf(cov[1], 1e-4f);
        if (featherRadius != 0.f)
            cov[0] = FEATHER_COVERAGE_BIAS - cov[0]; /* marks a feathered stroke */
        postTransformVertexOffset = mat_mul(M, mul2(vertexOffset, outset));
        if (vertexType != STROKE_VERTEX)
            o->discard = 1;
    }
    else
    {
        cov[0] = fillCoverage;
        cov[1] = -1.f;
        if (featherRadius != 0.f)
        {
            /* draw_path_common.glsl:659-741: a feathered edge; the spokes of
             * a feather join carry their corner. */
            cov[1] = FEATHER_COVERAGE_BIAS;
            cov[2] = HORIZONTAL_COTANGENT_VALUE;
            cov[3] = fillCoverage;
            if ((contourIDWithFlags & JOIN_TYPE_MASK) == FEATHER_JOIN_CONTOUR_FLAG &&
                vertexType == STROKE_VERTEX)
            {
                if (featherJoinCornerTheta < 0.f)
                {
                    featherJoinEdge0Theta += featherJoinCornerTheta;
                    featherJoinCornerTheta = -featherJoinCornerTheta;
                }
                float spokeTheta = theta - featherJoinEdge0Theta;
                spokeTheta = glsl_mod(spokeTheta + PI_F * .5f, TWO_PI_F) - PI_F * .5f;
                spokeTheta = clampf(spokeTheta, 0.f, featherJoinCornerTheta);
                if (spokeTheta > featherJoinCornerTheta * .5f)
                    spokeTheta = featherJoinCornerTheta - spokeTheta;
                float spokeS, spokeC;
                rc_sincosf(spokeTheta, &spokeS, &spokeC);
                f2 spokeNorm = {spokeS, spokeC};
                pack_feathered_fill_coverages(featherJoinCornerTheta, spokeNorm, outset, cov);
            }
            postTransformVertexOffset = mat_mul(M, mul2(norm, outset * featherRadius));
        }
        else
        {
            /* sign(MUL(outset * norm, inverse(M))) * AA_RADIUS: row vector
             * times the inverse matrix. */
            f2 on = mul2(norm, outset);
            float det = M[0] * M[3] - M[2] * M[1];
            float invDet = 1.f / det; /* inverse() = adjoint * (1 / det) */
            float i00 = M[3] * invDet, i01 = -M[1] * invDet; /* column 0 of inverse */
            float i10 = -M[2] * invDet, i11 = M[0] * invDet; /* column 1 of inverse */
            f2 r = {on.x * i00 + on.y * i01, on.x * i10 + on.y * i11};
            postTransformVertexOffset = (f2){signf(r.x) * AA_RADIUS, signf(r.y) * AA_RADIUS};
        }
        if (((contourIDWithFlags & MIRRORED_CONTOUR_CONTOUR_FLAG) != 0) !=
            ((contourIDWithFlags & NEGATE_PATH_FILL_COVERAGE_FLAG) != 0))
            cov[0] = -cov[0];
        if (vertexType == FAN_MIDPOINT_VERTEX)
            origin = midpoint;
        if ((contourIDWithFlags & RETROFIT_TRI_STRIP_CONTOUR_FLAG) &&
            vertexType != FAN_VERTEX)
            o->discard = 1;
    }
    if (d->wireframe)
    {
        cov[0] = 1.f;
        cov[1] = -1.f;
    }
    f2 mo = mat_mul(M, origin);
    o->pos = add2(add2(mo, postTransformVertexOffset), translate);
    o->cov[0] = cov[0];
    o->cov[1] = cov[1];
    o->cov[2] = cov[2];
    o->cov[3] = cov[3];
    o->pathID = pathID;
    return 0;
}

typedef struct
{
    int64_t x[3], y[3]; /* fixed point, SUBPIXEL_BITS */
    float cov[3][4];
    uint32_t pathID;
    uint32_t features;
    int32_t bx0, by0, bx1, by1; /* pixel bbox, inclusive-exclusive */
    int interior; /* an interior-triangulation triangle (DRAW_INTERIOR_TRIANGLES) */
    int blit;     /* a featherAtlasBlit triangle: coverage sampled from the atlas */
    int negate;   /* an atlas fill triangle that faced away: coverage negated */
    const oracle_texture* image; /* the batch's image (NULL: none) */
    uint32_t sampler;            /* its ImageSampler key */
    /* An image-mesh triangle: its texture-coordinate planes (u0, du/dx,
     * du/dy, v0, dv/dx, dv/dy, anchor x, anchor y), ImageDrawInstance and
     * mip level. */
    int mesh;
    float planes[8];
    uint32_t imageDraw;
    int level;
} tri_rec;

static inline int64_t snap(float v)
{
    return (int64_t)llrint((double)v * SUBPIXEL_ONE);
}

/* PLS state of one pixel (draw_raster_order_path.frag:7-12). */
typedef struct
{
    uint8_t color[4];
    uint32_t clip;
    uint8_t scratch[4];
    uint32_t coverage;
} pls_pixel;

static inline uint16_t id_bits_to_f16(uint32_t idBits, uint32_t granularity)
{
    return idBits == 0 ? 0 : (uint16_t)((idBits + MAX_DENORM_F16) * granularity);
}
static inline float h2f(uint16_t h) { return oracle_f16_to_f32(h); }

/* ---- Feather lookup table ------------------------------------------------
 * The integral of the normal distribution over -3..+3 standard deviations in
 * 512 fp16 entries, the R16F texture the feather passes sample with a linear
 * filter (constants.glsl:19-26, gpu.hpp:2083-2091). Restated from its
 * generator (renderer/src/gpu.cpp:1983-2062): 7 samples per entry of the
 * normal distribution, shifted so the middle is exactly 1/2, made monotonic
 * and clamped to [0, 1], with an 8-entry ease to 0 and 1 at the ends. */
static uint16_t g_feather16[GAUSSIAN_TABLE_SIZE];
static float g_feather[GAUSSIAN_TABLE_SIZE];
static int g_featherReady;

static float eval_normal_distribution(float x, float mu, float inverseSigma)
{
    const float ONE_OVER_SQRT_2_PI = 0.398942280401433f;
    float y = (x - mu) * inverseSigma;
    return expf(-.5 * y * y) * inverseSigma * ONE_OVER_SQRT_2_PI;
}

static void build_feather_table(void)
{
    if (g_featherReady)
        return;
    float table[GAUSSIAN_TABLE_SIZE];
    float sigma = GAUSSIAN_TABLE_SIZE / (GAUSSIAN_INTEGRAL_TEXTURE_STDDEVS * 2);
    float inverseSigma = 1 / sigma;
    float mu = GAUSSIAN_TABLE_SIZE * .5f;
    float integral = 0;
    for (int i = 0; i < GAUSSIAN_TABLE_SIZE; ++i)
    {
        const int SAMPLES = 7;
        float barCenterX = (float)i;
        for (int sample = 0; sample < SAMPLES; ++sample)
        {
            float dx = (float)(sample - (SAMPLES >> 1)) / SAMPLES;
            integral += eval_normal_distribution(barCenterX + dx, mu, inverseSigma) / SAMPLES;
        }
        table[i] = integral;
    }
    float shift = .5 - (table[GAUSSIAN_TABLE_SIZE / 2 - 1] + table[GAUSSIAN_TABLE_SIZE / 2]) / 2;
    table[0] = fminf(fmaxf(0, table[0] + shift), 1);
    for (int i = 1; i < GAUSSIAN_TABLE_SIZE; ++i)
        table[i] = fminf(fmaxf(table[i - 1], table[i] + shift), 1);
    const int EASE = 8;
    for (int i = 0; i < GAUSSIAN_TABLE_SIZE; ++i)
    {
        if (i < EASE)
            table[i] *= (float)i / (float)EASE;
        if (i > (GAUSSIAN_TABLE_SIZE - EASE) - 1)
        {
            float diffToOne = 1.0 - table[i];
            float fi = (float)(i - (GAUSSIAN_TABLE_SIZE - EASE) + 1) / (float)EASE;
            table[i] = table[i] + (diffToOne * fi);
        }
    }
    for (int i = 0; i < GAUSSIAN_TABLE_SIZE; ++i)
    {
        g_feather16[i] = oracle_f32_to_f16(table[i]);
        g_feather[i] = oracle_f16_to_f32(g_feather16[i]);
    }
    build_inverse_feather_table();
    g_featherReady = 1;
}

void oracle_feather_table(uint16_t* out)
{
    build_feather_table();
    memcpy(out, g_feather16, sizeof(g_feather16));
}


/* FEATHER(x) (common.glsl:53-60): the table sampled at normalised x with a
 * linear filter and clamp-to-edge addressing. */
static float feather_lut(float x)
{
    float t = x * GAUSSIAN_TABLE_SIZE - .5f;
    if (!(t == t))
        return g_feather[0];
    float f = floorf(t);
    float w = t - f;
    float fc = fminf(fmaxf(f, -1.f), (float)GAUSSIAN_TABLE_SIZE);
    int i0 = (int)fc;
    int a = i0 < 0 ? 0 : (i0 > GAUSSIAN_TABLE_SIZE - 1 ? GAUSSIAN_TABLE_SIZE - 1 : i0);
    int b = i0 + 1 < 0 ? 0 : (i0 + 1 > GAUSSIAN_TABLE_SIZE - 1 ? GAUSSIAN_TABLE_SIZE - 1 : i0 + 1);
    return g_feather[a] + (g_feather[b] - g_feather[a]) * w;
}

/* eval_feathered_stroke (draw_path_common.glsl:242-258):
 * 1 - feather(1 - leftCoverage) - feather(1 - rightCoverage), with the left
 * coverage carried biased by FEATHER_COVERAGE_BIAS. */
static uint16_t g_inverse16[GAUSSIAN_TABLE_SIZE];
static float g_inverse[GAUSSIAN_TABLE_SIZE];

/* The inverse table (renderer/src/gpu.cpp:2125-2190, restated): 32 samples per
 * entry of the running integral; each cell holds the height at which the
 * integral crosses the cell's centre, the middle cell exactly 1/2. */
static void build_inverse_feather_table(void)
{
    float table[GAUSSIAN_TABLE_SIZE];
    memset(table, 0, sizeof(table));
    const size_t MULTIPLIER = 32;
    float sigma = GAUSSIAN_TABLE_SIZE / (GAUSSIAN_INTEGRAL_TEXTURE_STDDEVS * 2);
    float inverseSigma = 1 / sigma;
    float mu = GAUSSIAN_TABLE_SIZE * .5f;
    size_t samples = GAUSSIAN_TABLE_SIZE * MULTIPLIER;
    float integral = 0;
    for (size_t i = 0; i < (samples + 1) / 2; ++i)
    {
        float barCenterX = (float)i / MULTIPLIER;
        integral += eval_normal_distribution(barCenterX, mu, inverseSigma) / MULTIPLIER;
    }
    integral = .5 - integral;
    float lastInverseX = NAN, lastInverseY = 0;
    table[0] = 0;
    table[GAUSSIAN_TABLE_SIZE - 1] = 1;
    for (size_t i = 0; i < samples; ++i)
    {
        float barCenterX = (float)i / MULTIPLIER;
        integral += eval_normal_distribution(barCenterX, mu, inverseSigma) / MULTIPLIER;
        float inverseX = fminf(fmaxf(0, integral), 1) * GAUSSIAN_TABLE_SIZE;
        float inverseY = (i + .5f) / samples;
        size_t cell = (size_t)inverseX;
        float cellCenterX = cell + .5f;
        if (cellCenterX == mu)
        {
            table[cell] = .5f;
        }
        else if (lastInverseX <= cellCenterX && inverseX >= cellCenterX)
        {
            float t = (cellCenterX - lastInverseX) / (inverseX - lastInverseX);
            float y = lastInverseY + (inverseY - lastInverseY) * t;
            if (cell < GAUSSIAN_TABLE_SIZE)
                table[cell] = y;
        }
        lastInverseX = inverseX;
        lastInverseY = inverseY;
    }
    for (int i = 0; i < GAUSSIAN_TABLE_SIZE; ++i)
    {
        g_inverse16[i] = oracle_f32_to_f16(table[i]);
        g_inverse[i] = oracle_f16_to_f32(g_inverse16[i]);
    }
}

void oracle_inverse_feather_table(uint16_t* out)
{
    build_feather_table();
    memcpy(out, g_inverse16, sizeof(g_inverse16));
}

/* INVERSE_FEATHER(x) (common.glsl:61-68): layer 1 of the same 1D array
 * texture, sampled the same way. */
static float inverse_feather_lut(float x)
{
    float t = x * GAUSSIAN_TABLE_SIZE - .5f;
    if (!(t == t))
        return g_inverse[0];
    float f = floorf(t);
    float w = t - f;
    float fc = fminf(fmaxf(f, -1.f), (float)GAUSSIAN_TABLE_SIZE);
    int i0 = (int)fc;
    int a = i0 < 0 ? 0 : (i0 > GAUSSIAN_TABLE_SIZE - 1 ? GAUSSIAN_TABLE_SIZE - 1 : i0);
    int b = i0 + 1 < 0 ? 0 : (i0 + 1 > GAUSSIAN_TABLE_SIZE - 1 ? GAUSSIAN_TABLE_SIZE - 1 : i0 + 1);
    return g_inverse[a] + (g_inverse[b] - g_inverse[a]) * w;
}

/* eval_feathered_fill (draw_path_common.glsl:152-240): the feather of a flat
 * edge, or of a corner through a 4-sample integral of the second edge. */
static float eval_feathered_fill(float cx, float cy, float cz, float cw)
{
    float cotTheta = cz;
    float y0 = maxf(cw, 0.f);
    float featherCoverage = cotTheta >= 0.f ? feather_lut(y0) : 0.f;
    if (fabsf(cotTheta) < HORIZONTAL_COTANGENT_THRESHOLD)
    {
        float x = fabsf(cx) - FEATHER_X_COORD_BIAS;
        float y = -cy + FEATHER_COVERAGE_BIAS;
        float dt = (y - y0) * 0.5984134206f;
        static const float k[4] = {0.20888568955f, 0.62665706865f, 1.04442844776f,
                                   1.46219982687f};
        float sum = 0.f;
        for (int i = 0; i < 4; ++i)
        {
            float t = y0 + dt * k[i];
            float u = t * -cotTheta + (y * cotTheta + x);
            float t_ = t * 5.09593080173f + -2.54796540086f;
            float ddt = exp2f(-t_ * t_);
            sum += feather_lut(u) * ddt;
        }
        featherCoverage += sum * dt;
    }
    return featherCoverage * signf(cx);
}

static float eval_feathered_stroke(float covx, float covy)
{
    float featherCoverage = 1.f;
    float leftOutsideCoverage = (1.f - FEATHER_COVERAGE_BIAS) + covx;
    featherCoverage -= feather_lut(leftOutsideCoverage);
    float rightOutsideCoverage = 1.f - covy;
    featherCoverage -= feather_lut(rightOutsideCoverage);
    return featherCoverage;
}

/* advanced_blend.glsl:94-154 */
static float lum_from_rgb(const float c[3])
{
    return c[0] * .30f + c[1] * .59f + c[2] * .11f;
}
static float min3(const float c[3]) { return minf(minf(c[0], c[1]), c[2]); }
static float max3(const float c[3]) { return maxf(maxf(c[0], c[1]), c[2]); }
static void set_lum(const float base[3], const float lumColor[3], float out[3])
{
    float lumTarget = lum_from_rgb(lumColor);
    float lb = lum_from_rgb(base);
    float biased[3] = {base[0] - lb, base[1] - lb, base[2] - lb};
    float sx = lumTarget / maxf(EPSILON_FP16_NON_DENORM, -min3(biased));
    float sy = (1.f - lumTarget) / maxf(EPSILON_FP16_NON_DENORM, max3(biased));
    float satScale = minf(1.f, minf(sx, sy));
    for (int i = 0; i < 3; ++i)
        out[i] = biased[i] * satScale + lumTarget;
}
static void set_lum_sat(const float hue[3],
                        const float sat[3],
                        const float lum[3],
                        float out[3])
{
    float satTarget = max3(sat) - min3(sat);
    float mn = min3(hue);
    float h[3] = {hue[0] - mn, hue[1] - mn, hue[2] - mn};
    float satSource = max3(h);
    float scale = satTarget / maxf(EPSILON_FP16_NON_DENORM, satSource);
    float hs[3] = {h[0] * scale, h[1] * scale, h[2] * scale};
    set_lum(hs, lum, out);
}

/* advanced_blend_coeffs (advanced_blend.glsl:156-301). */
void oracle_advanced_blend_coeffs(const float srcIn[3],
                                  const float dstPremulIn[4],
                                  int mode,
                                  float co[3])
{
    float src[3] = {srcIn[0], srcIn[1], srcIn[2]};
    float dp[4] = {dstPremulIn[0], dstPremulIn[1], dstPremulIn[2], dstPremulIn[3]};
    float inv = dp[3] != 0.f ? 1.f / dp[3] : 0.f;
    float dst[3] = {dp[0] * inv, dp[1] * inv, dp[2] * inv};
    co[0] = co[1] = co[2] = 0.f;
    switch (mode)
    {
        case BLEND_MODE_MULTIPLY:
            for (int i = 0; i < 3; ++i)
                co[i] = src[i] * dst[i];
            break;
        case BLEND_MODE_SCREEN:
            for (int i = 0; i < 3; ++i)
                co[i] = src[i] + dst[i] - src[i] * dst[i];
            break;
        case BLEND_MODE_OVERLAY:
            for (int i = 0; i < 3; ++i)
            {
                float sd = src[i] * dst[i];
                co[i] = 2.f * (dst[i] > .5f ? src[i] + dst[i] - sd - .5f : sd);
            }
            break;
        case BLEND_MODE_DARKEN:
            for (int i = 0; i < 3; ++i)
                co[i] = minf(src[i], dst[i]);
            break;
        case BLEND_MODE_LIGHTEN:
            for (int i = 0; i < 3; ++i)
                co[i] = maxf(src[i], dst[i]);
            break;
        case BLEND_MODE_COLORDODGE:
            for (int i = 0; i < 3; ++i)
            {
                float dpc = clampf(dp[i], 0.f, dp[3]);
                float denom = clampf(1.f - src[i], 0.f, 1.f) * dp[3];
                co[i] = denom == 0.f ? signf(dpc) : minf(1.f, dpc / denom);
            }
            break;
        case BLEND_MODE_COLORBURN:
        {
            float a = dp[3] == 0.f ? 1.f : dp[3];
            for (int i = 0; i < 3; ++i)
            {
                float s = clampf(src[i], 0.f, 1.f);
                float dpc = clampf(dp[i], 0.f, dp[3]);
                float numer = a - dpc;
                co[i] = 1.f - (s == 0.f ? signf(numer) : minf(1.f, numer / (s * a)));
            }
            break;
        }
        case BLEND_MODE_HARDLIGHT:
            for (int i = 0; i < 3; ++i)
            {
                float sd = src[i] * dst[i];
                co[i] = 2.f * (src[i] > .5f ? src[i] + dst[i] - sd - .5f : sd);
            }
            break;
        case BLEND_MODE_SOFTLIGHT:
            for (int i = 0; i < 3; ++i)
            {
                float c;
                if (src[i] <= .5f)
                    c = 1.f - dst[i];
                else if (dst[i] <= .25f)
                    c = (16.f * dst[i] - 12.f) * dst[i] + 3.f;
                else
                    c = 1.f / sqrtf(dst[i]) - 1.f;
                co[i] = dst[i] + dst[i] * (2.f * src[i] - 1.f) * c;
            }
            break;
        case BLEND_MODE_DIFFERENCE:
            for (int i = 0; i < 3; ++i)
                co[i] = fabsf(dst[i] - src[i]);
            break;
        case BLEND_MODE_EXCLUSION:
            for (int i = 0; i < 3; ++i)
                co[i] = src[i] + dst[i] - 2.f * src[i] * dst[i];
            break;
        case BLEND_MODE_HUE:
        case BLEND_MODE_SATURATION:
        case BLEND_MODE_COLOR:
        case BLEND_MODE_LUMINOSITY:
        {
            float s[3];
            for (int i = 0; i < 3; ++i)
                s[i] = clampf(src[i], 0.f, 1.f);
            if (mode == BLEND_MODE_HUE)
                set_lum_sat(s, dst, dst, co);
            else if (mode == BLEND_MODE_SATURATION)
                set_lum_sat(dst, s, dst, co);
            else if (mode == BLEND_MODE_COLOR)
                set_lum(s, dst, co);
            else
                set_lum(dst, s, co);
            break;
        }
        default:
            break;
    }
}

/* advanced_color_blend (advanced_blend.glsl:303-327). */
void oracle_advanced_blend(const float srcIn[3],
                           const float dstPremulIn[4],
                           int mode,
                           float out[3])
{
    float co[3];
    oracle_advanced_blend_coeffs(srcIn, dstPremulIn, mode, co);
    /* mix(src, coeffs, dstPremul.a) = src * (1 - a) + coeffs * a, with the
     * caller's (unclamped) src: advanced_blend_coeffs takes src by value. */
    float a = dstPremulIn[3];
    for (int i = 0; i < 3; ++i)
        out[i] = srcIn[i] * (1.f - a) + co[i] * a;
}

/* Bilinear sample of the RGBA8 gradient texture with clamp-to-edge. */
static void sample_grad(const uint8_t* grad,
                        uint32_t H,
                        uint32_t textureH,
                        float u,
                        float v,
                        float out[4])
{
    /* Normalised coordinates address the whole allocated texture (textureH
     * rows); only the first H rows hold ramps. */
    float fx = u * GRAD_TEXTURE_WIDTH - .5f;
    float fy = v * (float)textureH - .5f;
    float x0f = floorf(fx), y0f = floorf(fy);
    float ax = fx - x0f, ay = fy - y0f;
    int x0 = (int)x0f, y0 = (int)y0f;
    for (int k = 0; k < 4; ++k)
        out[k] = 0.f;
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i)
        {
            int xi = x0 + i, yj = y0 + j;
            xi = xi < 0 ? 0 : (xi >= GRAD_TEXTURE_WIDTH ? GRAD_TEXTURE_WIDTH - 1 : xi);
            yj = yj < 0 ? 0 : (yj >= (int)H ? (int)H - 1 : yj);
            float w = (i ? ax : 1.f - ax) * (j ? ay : 1.f - ay);
            const uint8_t* t = grad + ((size_t)yj * GRAD_TEXTURE_WIDTH + xi) * 4;
            for (int k = 0; k < 4; ++k)
                out[k] += w * ((float)t[k] / 255.f);
        }
}

/* common.glsl:269-274 */
static float ign(float fx, float fy, float scale, float bias)
{
    float v1 = fractf(0.06711056f * fx + 0.00583715f * fy);
    float v2 = fractf(52.9829189f * v1);
    return v2 * scale + bias;
}

typedef struct
{
    const rive_cuda_flush_desc* d;
    const oracle_buffers* b;
    const uint8_t* grad;
    uint32_t granularity;
    float ditherScale, ditherBias;
    /* The feather atlas the flush rendered first (fp16 values held as
     * floats), atlasW x atlasH texels; NULL without atlas draws. */
    const float* atlas;
    int atlasW, atlasH;
} frag_ctx;

/* ---- Images ----------------------------------------------------------- */

int oracle_texture_prepare(oracle_texture* t)
{
    if (!t || !t->rgba || t->width == 0 || t->height == 0 || t->levels == 0 || t->levels > 16)
        return -1;
    uint32_t total = 0;
    for (uint32_t l = 0; l < t->levels; ++l)
    {
        uint32_t w = t->width >> l, h = t->height >> l;
        t->off[l] = total;
        total += (w ? w : 1) * (h ? h : 1);
    }
    t->mips = (uint8_t*)malloc((size_t)total * 4);
    if (!t->mips)
        return -4;
    memcpy(t->mips, t->rgba, (size_t)t->width * t->height * 4);
    for (uint32_t l = 1; l < t->levels; ++l)
    {
        uint32_t sw = t->width >> (l - 1), sh = t->height >> (l - 1);
        uint32_t dw = t->width >> l, dh = t->height >> l;
        sw = sw ? sw : 1;
        sh = sh ? sh : 1;
        dw = dw ? dw : 1;
        dh = dh ? dh : 1;
        const uint8_t* src = t->mips + (size_t)t->off[l - 1] * 4;
        uint8_t* dst = t->mips + (size_t)t->off[l] * 4;
        for (uint32_t y = 0; y < dh; ++y)
            for (uint32_t x = 0; x < dw; ++x)
            {
                uint32_t x0 = 2 * x < sw - 1 ? 2 * x : sw - 1;
                uint32_t x1 = 2 * x + 1 < sw - 1 ? 2 * x + 1 : sw - 1;
                uint32_t y0 = 2 * y < sh - 1 ? 2 * y : sh - 1;
                uint32_t y1 = 2 * y + 1 < sh - 1 ? 2 * y + 1 : sh - 1;
                for (int k = 0; k < 4; ++k)
                {
                    uint32_t sum = src[((size_t)y0 * sw + x0) * 4 + k] +
                                   src[((size_t)y0 * sw + x1) * 4 + k] +
                                   src[((size_t)y1 * sw + x0) * 4 + k] +
                                   src[((size_t)y1 * sw + x1) * 4 + k];
                    dst[((size_t)y * dw + x) * 4 + k] = (uint8_t)((sum + 2) >> 2);
                }
            }
    }
    return 0;
}

void oracle_texture_release(oracle_texture* t)
{
    if (t)
    {
        free(t->mips);
        t->mips = NULL;
    }
}

/* A texel address under a wrap mode: the Vulkan sampler address modes the
 * reference maps ImageWrap to (pipeline_manager_vulkan.cpp:25-38). */
static int wrap_texel(int i, int n, uint32_t wrap)
{
    if (wrap == 1) /* repeat */
    {
        i %= n;
        return i < 0 ? i + n : i;
    }
    if (wrap == 2) /* mirrored repeat */
    {
        int m = i % (2 * n);
        if (m < 0)
            m += 2 * n;
        int a = m - n;
        return (n - 1) - (a >= 0 ? a : -(1 + a));
    }
    return i < 0 ? 0 : (i > n - 1 ? n - 1 : i); /* clamp to edge */
}

/* The image at normalised (u, v) with an explicit level of detail: nearest
 * mip selection (VK_SAMPLER_MIPMAP_MODE_NEAREST: level ceil(lod + 1/2) - 1
 * above 1/2, else 0), the sampler's filter within the level. */
static void sample_image_level(const oracle_texture* t, uint32_t sampler, int level, float u,
                               float v, float out[4])
{
    const uint32_t wrapX = sampler % 3u, wrapY = (sampler / 3u) % 3u;
    const int nearest = sampler >= 9u;
    int w = (int)(t->width >> level), h = (int)(t->height >> level);
    w = w ? w : 1;
    h = h ? h : 1;
    const uint8_t* tex = t->mips + (size_t)t->off[level] * 4;
    if (nearest)
    {
        int x = wrap_texel((int)floorf(u * (float)w), w, wrapX);
        int y = wrap_texel((int)floorf(v * (float)h), h, wrapY);
        for (int k = 0; k < 4; ++k)
            out[k] = (float)tex[((size_t)y * w + x) * 4 + k] / 255.f;
        return;
    }
    float fx = u * (float)w - .5f, fy = v * (float)h - .5f;
    float x0f = floorf(fx), y0f = floorf(fy);
    float ax = fx - x0f, ay = fy - y0f;
    int x0 = (int)x0f, y0 = (int)y0f;
    for (int k = 0; k < 4; ++k)
        out[k] = 0.f;
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i)
        {
            int xi = wrap_texel(x0 + i, w, wrapX), yj = wrap_texel(y0 + j, h, wrapY);
            float wgt = (i ? ax : 1.f - ax) * (j ? ay : 1.f - ay);
            for (int k = 0; k < 4; ++k)
                out[k] += wgt * ((float)tex[((size_t)yj * w + xi) * 4 + k] / 255.f);
        }
}

static void sample_image(const oracle_texture* t, uint32_t sampler, float u, float v, float lod,
                         float out[4])
{
    int level = 0;
    if (lod > .5f)
    {
        level = (int)ceilf(lod + .5f) - 1;
        if (level > (int)t->levels - 1)
            level = (int)t->levels - 1;
    }
    sample_image_level(t, sampler, level, u, v, out);
}

/* ---- Image meshes (draw_image_mesh.vert, draw_mesh.frag) ----------------- */

static float clip_rect_distance(const float* aux, float fragX, float fragY);

/* The mip level of an image-mesh triangle: the implicit level of detail plus
 * FlushUniforms::mipMapLODBias under the Vulkan rules (lambda = log2(rho) +
 * bias, rho the larger texel-space length of d(uv)/dx and d(uv)/dy, clamped
 * to [0, levels - 1]; nearest mip ceil(lambda + 1/2) - 1). Level k is reached
 * when rho^2 > 2^(2k - 1 - 2 bias), a power-of-two comparison (bias taken to
 * the nearest half-integer; the reference's is -1/2). */
static int mesh_mip_level(float rho2, float bias, uint32_t levels)
{
    const int twoBias = (int)rintf(2.f * bias);
    int level = 0;
    for (uint32_t k = 1; k < levels; ++k)
    {
        if (!(rho2 > ldexpf(1.f, 2 * (int)k - 1 - twoBias)))
            break;
        level = (int)k;
    }
    return level;
}

int oracle_mesh_mip_level(float rho2, float bias, uint32_t levels)
{
    return mesh_mip_level(rho2, bias, levels);
}

/* The texture-coordinate planes of a set-up mesh triangle (vertex order after
 * the two-sided turn), anchored at its first snapped vertex, and its mip
 * level for `tex`: texture coordinates are affine over the triangle, so the
 * derivatives the implicit level of detail uses are the planes' slopes. */
static void mesh_planes(tri_rec* t, const oracle_texture* tex, float bias)
{
    const float s = 1.f / 256.f;
    const float p0x = (float)t->x[0] * s, p0y = (float)t->y[0] * s;
    const float p1x = (float)t->x[1] * s, p1y = (float)t->y[1] * s;
    const float p2x = (float)t->x[2] * s, p2y = (float)t->y[2] * s;
    const int64_t area2 = (t->x[1] - t->x[0]) * (t->y[2] - t->y[0]) -
                          (t->x[2] - t->x[0]) * (t->y[1] - t->y[0]);
    const float d1x = p1x - p0x, d1y = p1y - p0y;
    const float d2x = p2x - p0x, d2y = p2y - p0y;
    const float inv = 1.f / ((float)area2 * (s * s));
    const float uA = t->cov[0][0], uB = t->cov[1][0], uC = t->cov[2][0];
    const float vA = t->cov[0][1], vB = t->cov[1][1], vC = t->cov[2][1];
    const float ugx = ((uB - uA) * d2y - (uC - uA) * d1y) * inv;
    const float ugy = ((uC - uA) * d1x - (uB - uA) * d2x) * inv;
    const float vgx = ((vB - vA) * d2y - (vC - vA) * d1y) * inv;
    const float vgy = ((vC - vA) * d1x - (vB - vA) * d2x) * inv;
    const float pl[8] = {uA, ugx, ugy, vA, vgx, vgy, p0x, p0y};
    memcpy(t->planes, pl, sizeof(pl));
    const float W = (float)tex->width, H = (float)tex->height;
    const float ux = ugx * W, vx = vgx * H, uy = ugy * W, vy = vgy * H;
    const float rho2 = maxf(ux * ux + vx * vx, uy * uy + vy * vy);
    t->level = mesh_mip_level(rho2, bias, tex->levels);
}

/* One fragment of an image-mesh triangle (draw_mesh.frag:60-225 with
 * DRAW_IMAGE_MESH): the image at the pixel's texture coordinates and the
 * triangle's mip level, coverage 1 cut by the clip rect and the clip, times
 * the opacity; advanced blending unmultiplies the texel; dither, then
 * src-over, straight into the colour plane. */
static void mesh_fragment(const frag_ctx* fc, const tri_rec* t, int px, int py, pls_pixel* pls)
{
    const uint32_t features = t->features;
    const float fragX = (float)px + .5f, fragY = (float)py + .5f;
    const float* pl = t->planes;
    const float dx = fragX - pl[6], dy = fragY - pl[7];
    const float u = (pl[0] + pl[1] * dx) + pl[2] * dy;
    const float v = (pl[3] + pl[4] * dx) + pl[5] * dy;
    float color[4];
    sample_image_level(t->image, t->sampler, t->level, u, v, color);
    /* ImageDrawInstance (gpu.hpp:1742-1774): view matrix, clip-rect inverse
     * matrix, translates, then opacity, clip ID, blend mode, z index. */
    const float* inst = (const float*)fc->b->image_draws + 16 * (size_t)t->imageDraw;
    uint32_t clipIDBits, blendMode;
    memcpy(&clipIDBits, inst + 13, 4);
    memcpy(&blendMode, inst + 14, 4);
    float coverage = 1.f;
    if (features & SF_CLIP_RECT)
    {
        /* clip_rect_distance reads PaintAuxData words 8-13. */
        float aux[14] = {0};
        memcpy(aux + 8, inst + 4, 4 * sizeof(float));
        aux[12] = inst[10];
        aux[13] = inst[11];
        coverage = minf(maxf(clip_rect_distance(aux, fragX, fragY), 0.f), coverage);
    }
    if (features & SF_CLIPPING)
    {
        uint16_t clipID = id_bits_to_f16(clipIDBits, fc->granularity);
        if (clipID != 0)
        {
            uint16_t clipContentID = (uint16_t)(pls->clip >> 16);
            float clipCoverage = clipContentID == clipID ? h2f((uint16_t)(pls->clip & 0xffffu))
                                                         : 0.f;
            coverage = minf(coverage, maxf(clipCoverage, 0.f));
        }
    }
    coverage *= inst[12]; /* opacity, after clipping */
    float dst[4];
    for (int k = 0; k < 4; ++k)
        dst[k] = (float)pls->color[k] / 255.f;
    if (features & SF_ADVANCED_BLEND)
    {
        /* unmultiply_rgb (common.glsl:210-216). */
        const float r = color[3] != 0.f ? 1.f / color[3] : 0.f;
        color[0] *= r;
        color[1] *= r;
        color[2] *= r;
        if (blendMode != BLEND_SRC_OVER &&
            ((int)blendMode < BLEND_MODE_HUE || (features & SF_HSL_BLEND_MODES)))
        {
            float rgb[3];
            oracle_advanced_blend(color, dst, (int)blendMode, rgb);
            color[0] = rgb[0];
            color[1] = rgb[1];
            color[2] = rgb[2];
        }
        color[3] *= coverage;
        color[0] *= color[3];
        color[1] *= color[3];
        color[2] *= color[3];
    }
    else
    {
        for (int k = 0; k < 4; ++k)
            color[k] *= coverage;
    }
    if ((features & SF_DITHER) && color[3] != 0.f)
    {
        float n = ign(fragX, fragY, fc->ditherScale, fc->ditherBias);
        color[0] += n;
        color[1] += n;
        color[2] += n;
    }
    const float a = color[3];
    for (int k = 0; k < 4; ++k)
        pls->color[k] = unorm8(dst[k] * (1.f - a) + color[k]);
}

/* ENABLE_MODULATED_IMAGE (draw_path.vert:343-361, 478-493): the paint's
 * colour times its batch's image, sampled at the image matrix applied to the
 * pixel centre at the front end's level of detail (PaintAuxData words 16-22).
 * Texels are premultiplied; advanced blending wants them straight. */
static void image_modulate(const tri_rec* t,
                           const float* aux,
                           float fragX,
                           float fragY,
                           int unmultiplied,
                           float color[4])
{
    float m[4] = {aux[16], aux[17], aux[18], aux[19]};
    f2 uv = add2(mat_mul(m, (f2){fragX, fragY}), (f2){aux[20], aux[21]});
    float lod = (1.f + aux[22]) - 1.f; /* v_image.z = 1 + lod, then - 1 */
    float img[4];
    sample_image(t->image, t->sampler, uv.x, uv.y, lod, img);
    if (unmultiplied && img[3] != 0.f)
    {
        img[0] /= img[3];
        img[1] /= img[3];
        img[2] /= img[3];
    }
    for (int k = 0; k < 4; ++k)
        color[k] *= img[k];
}

/* find_paint_color (draw_path.vert:431-496, evaluated per fragment): the
 * paint's colour at the pixel centre with its alpha multiplied by `coverage`,
 * premultiplied unless advanced blending wants it straight. */
static void paint_color(const frag_ctx* fc,
                        const tri_rec* t,
                        uint32_t paintType,
                        const uint32_t* paint,
                        const float* aux,
                        float fragX,
                        float fragY,
                        float coverage,
                        int unmultiplied,
                        float color[4])
{
    if (paintType == SOLID_COLOR_PAINT_TYPE)
    {
        uint32_t c = paint[1];
        color[0] = (float)(c & 0xffu) / 255.f;
        color[1] = (float)((c >> 8) & 0xffu) / 255.f;
        color[2] = (float)((c >> 16) & 0xffu) / 255.f;
        color[3] = (float)(c >> 24) / 255.f;
        if (!unmultiplied)
        {
            color[0] *= color[3];
            color[1] *= color[3];
            color[2] *= color[3];
            for (int k = 0; k < 4; ++k)
                color[k] *= coverage;
        }
        else
            color[3] *= coverage;
    }
    else if (paintType == LINEAR_GRADIENT_PAINT_TYPE ||
             paintType == RADIAL_GRADIENT_PAINT_TYPE)
    {
        float pm[4] = {aux[0], aux[1], aux[2], aux[3]};
        f2 pc = add2(mat_mul(pm, (f2){fragX, fragY}), (f2){aux[4], aux[5]});
        float gradientSpan = aux[6];
        float spanB = gradientSpan > .9f ? 2.f : aux[7];
        float t = paintType == LINEAR_GRADIENT_PAINT_TYPE ? pc.x
                                                          : sqrtf(dot2(pc, pc));
        /* GLSL clamp() is min(max(t, 0), 1); GPUs evaluate min/max with
         * IEEE minNum/maxNum, so a NaN coordinate (a degenerate gradient,
         * whose paint matrix the front end writes as NaN) clamps to 0. */
        t = fminf(fmaxf(t, 0.f), 1.f);
        float x = spanB > 1.f
                      ? (1.f - 1.f / GRAD_TEXTURE_WIDTH) * t + (.5f / GRAD_TEXTURE_WIDTH)
                      : (1.f / GRAD_TEXTURE_WIDTH) * t + spanB;
        float row = u2f(paint[1]);
        sample_grad(fc->grad, fc->d->grad_data_height,
                    fc->d->grad_texture_height ? fc->d->grad_texture_height
                                               : fc->d->grad_data_height,
                    x, row, color);
        color[3] *= coverage;
        if (!unmultiplied)
        {
            color[0] *= color[3];
            color[1] *= color[3];
            color[2] *= color[3];
        }
    }
    else
    {
        /* Clip-update paint outside ENABLE_CLIPPING draws nothing sensible;
         * the reference leaves v_paint zero. */
        color[0] = color[1] = color[2] = color[3] = 0.f;
    }
    if ((t->features & SF_MODULATED_IMAGE) && (paint[0] & PAINT_FLAG_HAS_IMAGE) && t->image &&
        t->image->mips)
        image_modulate(t, aux, fragX, fragY, unmultiplied, color);
}

/* min_component of find_clip_rect_coverage_distances (common.glsl:376-400)
 * at the pixel centre. */
static float clip_rect_distance(const float* aux, float fragX, float fragY)
{
    float cm[4] = {aux[8], aux[9], aux[10], aux[11]};
    f2 ct = {aux[12], aux[13]};
    f2 aaw = {fabsf(cm[0]) + fabsf(cm[2]), fabsf(cm[1]) + fabsf(cm[3])};
    float cr[4];
    if (aaw.x != 0.f && aaw.y != 0.f)
    {
        f2 r = {1.f / aaw.x, 1.f / aaw.y};
        f2 cc = add2(mat_mul(cm, (f2){fragX, fragY}), ct);
        cr[0] = cc.x * r.x + r.x + .5f;
        cr[1] = cc.y * r.y + r.y + .5f;
        cr[2] = -cc.x * r.x + r.x + .5f;
        cr[3] = -cc.y * r.y + r.y + .5f;
    }
    else
    {
        cr[0] = cr[2] = ct.x;
        cr[1] = cr[3] = ct.y;
    }
    return minf(minf(cr[0], cr[1]), minf(cr[2], cr[3]));
}

/* The feather atlas sampled at atlas pixel coordinates (x, y): the linear
 * filter with clamp-to-edge addressing of the atlas sampler
 * (draw_mesh.frag:89-97), texel centres at half-integers. Addresses clamp to
 * the atlas content, the texels the atlas pass wrote. */
static float atlas_sample(const frag_ctx* fc, float x, float y)
{
    if (!fc->atlas || fc->atlasW <= 0 || fc->atlasH <= 0)
        return 0.f;
    const float u = x - .5f, v = y - .5f;
    if (!(u == u) || !(v == v))
        return 0.f;
    const float fu = floorf(u), fv = floorf(v);
    const float wu = u - fu, wv = v - fv;
    const float cu = fminf(fmaxf(fu, -1.f), (float)fc->atlasW);
    const float cv = fminf(fmaxf(fv, -1.f), (float)fc->atlasH);
    const int iu = (int)cu, iv = (int)cv;
    const int u0 = iu < 0 ? 0 : (iu > fc->atlasW - 1 ? fc->atlasW - 1 : iu);
    const int u1 = iu + 1 < 0 ? 0 : (iu + 1 > fc->atlasW - 1 ? fc->atlasW - 1 : iu + 1);
    const int v0 = iv < 0 ? 0 : (iv > fc->atlasH - 1 ? fc->atlasH - 1 : iv);
    const int v1 = iv + 1 < 0 ? 0 : (iv + 1 > fc->atlasH - 1 ? fc->atlasH - 1 : iv + 1);
    const float* a = fc->atlas;
    const size_t W = (size_t)fc->atlasW;
    const float t00 = a[v0 * W + u0], t10 = a[v0 * W + u1];
    const float t01 = a[v1 * W + u0], t11 = a[v1 * W + u1];
    const float top = t00 + (t10 - t00) * wu;
    const float bot = t01 + (t11 - t01) * wu;
    return top + (bot - top) * wv;
}

/* One fragment of a featherAtlasBlit draw (draw_mesh.frag:60-225 with
 * FEATHER_ATLAS_BLIT): the coverage is the atlas texel the pixel maps to,
 * clamped to [0, 1], cut by the clip rect and the clip; the paint is blended
 * straight into the colour plane (the coverage plane is left as it is). */
static void blit_fragment(const frag_ctx* fc,
                          const tri_rec* t,
                          float atlasX,
                          float atlasY,
                          int px,
                          int py,
                          pls_pixel* pls)
{
    const uint32_t features = t->features;
    const uint32_t pathID = t->pathID;
    const uint32_t* paint =
        (const uint32_t*)fc->b->paints + 2 * ((size_t)fc->d->first_paint + pathID);
    const float* aux =
        (const float*)fc->b->paint_aux + 32 * ((size_t)fc->d->first_paint_aux + pathID);
    const uint32_t paintType = paint[0] & 0xfu;
    const float fragX = (float)px + .5f, fragY = (float)py + .5f;
    float coverage = clampf(atlas_sample(fc, atlasX, atlasY), 0.f, 1.f);
    if (features & SF_CLIP_RECT)
        coverage = minf(maxf(clip_rect_distance(aux, fragX, fragY), 0.f), coverage);
    if (features & SF_CLIPPING)
    {
        uint32_t clipIDBits = (paintType == CLIP_UPDATE_PAINT_TYPE ? paint[1] : paint[0]) >> 16;
        uint16_t clipID = id_bits_to_f16(clipIDBits, fc->granularity);
        if (clipID != 0)
        {
            uint16_t clipContentID = (uint16_t)(pls->clip >> 16);
            float clipCoverage = clipContentID == clipID ? h2f((uint16_t)(pls->clip & 0xffffu))
                                                         : 0.f;
            clipCoverage = maxf(clipCoverage, 0.f);
            coverage = minf(coverage, clipCoverage);
        }
    }
    const int unmultiplied = (features & SF_ADVANCED_BLEND) != 0;
    float color[4];
    paint_color(fc, t, paintType, paint, aux, fragX, fragY, 1.f, unmultiplied, color);
    float dst[4];
    for (int k = 0; k < 4; ++k)
        dst[k] = (float)pls->color[k] / 255.f;
    if (unmultiplied)
    {
        uint32_t blendMode = (paint[0] >> 4) & 0xfu;
        if (blendMode != BLEND_SRC_OVER &&
            ((int)blendMode < BLEND_MODE_HUE || (features & SF_HSL_BLEND_MODES)))
        {
            float rgb[3];
            oracle_advanced_blend(color, dst, (int)blendMode, rgb);
            color[0] = rgb[0];
            color[1] = rgb[1];
            color[2] = rgb[2];
        }
        color[3] *= coverage;
        color[0] *= color[3];
        color[1] *= color[3];
        color[2] *= color[3];
    }
    else
    {
        for (int k = 0; k < 4; ++k)
            color[k] *= coverage;
    }
    if ((features & SF_DITHER) && color[3] != 0.f)
    {
        float n = ign(fragX, fragY, fc->ditherScale, fc->ditherBias);
        color[0] += n;
        color[1] += n;
        color[2] += n;
    }
    const float a = color[3];
    for (int k = 0; k < 4; ++k)
        pls->color[k] = unorm8(dst[k] * (1.f - a) + color[k]);
}

/* One fragment of draw_raster_order_path.frag:14-238. */
static void fragment(const frag_ctx* fc,
                     const tri_rec* t,
                     float covx,
                     float covy,
                     float covz,
                     float covw,
                     int px,
                     int py,
                     pls_pixel* pls)
{
    const uint32_t features = t->features;
    const uint32_t pathID = t->pathID;
    const uint32_t* paint =
        (const uint32_t*)fc->b->paints + 2 * ((size_t)fc->d->first_paint + pathID);
    const float* aux =
        (const float*)fc->b->paint_aux + 32 * ((size_t)fc->d->first_paint_aux + pathID);
    uint16_t vPathID = id_bits_to_f16(pathID, fc->granularity);
    int evenOdd = (paint[0] & PAINT_FLAG_EVEN_ODD_FILL) != 0;
    if (evenOdd)
        vPathID ^= 0x8000u;
    uint32_t paintType = paint[0] & 0xfu;
    float fragX = (float)px + .5f, fragY = (float)py + .5f;

    /* Coverage. */
    uint16_t covBufferID = (uint16_t)(pls->coverage >> 16);
    float coverageCount =
        covBufferID == vPathID ? h2f((uint16_t)(pls->coverage & 0xffffu)) : 0.f;
    if (t->interior)
    {
        /* draw_raster_order_path.frag:48-53: add the winding weight; the
         * coverage plane is preserved, not written. */
        coverageCount = coverageCount + covx;
    }
    else
    {
        if (covy >= 0.f) /* stroke */
        {
            /* find_stroke_coverage (draw_path.vert:501-509) */
            float frag = ((features & SF_FEATHER) && covx < FEATHER_COVERAGE_THRESHOLD)
                             ? eval_feathered_stroke(covx, covy)
                             : minf(covx, covy);
            coverageCount = maxf(frag, coverageCount);
        }
        else
        {
            /* find_fill_coverage (draw_path.vert:511-519) */
            float frag = ((features & SF_FEATHER) && covy < FEATHER_COVERAGE_THRESHOLD)
                             ? eval_feathered_fill(covx, covy, covz, covw)
                             : covx;
            coverageCount = coverageCount + frag;
        }
        uint16_t storedCount = oracle_f32_to_f16(coverageCount);
        pls->coverage = ((uint32_t)vPathID << 16) | storedCount;
        coverageCount = h2f(storedCount);
    }

    /* draw_raster_order_path.frag:63-82: clockwise fills keep positive
     * windings only; otherwise nonzero or even-odd. */
    float coverage;
    if (features & FEATURE_CLOCKWISE_FILL)
    {
        coverage = minf(maxf(coverageCount, 0.f), 1.f);
    }
    else
    {
        coverage = fabsf(coverageCount);
        if ((features & SF_EVEN_ODD) && evenOdd)
            coverage = 1.f - fabsf(fractf(coverage * .5f) * 2.f + -1.f);
        coverage = minf(coverage, 1.f);
    }

    /* Clip IDs (draw_path.vert:203-220). */
    float clipIDx = 0.f, clipIDy = 0.f;
    uint16_t clipIDxBits = 0;
    if (features & SF_CLIPPING)
    {
        uint32_t clipIDBits =
            (paintType == CLIP_UPDATE_PAINT_TYPE ? paint[1] : paint[0]) >> 16;
        clipIDxBits = id_bits_to_f16(clipIDBits, fc->granularity);
        clipIDx = h2f(clipIDxBits);
        if (paintType == CLIP_UPDATE_PAINT_TYPE)
        {
            clipIDx = -clipIDx;
            clipIDy = h2f(id_bits_to_f16(paint[0] >> 16, fc->granularity));
        }
    }

    if ((features & SF_CLIPPING) && clipIDx < 0.f)
    {
        uint16_t clipIDBitsPos = clipIDxBits; /* == -clipIDx */
        if ((features & SF_NESTED_CLIPPING) && clipIDy != 0.f)
        {
            uint16_t outerBits = id_bits_to_f16(paint[0] >> 16, fc->granularity);
            uint16_t clipContentID = (uint16_t)(pls->clip >> 16);
            float outerClipCoverage;
            if (clipContentID != clipIDBitsPos)
            {
                outerClipCoverage = clipContentID == outerBits
                                        ? h2f((uint16_t)(pls->clip & 0xffffu))
                                        : 0.f;
                if (!t->interior) /* interior triangles never hit twice */
                {
                    pls->scratch[0] = unorm8(outerClipCoverage);
                    pls->scratch[1] = pls->scratch[2] = pls->scratch[3] = 0;
                }
            }
            else
            {
                outerClipCoverage = (float)pls->scratch[0] / 255.f;
            }
            coverage = minf(coverage, outerClipCoverage);
        }
        pls->clip = ((uint32_t)clipIDBitsPos << 16) | oracle_f32_to_f16(coverage);
        return;
    }

    if (features & SF_CLIPPING)
    {
        if (clipIDx != 0.f)
        {
            uint16_t clipContentID = (uint16_t)(pls->clip >> 16);
            coverage = clipContentID == clipIDxBits
                           ? minf(h2f((uint16_t)(pls->clip & 0xffffu)), coverage)
                           : 0.f;
        }
    }
    if ((features & SF_CLIP_RECT))
        coverage = clampf(clip_rect_distance(aux, fragX, fragY), 0.f, coverage);

    int unmultiplied = (features & SF_ADVANCED_BLEND) != 0;
    float color[4];
    paint_color(fc, t, paintType, paint, aux, fragX, fragY, coverage, unmultiplied, color);

    float dst[4];
    if (covBufferID != vPathID)
    {
        for (int k = 0; k < 4; ++k)
            dst[k] = (float)pls->color[k] / 255.f;
        if (!t->interior) /* interior triangles are a path's last fragment here */
            memcpy(pls->scratch, pls->color, 4);
    }
    else
    {
        for (int k = 0; k < 4; ++k)
            dst[k] = (float)pls->scratch[k] / 255.f;
    }

    if (unmultiplied)
    {
        uint32_t blendMode = (paint[0] >> 4) & 0xfu;
        if (blendMode != BLEND_SRC_OVER)
        {
            int mode = (int)blendMode;
            if (mode >= BLEND_MODE_HUE && !(features & SF_HSL_BLEND_MODES))
            {
                /* Without the HSL feature the coeffs are left undefined in the
                 * reference; treat as srcOver. */
            }
            else
            {
                float rgb[3];
                oracle_advanced_blend(color, dst, mode, rgb);
                color[0] = rgb[0];
                color[1] = rgb[1];
                color[2] = rgb[2];
            }
        }
        color[0] *= color[3];
        color[1] *= color[3];
        color[2] *= color[3];
    }
    float paintAlpha = color[3];
    for (int k = 0; k < 4; ++k)
        color[k] += dst[k] * (1.f - paintAlpha);
    if ((features & SF_DITHER) && paintAlpha != 0.f)
    {
        float n = ign(fragX, fragY, fc->ditherScale, fc->ditherBias);
        color[0] += n;
        color[1] += n;
        color[2] += n;
    }
    for (int k = 0; k < 4; ++k)
        pls->color[k] = unorm8(color[k]);
}

/* Primitive assembly of one triangle into the pixel rectangle [x0, x1) x
 * [y0, y1) (the viewport, or an atlas batch's scissor). Counterclockwise
 * triangles are culled, except with `twoSided` (the atlas fill pipeline,
 * CullFace::none, gpu.hpp:2076-2077): they are turned clockwise and marked
 * `negate`, since a back-facing atlas fill subtracts its coverage. */
static int setup_triangle_rect(const vtx_out* a,
                               const vtx_out* bb,
                               const vtx_out* c,
                               uint32_t features,
                               int x0,
                               int y0,
                               int x1,
                               int y1,
                               int twoSided,
                               tri_rec* t)
{
    if (a->discard || bb->discard || c->discard)
        return 0;
    const vtx_out* v[3] = {a, bb, c};
    for (int i = 0; i < 3; ++i)
    {
        if (!isfinite(v[i]->pos.x) || !isfinite(v[i]->pos.y))
            return 0;
        if (fabsf(v[i]->pos.x) > 4.0e6f || fabsf(v[i]->pos.y) > 4.0e6f)
            return -3; /* outside the fixed-point range of this rasteriser */
        t->x[i] = snap(v[i]->pos.x);
        t->y[i] = snap(v[i]->pos.y);
        t->cov[i][0] = v[i]->cov[0];
        t->cov[i][1] = v[i]->cov[1];
        t->cov[i][2] = v[i]->cov[2];
        t->cov[i][3] = v[i]->cov[3];
    }
    int64_t area2 = (t->x[1] - t->x[0]) * (t->y[2] - t->y[0]) -
                    (t->x[2] - t->x[0]) * (t->y[1] - t->y[0]);
    t->negate = 0;
    if (area2 < 0 && twoSided)
    {
        int64_t tx = t->x[1], ty = t->y[1];
        t->x[1] = t->x[2];
        t->y[1] = t->y[2];
        t->x[2] = tx;
        t->y[2] = ty;
        for (int k = 0; k < 4; ++k)
        {
            float tc = t->cov[1][k];
            t->cov[1][k] = t->cov[2][k];
            t->cov[2][k] = tc;
        }
        area2 = -area2;
        t->negate = 1;
    }
    if (area2 <= 0) /* counterclockwise faces are culled; degenerate drop */
        return 0;
    int64_t minx = t->x[0], maxx = t->x[0], miny = t->y[0], maxy = t->y[0];
    for (int i = 1; i < 3; ++i)
    {
        if (t->x[i] < minx) minx = t->x[i];
        if (t->x[i] > maxx) maxx = t->x[i];
        if (t->y[i] < miny) miny = t->y[i];
        if (t->y[i] > maxy) maxy = t->y[i];
    }
    /* Pixels whose centres (k + 1/2) lie in [min, max]. */
    int64_t bx0 = (minx - SUBPIXEL_ONE / 2 + SUBPIXEL_ONE - 1) >> SUBPIXEL_BITS;
    int64_t bx1 = ((maxx - SUBPIXEL_ONE / 2) >> SUBPIXEL_BITS) + 1;
    int64_t by0 = (miny - SUBPIXEL_ONE / 2 + SUBPIXEL_ONE - 1) >> SUBPIXEL_BITS;
    int64_t by1 = ((maxy - SUBPIXEL_ONE / 2) >> SUBPIXEL_BITS) + 1;
    if (bx0 < x0) bx0 = x0;
    if (by0 < y0) by0 = y0;
    if (bx1 > x1) bx1 = x1;
    if (by1 > y1) by1 = y1;
    if (bx0 >= bx1 || by0 >= by1)
        return 0;
    t->bx0 = (int32_t)bx0;
    t->bx1 = (int32_t)bx1;
    t->by0 = (int32_t)by0;
    t->by1 = (int32_t)by1;
    t->pathID = v[0]->pathID;
    t->features = features;
    t->interior = 0;
    t->blit = 0;
    t->image = NULL;
    t->sampler = 0;
    t->mesh = 0;
    return 1;
}

static int setup_triangle(const vtx_out* a,
                          const vtx_out* bb,
                          const vtx_out* c,
                          uint32_t features,
                          int W,
                          int H,
                          tri_rec* t)
{
    return setup_triangle_rect(a, bb, c, features, 0, 0, W, H, 0, t);
}

/* Edge function of edge a->b at point p, with the top-left tie rule for
 * clockwise (screen-space, y down) triangles. Returns > 0 when p is inside. */
static inline int edge_inside(int64_t ax, int64_t ay, int64_t bx, int64_t by,
                              int64_t px, int64_t py, int64_t* e)
{
    int64_t dx = bx - ax, dy = by - ay;
    int64_t v = dx * (py - ay) - dy * (px - ax);
    *e = v;
    if (v > 0)
        return 1;
    if (v < 0)
        return 0;
    return (dy == 0 && dx > 0) || dy < 0;
}

static void raster_triangle_rows(const frag_ctx* fc,
                                 const tri_rec* t,
                                 int row0,
                                 int row1,
                                 pls_pixel* pls,
                                 int W,
                                 uint64_t* frags)
{
    int y0 = t->by0 > row0 ? t->by0 : row0;
    int y1 = t->by1 < row1 ? t->by1 : row1;
    if (y0 >= y1)
        return;
    double area2 = (double)((t->x[1] - t->x[0]) * (t->y[2] - t->y[0]) -
                            (t->x[2] - t->x[0]) * (t->y[1] - t->y[0]));
    for (int py = y0; py < y1; ++py)
    {
        int64_t cy = ((int64_t)py << SUBPIXEL_BITS) + SUBPIXEL_ONE / 2;
        for (int px = t->bx0; px < t->bx1; ++px)
        {
            int64_t cx = ((int64_t)px << SUBPIXEL_BITS) + SUBPIXEL_ONE / 2;
            int64_t e0, e1, e2;
            /* e0: edge v1->v2 (weight of v0), e1: v2->v0, e2: v0->v1 */
            if (!edge_inside(t->x[1], t->y[1], t->x[2], t->y[2], cx, cy, &e0))
                continue;
            if (!edge_inside(t->x[2], t->y[2], t->x[0], t->y[0], cx, cy, &e1))
                continue;
            if (!edge_inside(t->x[0], t->y[0], t->x[1], t->y[1], cx, cy, &e2))
                continue;
            float l0 = (float)((double)e0 / area2);
            float l1 = (float)((double)e1 / area2);
            float l2 = (float)((double)e2 / area2);
            float covx = l0 * t->cov[0][0] + l1 * t->cov[1][0] + l2 * t->cov[2][0];
            float covy = l0 * t->cov[0][1] + l1 * t->cov[1][1] + l2 * t->cov[2][1];
            float covz = 0.f, covw = 0.f;
            if (covy < FEATHER_COVERAGE_THRESHOLD) /* a feathered fill needs all four */
            {
                covz = l0 * t->cov[0][2] + l1 * t->cov[1][2] + l2 * t->cov[2][2];
                covw = l0 * t->cov[0][3] + l1 * t->cov[1][3] + l2 * t->cov[2][3];
            }
            if (t->mesh)
                mesh_fragment(fc, t, px, py, pls + (size_t)py * W + px);
            else if (t->blit)
                blit_fragment(fc, t, covx, covy, px, py, pls + (size_t)py * W + px);
            else
                fragment(fc, t, covx, covy, covz, covw, px, py, pls + (size_t)py * W + px);
            ++*frags;
        }
    }
}

/* The atlas pass's fragments of one triangle on rows [row0, row1)
 * (render_atlas.glsl:58-77, the floating-point render target with fixed
 * function blending): a fill adds its feathered coverage, negated when the
 * triangle faced away, a stroke keeps the maximum; the R16F target rounds
 * every blend result to fp16. */
static void raster_atlas_rows(const tri_rec* t, int row0, int row1, float* atlas, int W)
{
    int y0 = t->by0 > row0 ? t->by0 : row0;
    int y1 = t->by1 < row1 ? t->by1 : row1;
    if (y0 >= y1)
        return;
    double area2 = (double)((t->x[1] - t->x[0]) * (t->y[2] - t->y[0]) -
                            (t->x[2] - t->x[0]) * (t->y[1] - t->y[0]));
    for (int py = y0; py < y1; ++py)
    {
        int64_t cy = ((int64_t)py << SUBPIXEL_BITS) + SUBPIXEL_ONE / 2;
        for (int px = t->bx0; px < t->bx1; ++px)
        {
            int64_t cx = ((int64_t)px << SUBPIXEL_BITS) + SUBPIXEL_ONE / 2;
            int64_t e0, e1, e2;
            if (!edge_inside(t->x[1], t->y[1], t->x[2], t->y[2], cx, cy, &e0))
                continue;
            if (!edge_inside(t->x[2], t->y[2], t->x[0], t->y[0], cx, cy, &e1))
                continue;
            if (!edge_inside(t->x[0], t->y[0], t->x[1], t->y[1], cx, cy, &e2))
                continue;
            float l0 = (float)((double)e0 / area2);
            float l1 = (float)((double)e1 / area2);
            float l2 = (float)((double)e2 / area2);
            float covx = l0 * t->cov[0][0] + l1 * t->cov[1][0] + l2 * t->cov[2][0];
            float covy = l0 * t->cov[0][1] + l1 * t->cov[1][1] + l2 * t->cov[2][1];
            float* texel = atlas + (size_t)py * W + px;
            if (covy >= 0.f)
            {
                float c = eval_feathered_stroke(covx, covy);
                *texel = h2f(oracle_f32_to_f16(maxf(*texel, c)));
            }
            else
            {
                float c = covx;
                if (covy < FEATHER_COVERAGE_THRESHOLD)
                {
                    float covz = l0 * t->cov[0][2] + l1 * t->cov[1][2] + l2 * t->cov[2][2];
                    float covw = l0 * t->cov[0][3] + l1 * t->cov[1][3] + l2 * t->cov[2][3];
                    c = eval_feathered_fill(covx, covy, covz, covw);
                }
                if (t->negate)
                    c = -c;
                *texel = h2f(oracle_f32_to_f16(*texel + c));
            }
        }
    }
}

static int grow_tris(tri_rec** tris, size_t* cap, size_t n)
{
    if (n < *cap)
        return 0;
    size_t nc = *cap * 2;
    tri_rec* nt = (tri_rec*)realloc(*tris, nc * sizeof(tri_rec));
    if (!nt)
        return -4;
    *tris = nt;
    *cap = nc;
    return 0;
}

/* The feather atlas pass (RenderContextGLImpl's atlas fill and stroke
 * draws, render_context_gl_impl.cpp:2545-2590; render_atlas.glsl): every
 * atlas batch's patches -- center-AA midpoint fans for fills, the border
 * triangles of midpoint fans for strokes -- shaded as in the main pass, moved
 * into the atlas by their path's atlas transform (PathData words 9-11,
 * render_atlas.glsl:30-35), scissored, and rasterised into a cleared
 * atlasContentWidth x atlasContentHeight fp16 target: fill batches first,
 * then stroke batches, each in patch order. */
static int render_atlas(const rive_cuda_flush_desc* d,
                        const oracle_buffers* b,
                        const uint32_t* tess,
                        size_t tessTexels,
                        float** out,
                        int threads)
{
    *out = NULL;
    const uint32_t nb = d->atlas_fill_batch_count + d->atlas_stroke_batch_count;
    const int W = (int)d->atlas_content_width, H = (int)d->atlas_content_height;
    if (W <= 0 || H <= 0)
        return nb ? -1 : 0;
    if (W > 16384 || H > 16384 || (nb && !d->atlas_batches))
        return -1;
    float* atlas = (float*)calloc((size_t)W * H, sizeof(float));
    if (!atlas)
        return -4;
    size_t cap = 1024, n = 0;
    tri_rec* tris = (tri_rec*)malloc(cap * sizeof(tri_rec));
    if (!tris)
    {
        free(atlas);
        return -4;
    }
    int rc = 0;
    for (uint32_t bi = 0; bi < nb && rc == 0; ++bi)
    {
        const rive_cuda_atlas_batch* ab = &d->atlas_batches[bi];
        const int fill = bi < d->atlas_fill_batch_count;
        const patch_vertex* table = fill ? g_center : g_patch;
        const uint16_t* idx = fill ? g_center_idx : g_patch_idx;
        const int nv = fill ? CENTER_VERTEX_COUNT : PATCH_VERTEX_COUNT;
        /* kMidpointFanCenterAAPatchIndexCount, kMidpointFanPatchBorderIndexCount */
        const int ni = fill ? CENTER_INDEX_COUNT : 8 * 6;
        int sx0 = ab->scissor[0], sy0 = ab->scissor[1];
        int sx1 = ab->scissor[2] < W ? ab->scissor[2] : W;
        int sy1 = ab->scissor[3] < H ? ab->scissor[3] : H;
        for (uint32_t inst = ab->base_patch; inst < ab->base_patch + ab->patch_count && rc == 0;
             ++inst)
        {
            vtx_out vo[OUTER_VERTEX_COUNT];
            for (int k = 0; k < nv && rc == 0; ++k)
            {
                rc = patch_vertex_shader(d, b, tess, tessTexels, &table[k], inst, &vo[k]);
                if (rc == 0 && !vo[k].discard)
                {
                    const float* path = path_record(d, b, vo[k].pathID);
                    if (!path)
                    {
                        rc = -1;
                        break;
                    }
                    /* vertexPosition * atlasTransform.x + atlasTransform.yz */
                    vo[k].pos.x = vo[k].pos.x * path[9] + path[10];
                    vo[k].pos.y = vo[k].pos.y * path[9] + path[11];
                }
            }
            for (int k = 0; k < ni && rc == 0; k += 3)
            {
                rc = grow_tris(&tris, &cap, n);
                if (rc == 0)
                {
                    int r = setup_triangle_rect(&vo[idx[k]], &vo[idx[k + 1]], &vo[idx[k + 2]], 0,
                                                sx0, sy0, sx1, sy1, fill, &tris[n]);
                    if (r < 0)
                        rc = r;
                    else
                        n += (size_t)r;
                }
            }
        }
    }
    if (rc == 0)
    {
        const int band = 8;
        const int nbands = (H + band - 1) / band;
#ifdef _OPENMP
        if (threads > 0)
            omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
        for (int bnd = 0; bnd < nbands; ++bnd)
        {
            int r0 = bnd * band, r1 = r0 + band < H ? r0 + band : H;
            for (size_t i = 0; i < n; ++i)
                raster_atlas_rows(&tris[i], r0, r1, atlas, W);
        }
    }
    free(tris);
    if (rc != 0)
    {
        free(atlas);
        return rc;
    }
    *out = atlas;
    return 0;
}

int oracle_draw(const rive_cuda_flush_desc* d,
                const oracle_buffers* b,
                const uint32_t* tess,
                const uint8_t* grad,
                uint8_t* fb,
                int threads)
{
    build_patch_tables();
    const int W = (int)d->render_target_width, H = (int)d->render_target_height;
    const size_t tessTexels = (size_t)TESS_TEXTURE_WIDTH * d->tess_data_height;
    if (d->interlock_mode != 0)
        return -2;
    if (b->flush_uniforms_bytes < d->flush_uniform_offset_bytes + 256u)
        return -1;
    const uint8_t* uni = (const uint8_t*)b->flush_uniforms + d->flush_uniform_offset_bytes;
    /* FlushUniforms (gpu.hpp:1466-1537): pathIDGranularity at byte 72,
     * ditherScale at 88, ditherBias at 92. */
    uint32_t granularity;
    float ditherScale, ditherBias, mipLodBias;
    memcpy(&granularity, uni + 72, 4);
    memcpy(&mipLodBias, uni + 80, 4);
    memcpy(&ditherScale, uni + 88, 4);
    memcpy(&ditherBias, uni + 92, 4);

    build_feather_table(); /* before any parallel region reads it */

    /* The feather atlas first: the main pass's blits sample it. */
    float* atlas = NULL;
    {
        int arc = render_atlas(d, b, tess, tessTexels, &atlas, threads);
        if (arc != 0)
            return arc;
    }

    /* Vertex processing + primitive assembly, in primitive order. */
    size_t cap = 1024, n = 0;
    tri_rec* tris = (tri_rec*)malloc(cap * sizeof(tri_rec));
    if (!tris)
    {
        free(atlas);
        return -4;
    }
    for (uint32_t bi = 0; bi < d->draw_batch_count; ++bi)
    {
        const rive_cuda_draw_batch* batch = &d->draw_batches[bi];
        /* ENABLE_FEATHER: feathered strokes (midpoint-fan batches) and
         * feathered fills (center-AA batches). */
        if (((batch->shader_features & SF_FEATHER) &&
             batch->draw_type != RIVE_CUDA_DRAW_MIDPOINT_FAN_PATCHES &&
             batch->draw_type != DRAW_TYPE_MIDPOINT_FAN_CENTER_AA_PATCHES) ||
            (batch->shader_misc_flags & ~MISC_CLOCKWISE_FILL))
        {
            free(tris);
            return -2;
        }
        const uint32_t features =
            batch->shader_features |
            ((batch->shader_misc_flags & MISC_CLOCKWISE_FILL) ? FEATURE_CLOCKWISE_FILL : 0u);
        const size_t batchFirstTri = n;
        int rc = 0;
        if (batch->draw_type == RIVE_CUDA_DRAW_MIDPOINT_FAN_PATCHES ||
            batch->draw_type == DRAW_TYPE_MIDPOINT_FAN_CENTER_AA_PATCHES ||
            batch->draw_type == DRAW_TYPE_OUTER_CURVE_PATCHES)
        {
            const int outer = batch->draw_type == DRAW_TYPE_OUTER_CURVE_PATCHES;
            const int center = batch->draw_type == DRAW_TYPE_MIDPOINT_FAN_CENTER_AA_PATCHES;
            const patch_vertex* table = outer ? g_outer : center ? g_center : g_patch;
            const uint16_t* idx = outer ? g_outer_idx : center ? g_center_idx : g_patch_idx;
            const int nv = outer ? OUTER_VERTEX_COUNT : center ? CENTER_VERTEX_COUNT
                                                                : PATCH_VERTEX_COUNT;
            const int ni = outer ? OUTER_INDEX_COUNT : center ? CENTER_INDEX_COUNT
                                                               : PATCH_INDEX_COUNT;
            for (uint32_t inst = batch->base_element;
                 inst < batch->base_element + batch->element_count && rc == 0;
                 ++inst)
            {
                vtx_out vo[OUTER_VERTEX_COUNT];
                for (int k = 0; k < nv && rc == 0; ++k)
                    rc = patch_vertex_shader(d, b, tess, tessTexels, &table[k], inst, &vo[k]);
                for (int k = 0; k < ni && rc == 0; k += 3)
                {
                    rc = grow_tris(&tris, &cap, n);
                    if (rc == 0)
                    {
                        int r = setup_triangle(&vo[idx[k]], &vo[idx[k + 1]], &vo[idx[k + 2]],
                                               features, W, H, &tris[n]);
                        if (r < 0)
                            rc = r;
                        else
                            n += (size_t)r;
                    }
                }
            }
        }
        else if (batch->draw_type == DRAW_TYPE_INTERIOR_TRIANGULATION)
        {
            /* unpack_interior_triangle_vertex (draw_path_common.glsl:792-819):
             * three TriangleVertex records {x, y, weight << 16 | pathID} per
             * triangle, drawn with the winding weight as constant coverage. */
            if (batch->element_count % 3 ||
                ((size_t)batch->base_element + batch->element_count) * 12 > b->triangles_bytes)
                rc = -1;
            const uint32_t* tv = (const uint32_t*)b->triangles;
            for (uint32_t v = batch->base_element;
                 v < batch->base_element + batch->element_count && rc == 0; v += 3)
            {
                vtx_out vo[3];
                for (int k = 0; k < 3 && rc == 0; ++k)
                {
                    const uint32_t* r = tv + 3 * ((size_t)v + k);
                    uint32_t pathID = r[2] & 0xffffu;
                    const float* path = path_record(d, b, pathID);
                    if (!path)
                    {
                        rc = -1;
                        break;
                    }
                    float M[4] = {path[0], path[1], path[2], path[3]};
                    f2 p = mat_mul(M, (f2){u2f(r[0]), u2f(r[1])});
                    vo[k].pos = (f2){p.x + path[4], p.y + path[5]};
                    vo[k].cov[0] = (float)((int32_t)r[2] >> 16);
                    vo[k].cov[1] = -1.f;
                    vo[k].cov[2] = vo[k].cov[3] = 0.f;
                    vo[k].pathID = pathID;
                    vo[k].discard = 0;
                }
                if (rc == 0)
                    rc = grow_tris(&tris, &cap, n);
                if (rc == 0)
                {
                    int r = setup_triangle(&vo[0], &vo[1], &vo[2], features, W, H, &tris[n]);
                    if (r < 0)
                        rc = r;
                    else if (r > 0)
                        tris[n++].interior = 1;
                }
            }
        }
        else if (batch->draw_type == DRAW_TYPE_FEATHER_ATLAS_BLIT)
        {
            /* unpack_atlas_coverage_vertex (draw_path_common.glsl:822-844):
             * the rectangle's TriangleVertex records are screen positions;
             * each carries its atlas position, screen * scale + translate
             * by the path's atlas transform, for the fragment to sample. */
            if (batch->element_count % 3 ||
                ((size_t)batch->base_element + batch->element_count) * 12 > b->triangles_bytes)
                rc = -1;
            const uint32_t* tv = (const uint32_t*)b->triangles;
            for (uint32_t v = batch->base_element;
                 v < batch->base_element + batch->element_count && rc == 0; v += 3)
            {
                vtx_out vo[3];
                for (int k = 0; k < 3 && rc == 0; ++k)
                {
                    const uint32_t* r = tv + 3 * ((size_t)v + k);
                    uint32_t pathID = r[2] & 0xffffu;
                    const float* path = path_record(d, b, pathID);
                    if (!path)
                    {
                        rc = -1;
                        break;
                    }
                    vo[k].pos = (f2){u2f(r[0]), u2f(r[1])};
                    vo[k].cov[0] = vo[k].pos.x * path[9] + path[10];
                    vo[k].cov[1] = vo[k].pos.y * path[9] + path[11];
                    vo[k].cov[2] = vo[k].cov[3] = 0.f;
                    vo[k].pathID = pathID;
                    vo[k].discard = 0;
                }
                if (rc == 0)
                    rc = grow_tris(&tris, &cap, n);
                if (rc == 0)
                {
                    int r = setup_triangle(&vo[0], &vo[1], &vo[2], features, W, H, &tris[n]);
                    if (r < 0)
                        rc = r;
                    else if (r > 0)
                        tris[n++].blit = 1;
                }
            }
        }
        else if (batch->draw_type == DRAW_TYPE_IMAGE_MESH)
        {
            /* draw_image_mesh.vert: per index triple, the view matrix times
             * the local position plus the translate (ImageDrawInstance
             * batch->base_element), carrying the texture coordinates; no
             * face culled (get_cull_face, gpu.cpp:1552-1593). */
            const rive_cuda_batch_mesh* m = d->batch_meshes ? &d->batch_meshes[bi] : NULL;
            const oracle_texture* tex =
                d->batch_images ? (const oracle_texture*)d->batch_images[bi].texture : NULL;
            if (!m || !m->vertices || !m->uvs || !m->indices || !tex || m->index_count % 3 ||
                ((size_t)batch->base_element + 1) * 64 > b->image_draws_bytes)
                rc = -1;
            const oracle_render_buffer* vb = m ? (const oracle_render_buffer*)m->vertices : NULL;
            const oracle_render_buffer* ub = m ? (const oracle_render_buffer*)m->uvs : NULL;
            const oracle_render_buffer* ib = m ? (const oracle_render_buffer*)m->indices : NULL;
            if (rc == 0 && (size_t)m->index_count * 2 > ib->bytes)
                rc = -1;
            const size_t nv = rc == 0 ? (vb->bytes < ub->bytes ? vb->bytes : ub->bytes) / 8 : 0;
            const float* inst =
                rc == 0 ? (const float*)b->image_draws + 16 * (size_t)batch->base_element : NULL;
            for (uint32_t k3 = 0; rc == 0 && k3 < m->index_count; k3 += 3)
            {
                vtx_out vo[3];
                for (int k = 0; k < 3 && rc == 0; ++k)
                {
                    const uint16_t vi = ((const uint16_t*)ib->data)[k3 + k];
                    if (vi >= nv)
                    {
                        rc = -1;
                        break;
                    }
                    const float* p = (const float*)vb->data + 2 * (size_t)vi;
                    const float* uv = (const float*)ub->data + 2 * (size_t)vi;
                    vo[k].pos = (f2){inst[0] * p[0] + inst[2] * p[1] + inst[8],
                                     inst[1] * p[0] + inst[3] * p[1] + inst[9]};
                    vo[k].cov[0] = uv[0];
                    vo[k].cov[1] = uv[1];
                    vo[k].cov[2] = vo[k].cov[3] = 0.f;
                    vo[k].pathID = 0;
                    vo[k].discard = 0;
                }
                if (rc == 0)
                    rc = grow_tris(&tris, &cap, n);
                if (rc == 0)
                {
                    int r = setup_triangle_rect(&vo[0], &vo[1], &vo[2], features, 0, 0, W, H, 1,
                                                &tris[n]);
                    if (r < 0)
                        rc = r;
                    else if (r > 0)
                    {
                        tris[n].mesh = 1;
                        tris[n].imageDraw = batch->base_element;
                        tris[n].negate = 0;
                        mesh_planes(&tris[n], tex, mipLodBias);
                        ++n;
                    }
                }
            }
        }
        else
        {
            rc = -2;
        }
        if (rc != 0)
        {
            free(tris);
            free(atlas);
            return rc;
        }
        const oracle_texture* image =
            d->batch_images ? (const oracle_texture*)d->batch_images[bi].texture : NULL;
        for (size_t k = batchFirstTri; k < n; ++k)
        {
            tris[k].image = image;
            tris[k].sampler = image ? d->batch_images[bi].sampler_key : 0u;
        }
    }

    /* PLS planes at the start of the render pass. */
    pls_pixel* pls = (pls_pixel*)malloc((size_t)W * H * sizeof(pls_pixel));
    if (!pls)
    {
        free(tris);
        free(atlas);
        return -4;
    }
    uint8_t clear[4];
    {
        float c[4];
        unpack_color_int(d->color_clear_value, c);
        clear[0] = unorm8(c[0] * c[3]);
        clear[1] = unorm8(c[1] * c[3]);
        clear[2] = unorm8(c[2] * c[3]);
        clear[3] = unorm8(c[3]);
    }
    for (size_t i = 0; i < (size_t)W * H; ++i)
    {
        if (d->color_load_action == RIVE_CUDA_LOAD_CLEAR)
            memcpy(pls[i].color, clear, 4);
        else
            memcpy(pls[i].color, fb + i * 4, 4);
        pls[i].clip = 0;
        pls[i].coverage = 0;
        memset(pls[i].scratch, 0, 4);
    }

    frag_ctx fc = {d,          b,    grad, granularity, ditherScale, ditherBias, atlas,
                   (int)d->atlas_content_width, (int)d->atlas_content_height};
    const int band = 8;
    const int nbands = (H + band - 1) / band;
    uint64_t frags = 0;
#ifdef _OPENMP
    if (threads > 0)
        omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : frags)
#endif
    for (int bnd = 0; bnd < nbands; ++bnd)
    {
        int r0 = bnd * band, r1 = r0 + band < H ? r0 + band : H;
        uint64_t local = 0;
        for (size_t i = 0; i < n; ++i)
            raster_triangle_rows(&fc, &tris[i], r0, r1, pls, W, &local);
        frags += local;
    }
    for (size_t i = 0; i < (size_t)W * H; ++i)
        memcpy(fb + i * 4, pls[i].color, 4);
    g_stat_triangles = n;
    g_stat_fragments = frags;
    free(pls);
    free(tris);
    free(atlas);
    return 0;
}

void oracle_last_stats(uint64_t* triangles, uint64_t* fragments)
{
    if (triangles)
        *triangles = g_stat_triangles;
    if (fragments)
        *fragments = g_stat_fragments;
}

int oracle_flush(const rive_cuda_flush_desc* d,
                 const oracle_buffers* b,
                 uint8_t* fb,
                 int threads)
{
    size_t gradBytes = (size_t)GRAD_TEXTURE_WIDTH * (d->grad_data_height ? d->grad_data_height : 1) * 4;
    size_t tessBytes = (size_t)TESS_TEXTURE_WIDTH * (d->tess_data_height ? d->tess_data_height : 1) * 16;
    uint8_t* grad = (uint8_t*)calloc(1, gradBytes);
    uint32_t* tess = (uint32_t*)calloc(1, tessBytes);
    int rc = -4;
    if (grad && tess)
    {
        rc = oracle_color_ramps(d, b, grad);
        if (rc == 0)
            rc = oracle_tessellate(d, b, tess);
        if (rc == 0)
            rc = oracle_draw(d, b, tess, grad, fb, threads);
    }
    free(grad);
    free(tess);
    return rc;
}

/* The feather atlas of one logical flush (its tessellation, then the atlas
 * pass) as fp16 texels, atlas_content_width x atlas_content_height. */
int oracle_atlas(const rive_cuda_flush_desc* d,
                 const oracle_buffers* b,
                 uint16_t* out,
                 int threads)
{
    build_patch_tables();
    build_feather_table();
    size_t tessTexels = (size_t)TESS_TEXTURE_WIDTH * (d->tess_data_height ? d->tess_data_height : 1);
    uint32_t* tess = (uint32_t*)calloc(1, tessTexels * 16);
    if (!tess)
        return -4;
    int rc = oracle_tessellate(d, b, tess);
    float* atlas = NULL;
    if (rc == 0)
        rc = render_atlas(d, b, tess, (size_t)TESS_TEXTURE_WIDTH * d->tess_data_height, &atlas,
                          threads);
    if (rc == 0 && atlas)
    {
        const size_t n = (size_t)d->atlas_content_width * d->atlas_content_height;
        for (size_t i = 0; i < n; ++i)
            out[i] = oracle_f32_to_f16(atlas[i]);
    }
    free(atlas);
    free(tess);
    return rc;
}

/* ---- the shared fp32 elementary functions, for their accuracy test -------- */
/* fn: 0 sin, 1 cos, 2 acos, 3 cube root. */
int oracle_math_eval(int fn, const float* x, float* out, size_t n)
{
    for (size_t i = 0; i < n; ++i)
    {
        switch (fn)
        {
            case 0: out[i] = rc_sinf(x[i]); break;
            case 1: out[i] = rc_cosf(x[i]); break;
            case 2: out[i] = rc_acosf(x[i]); break;
            case 3: out[i] = rc_cbrtf(x[i]); break;
            default: return -1;
        }
    }
    return 0;
}

/* Shader functions of the tessellation pass on n inputs, for the tests that
 * hold them to the reference's bezier and Wang's-formula unit tests and to
 * the kernel's device functions. Per item, by fn:
 *   0 clamped_divide(a, b)                       in 2, out 1
 *   1 find_cubic_max_height(p0..p3)              in 8, out 2 (height, T)
 *   2 measure_cubic_local_curvature(p0..p3, T, spread)  in 10, out 1
 *   3 the De Casteljau point at T                in 9, out 2
 *   4 Wang's segment count under matrix m0..m3   in 12, out 1
 *   5 find_cubic_tangents(p0..p3)                in 8, out 4 */
int oracle_cubic_eval(int fn, const float* in, float* out, size_t n)
{
    static const int kIn[6] = {2, 8, 10, 9, 12, 8}, kOut[6] = {1, 2, 1, 2, 1, 4};
    if (fn < 0 || fn > 5)
        return -1;
    for (size_t i = 0; i < n; ++i)
    {
        const float* x = in + i * kIn[fn];
        float* y = out + i * kOut[fn];
        f2 p0 = {x[0], x[1]}, p1 = {x[2], x[3]}, p2 = {x[4], x[5]}, p3 = {x[6], x[7]};
        switch (fn)
        {
            case 0: y[0] = clamped_divide(x[0], x[1]); break;
            case 1: y[0] = find_cubic_max_height(p0, p1, p2, p3, &y[1]); break;
            case 2: y[0] = measure_cubic_local_curvature(p0, p1, p2, p3, x[8], x[9]); break;
            case 3:
            {
                f2 abc, bcd, q = eval_cubic_mix(p0, p1, p2, p3, x[8], &abc, &bcd);
                y[0] = q.x;
                y[1] = q.y;
                break;
            }
            case 4: y[0] = wang_cubic_segments(p0, p1, p2, p3, x + 8); break;
            default:
            {
                f2 t0, t1;
                find_cubic_tangents(p0, p1, p2, p3, &t0, &t1);
                y[0] = t0.x;
                y[1] = t0.y;
                y[2] = t1.x;
                y[3] = t1.y;
                break;
            }
        }
    }
    return 0;
}
