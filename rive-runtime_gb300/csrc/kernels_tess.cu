// Color-ramp and tessellation kernels (GPU passes 1 and 2 of a rasterOrdering
// flush).
//
//  * color_ramp_kernel restates renderer/src/shaders/color_ramp.glsl:40-107:
//    each GradientSpan paints a 1-texel-tall strip of the 512-wide RGBA8
//    gradient texture: a solid left border, a linear ramp between x0 and x1,
//    and a solid right border.
//  * tessellate_kernel restates renderer/src/shaders/tessellate.glsl:61-567:
//    each TessVertexSpan covers [x0, x1) (and optionally a mirrored range) of
//    one row of the 2048-wide tessellation texture; every texel is one
//    tessellated vertex (x, y, theta, contourIDWithFlags).
//
// GB300 mapping: one warp per span; the per-span set-up (tangents, polar step,
// join step) is evaluated once per lane without divergence, then lanes stride
// across the span's texels so each warp-wide store is 32 consecutive 16-byte
// texels (512 B, fully coalesced). The texture is plain linear HBM memory
// (row-major, 2048 texels per row), so the draw kernels read it with ordinary
// 128-bit loads.
#include "rive_cuda_internal.cuh"
#include "rive_fp32_math.h"

namespace rivecuda
{
namespace
{
__device__ __forceinline__ float2 f2sub(float2 a, float2 b)
{
    return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}
__device__ __forceinline__ float2 f2add(float2 a, float2 b)
{
    return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
}
__device__ __forceinline__ float2 f2scale(float2 a, float s)
{
    return make_float2(__fmul_rn(a.x, s), __fmul_rn(a.y, s));
}
__device__ __forceinline__ float f2dot(float2 a, float2 b)
{
    return __fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
__device__ __forceinline__ float f2cross(float2 a, float2 b)
{
    return __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y));
}
__device__ __forceinline__ bool f2ne(float2 a, float2 b)
{
    return a.x != b.x || a.y != b.y;
}
__device__ __forceinline__ float2 f2normalize(float2 v)
{
    float inv = __fdiv_rn(1.f, __fsqrt_rn(f2dot(v, v)));
    return f2scale(v, inv);
}
// (b - a) * t + a
__device__ __forceinline__ float2 f2lerp(float2 a, float2 b, float t)
{
    return f2add(f2scale(f2sub(b, a), t), a);
}

// bezier_utils.glsl:24-32
__device__ __forceinline__ float cos_between(float2 a, float2 b)
{
    float ab = f2dot(a, b);
    float p = __fmul_rn(f2dot(a, a), f2dot(b, b));
    if (p == 0.f)
        return 1.f;
    return fminf(fmaxf(__fmul_rn(ab, __fdiv_rn(1.f, __fsqrt_rn(p))), -1.f), 1.f);
}

// bezier_utils.glsl:65-71
__device__ __forceinline__ void cubic_tangents(float2 p0,
                                               float2 p1,
                                               float2 p2,
                                               float2 p3,
                                               float2& t0,
                                               float2& t1)
{
    t0 = f2sub(f2ne(p0, p1) ? p1 : (f2ne(p1, p2) ? p2 : p3), p0);
    t1 = f2sub(p3, f2ne(p3, p2) ? p2 : (f2ne(p2, p1) ? p1 : p0));
}

// common.glsl atan2(): acos of the normalized x, signed by y. The elementary
// functions of this file come from rive_fp32_math.h, which the oracle's
// tessellation shares, so its texels equal the oracle's bit for bit.
__device__ __forceinline__ float rive_atan2(float2 v)
{
    v = f2normalize(v);
    float theta = rc_acosf(fminf(fmaxf(v.x, -1.f), 1.f));
    return v.y >= 0.f ? theta : -theta;
}

// Compensated De Casteljau (Graillat, Langlois and Louvet's compensated
// evaluation): every mix (b - a) * t + a is computed with its exact rounding
// errors (TwoSum for the sums, a fused multiply-subtract for the product),
// the errors are carried through the levels with the values, and the point
// is value + error rounded once: as if evaluated in twice the precision, so
// the fp32 point is within about half an ulp of the exact point at T.
__device__ __forceinline__ float two_sum_err(float a, float b, float s)
{
    const float bb = __fsub_rn(s, a);
    return __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

struct CFloat
{
    float v, e; // value and its (first-order) error term
};

__device__ __forceinline__ CFloat cmix(CFloat a, CFloat b, float t)
{
    const float d = __fsub_rn(b.v, a.v);
    const float ed = two_sum_err(b.v, -a.v, d);
    const float p = __fmul_rn(d, t);
    const float ep = __fmaf_rn(d, t, -p);
    const float r = __fadd_rn(a.v, p);
    const float er = two_sum_err(a.v, p, r);
    // a + (b - a) t = r + er + ep + ed t, plus the inputs' errors mixed.
    const float e = __fadd_rn(__fadd_rn(__fadd_rn(er, ep), __fmul_rn(ed, t)),
                              __fmaf_rn(__fsub_rn(b.e, a.e), t, a.e));
    return CFloat{r, e};
}

__device__ __forceinline__ float eval_cubic_c(float a0, float a1, float a2, float a3, float t,
                                              float& t0, float& t1)
{
    const CFloat p0{a0, 0.f}, p1{a1, 0.f}, p2{a2, 0.f}, p3{a3, 0.f};
    const CFloat ab = cmix(p0, p1, t), bc = cmix(p1, p2, t), cd = cmix(p2, p3, t);
    const CFloat abc = cmix(ab, bc, t), bcd = cmix(bc, cd, t);
    const CFloat r = cmix(abc, bcd, t);
    t0 = abc.v;
    t1 = bcd.v;
    return __fadd_rn(r.v, r.e);
}

// The tessellated point at T by De Casteljau (tessellate.glsl:535-540),
// compensated as above. abc and bcd are the last level's pair, whose
// difference is the tangent.
__device__ __forceinline__ float2 eval_cubic_mix(float2 p0, float2 p1, float2 p2, float2 p3,
                                                 float T, float2& abc, float2& bcd)
{
    float2 q;
    q.x = eval_cubic_c(p0.x, p1.x, p2.x, p3.x, T, abc.x, bcd.x);
    q.y = eval_cubic_c(p0.y, p1.y, p2.y, p3.y, T, abc.y, bcd.y);
    return q;
}

// Wang's formula at precision 4 in pixel space under the path's 2x2 matrix m
// (columns (m.x, m.y), (m.z, m.w)): the CULL_EXCESS_TESSELLATION_SEGMENTS
// recount of the parametric segments (tessellate.glsl:195-211).
__device__ __forceinline__ float wang_cubic_segments(float2 p0, float2 p1, float2 p2, float2 p3,
                                                     float4 m)
{
    const float2 a = f2add(f2add(f2scale(p1, -2.f), p2), p0);
    const float2 c = f2add(f2add(f2scale(p2, -2.f), p3), p1);
    const float2 d0 = make_float2(__fadd_rn(__fmul_rn(m.x, a.x), __fmul_rn(m.z, a.y)),
                                  __fadd_rn(__fmul_rn(m.y, a.x), __fmul_rn(m.w, a.y)));
    const float2 d1 = make_float2(__fadd_rn(__fmul_rn(m.x, c.x), __fmul_rn(m.z, c.y)),
                                  __fadd_rn(__fmul_rn(m.y, c.x), __fmul_rn(m.w, c.y)));
    const float mm = fmaxf(f2dot(d0, d0), f2dot(d1, d1));
    return fmaxf(ceilf(__fsqrt_rn(__fmul_rn(.75f * 4.f, __fsqrt_rn(mm)))), 1.f);
}

// The inverse feather table (the height at which the Gaussian integral
// reaches x), fp16 values widened to float, written once per device by the
// host before any flush.
__device__ float g_inverseFeatherLUT[kGaussianTableSize];

// INVERSE_FEATHER(x) (common.glsl:61-68): linear filter, clamp to edge.
__device__ float inverse_feather_lut(float x)
{
    const float t = __fsub_rn(__fmul_rn(x, (float)kGaussianTableSize), .5f);
    if (!(t == t))
        return g_inverseFeatherLUT[0];
    const float f = floorf(t);
    const float w = __fsub_rn(t, f);
    const int i0 = (int)fminf(fmaxf(f, -1.f), (float)kGaussianTableSize);
    const int a = min(max(i0, 0), kGaussianTableSize - 1);
    const int b = min(max(i0 + 1, 0), kGaussianTableSize - 1);
    const float va = g_inverseFeatherLUT[a], vb = g_inverseFeatherLUT[b];
    return __fadd_rn(va, __fmul_rn(__fsub_rn(vb, va), w));
}

// mix(x, y, a) = x * (1 - a) + y * a
__device__ __forceinline__ float2 f2mix(float2 x, float2 y, float a)
{
    const float r = __fsub_rn(1.f, a);
    return make_float2(__fadd_rn(__fmul_rn(x.x, r), __fmul_rn(y.x, a)),
                       __fadd_rn(__fmul_rn(x.y, r), __fmul_rn(y.y, a)));
}

// clamp(a / b, 0, 1) without dividing when the result saturates
// (bezier_utils.glsl:164-169).
__device__ __forceinline__ float clamped_divide(float a, float b)
{
    if (b < 0.f)
        a = -a;
    b = fabsf(b);
    return a > 0.f ? (a < b ? __fdiv_rn(a, b) : 1.f) : 0.f;
}

// The height of a cubic above its chord at its highest point, found with three
// Newton steps from t = 1/2 (bezier_utils.glsl:173-245).
__device__ float cubic_max_height(float2 p0, float2 p1, float2 p2, float2 p3, float& outT)
{
    const float2 base = f2sub(p3, p0);
    const float lengthBase = __fsqrt_rn(f2dot(base, base));
    if (lengthBase == 0.f)
    {
        outT = .5f;
        return 0.f;
    }
    const float2 norm =
        make_float2(__fdiv_rn(-base.y, lengthBase), __fdiv_rn(base.x, lengthBase));
    const float h2 = f2dot(norm, f2sub(p2, p0));
    const float h1 = f2dot(norm, f2sub(p1, p0));
    const float dh = __fsub_rn(h1, h2);
    const float a3 = __fmul_rn(3.f, dh);
    const float b = __fsub_rn(-h1, dh);
    const float c = h1;
    float t = .5f;
    for (int i = 0; i < 3; ++i)
    {
        const float a3t = __fmul_rn(a3, t);
        t = clamped_divide(__fsub_rn(__fmul_rn(a3t, t), c), __fmul_rn(2.f, __fadd_rn(a3t, b)));
    }
    outT = t;
    return fabsf(__fmul_rn(
        t, __fadd_rn(__fmul_rn(t, __fadd_rn(__fmul_rn(t, a3), __fmul_rn(3.f, b))),
                     __fmul_rn(3.f, c))));
}

// The turn, in radians, of a cubic's tangent across an arc length of about
// 2 * desiredSpread centred at T (bezier_utils.glsl:77-153).
__device__ float cubic_local_curvature(float2 p0, float2 p1, float2 p2, float2 p3, float T,
                                       float desiredSpread)
{
    const float2 C = f2sub(p1, p0);
    const float2 D = f2sub(p2, p1);
    const float2 E = f2sub(p3, p0);
    const float2 B = f2sub(D, C);
    const float2 A = f2add(f2scale(D, -3.f), E);
    float2 tangent =
        f2scale(f2add(f2scale(f2add(f2scale(A, T), f2scale(B, 2.f)), T), C), 3.f);
    const float lengthTan = __fsqrt_rn(f2dot(tangent, tangent));
    if (lengthTan == 0.f)
        return 0.f;
    tangent = f2scale(tangent, __fdiv_rn(1.f, lengthTan));
    const float a = __fmul_rn(2.f, f2dot(A, tangent));
    const float c = __fadd_rn(
        __fmul_rn(__fmul_rn(3.f, __fadd_rn(__fmul_rn(a, T), __fmul_rn(4.f, f2dot(B, tangent)))),
                  T),
        __fmul_rn(6.f, f2dot(C, tangent)));
    const float maxDT = fminf(T, __fsub_rn(1.f, T));
    const float maxSpread = __fmul_rn(__fadd_rn(__fmul_rn(__fmul_rn(a, maxDT), maxDT), c), maxDT);
    const float targetSpread = fminf(desiredSpread, __fmul_rn(maxSpread, .9999f));
    float dt;
    if (a == 0.f)
    {
        dt = __fdiv_rn(targetSpread, c);
    }
    else
    {
        // The real root of a t^3 + c t - targetSpread (Cardano).
        const float r = __fdiv_rn(1.f, a);
        const float bb = __fmul_rn(c, r), cc = __fmul_rn(-targetSpread, r);
        const float Q = __fmul_rn(-1.f / 3.f, bb), R = __fmul_rn(.5f, cc);
        const float discr = __fsub_rn(__fmul_rn(R, R), __fmul_rn(__fmul_rn(Q, Q), Q));
        if (discr < 0.f)
        {
            const float sqrtQ = __fsqrt_rn(Q);
            const float th = rc_acosf(__fdiv_rn(R, __fmul_rn(__fmul_rn(sqrtQ, sqrtQ), sqrtQ)));
            dt = __fmul_rn(__fmul_rn(-2.f, sqrtQ),
                           rc_cosf(__fadd_rn(__fmul_rn(th, 1.f / 3.f), -kPi * 2.f / 3.f)));
        }
        else
        {
            float Aq = rc_cbrtf(__fadd_rn(fabsf(R), __fsqrt_rn(discr)));
            if (R < 0.f)
                Aq = -Aq;
            dt = Aq != 0.f ? __fadd_rn(Aq, __fdiv_rn(Q, Aq)) : 0.f;
        }
    }
    dt = fabsf(dt);
    const float t0 = __fsub_rn(T, dt), t1 = __fadd_rn(T, dt);
    const float2 dir0 = f2add(f2scale(f2add(f2scale(A, t0), f2scale(B, 2.f)), t0), C);
    const float2 dir1 = f2add(f2scale(f2add(f2scale(A, t1), f2scale(B, 2.f)), t1), C);
    float2 e0, e1;
    cubic_tangents(p0, p1, p2, p3, e0, e1);
    const float2 tan0 = t0 < 1e-3f ? e0 : dir0;
    const float2 tan1 = t1 > 1.f - 1e-3f ? e1 : dir1;
    return rc_acosf(cos_between(tan0, tan1));
}

struct SpanSetup
{
    float2 p0, p1, p2, p3;
    float2 joinTangent;
    float totalVertexCount;
    float parametricSegmentCount;
    float joinSegmentCount;
    float radsPerPolarSegment;
    float radsPerJoinSegment;
    uint32_t contourIDWithFlags; // without the mirrored flag
    bool valid;
};

// Per-span half of tessellate.glsl (the vertex shader, 61-287).
// kFeather: compiled with feathered-fill softening (ENABLE_FEATHER batches).
template <bool kFeather>
__device__ SpanSetup span_setup(const FlushParams& P, const uint4* sp)
{
    SpanSetup s;
    uint4 q0 = sp[0], q1 = sp[1], q2 = sp[2], q3 = sp[3];
    s.p0 = make_float2(__uint_as_float(q0.x), __uint_as_float(q0.y));
    s.p1 = make_float2(__uint_as_float(q0.z), __uint_as_float(q0.w));
    s.p2 = make_float2(__uint_as_float(q1.x), __uint_as_float(q1.y));
    s.p3 = make_float2(__uint_as_float(q1.z), __uint_as_float(q1.w));
    s.joinTangent = make_float2(__uint_as_float(q2.x), __uint_as_float(q2.y));
    uint32_t counts = q3.z;
    uint32_t parametric = counts & 0x3ffu;
    uint32_t polar = (counts >> 10) & 0x3ffu;
    uint32_t join = counts >> 20;
    uint32_t flags = q3.w;
    uint32_t contourID = flags & CONTOUR_ID_MASK;
    s.valid = true;
    uint32_t pathID = 0;
    if (contourID > 0)
    {
        if (contourID > P.contourCount)
        {
            atomicOr(P.error, ERR_BAD_CONTOUR);
            s.valid = false;
            return s;
        }
        pathID = P.contours[P.firstContour + contourID - 1].z;
    }
    float strokeRadius = 0.f, featherRadius = 0.f;
    uint4 pathRow0 = make_uint4(0, 0, 0, 0);
    if (pathID != 0)
    {
        if (pathID >= P.pathCount)
        {
            atomicOr(P.error, ERR_BAD_PATH);
            s.valid = false;
            return s;
        }
        const uint4* path = P.paths + 4 * (size_t)(P.firstPath + pathID);
        uint4 row1 = path[1];
        pathRow0 = path[0];
        strokeRadius = __uint_as_float(row1.z);
        featherRadius = __uint_as_float(row1.w);
    }
    if (kFeather && featherRadius != 0.f && strokeRadius == 0.f)
    {
        // tessellate.glsl:141-190: a feathered fill's cubic is pulled toward
        // its chord, the more the more it curves within one standard
        // deviation, mimicking the softening the feather gives a curve.
        float maxHeightT;
        const float height = cubic_max_height(s.p0, s.p1, s.p2, s.p3, maxHeightT);
        const float oneStddev = __fmul_rn(featherRadius, 1.f / kGaussianStddevs);
        const float curvature =
            cubic_local_curvature(s.p0, s.p1, s.p2, s.p3, maxHeightT, oneStddev);
        float dimming = __fsub_rn(1.f, __fmul_rn(curvature, 1.f / kPi));
        const float2 base = f2sub(s.p3, s.p0);
        const float stddevsPow2 = __fdiv_rn(f2dot(base, base), __fmul_rn(oneStddev, oneStddev));
        dimming = fminf(dimming, __fmul_rn(__fsub_rn(stddevsPow2, 1.f), .5f));
        dimming = fminf(dimming, .99f);
        const float x =
            __fadd_rn(__fmul_rn(inverse_feather_lut(__fmul_rn(.5f, dimming)), -2.f), 1.f);
        const float softness = clamped_divide(__fmul_rn(x, featherRadius), height);
        s.p1 = f2mix(s.p1, f2mix(s.p0, s.p3, 1.f / 3.f), softness);
        s.p2 = f2mix(s.p2, f2mix(s.p0, s.p3, 2.f / 3.f), softness);
    }
    if (flags & CULL_EXCESS_TESSELLATION_SEGMENTS_CONTOUR_FLAG)
    {
        const float4 m = make_float4(__uint_as_float(pathRow0.x), __uint_as_float(pathRow0.y),
                                     __uint_as_float(pathRow0.z), __uint_as_float(pathRow0.w));
        const uint32_t un = (uint32_t)wang_cubic_segments(s.p0, s.p1, s.p2, s.p3, m);
        parametric = min(un, parametric);
    }
    uint32_t total = parametric + polar + join - 1u;
    float2 t0, t1;
    cubic_tangents(s.p0, s.p1, s.p2, s.p3, t0, t1);
    float theta = rc_acosf(cos_between(t0, t1));
    float rpp = __fdiv_rn(theta, (float)polar);
    float turn = f2cross(f2sub(s.p2, s.p0), f2sub(s.p3, s.p1));
    if (turn == 0.f)
        turn = f2cross(t0, t1);
    if (turn < 0.f)
        rpp = -rpp;
    s.totalVertexCount = (float)total;
    s.parametricSegmentCount = (float)parametric;
    s.joinSegmentCount = (float)join;
    s.radsPerPolarSegment = rpp;
    s.radsPerJoinSegment = 0.f;
    if (join > 1u)
    {
        float joinTheta = rc_acosf(cos_between(t1, s.joinTangent));
        float joinSpan = (float)join;
        if ((flags & (JOIN_TYPE_MASK | EMULATED_STROKE_CAP_CONTOUR_FLAG)) ==
            (ROUND_JOIN_CONTOUR_FLAG | EMULATED_STROKE_CAP_CONTOUR_FLAG))
            joinSpan = __fsub_rn(joinSpan, 2.f);
        float rpj = __fdiv_rn(joinTheta, joinSpan);
        if (f2cross(t1, s.joinTangent) < 0.f)
            rpj = -rpj;
        s.radsPerJoinSegment = rpj;
    }
    s.contourIDWithFlags = flags;
    return s;
}

// Per-texel half of tessellate.glsl (the fragment shader, 294-567).
template <bool kFeather>
__device__ uint4 tess_vertex(const SpanSetup& s, float vertexIdxF, uint32_t flagsIn)
{
    float2 p0 = s.p0, p1 = s.p1, p2 = s.p2, p3 = s.p3;
    float2 tan0, tan1;
    cubic_tangents(p0, p1, p2, p3, tan0, tan1);
    float vertexIdx = fmaxf(floorf(vertexIdxF), 0.f);
    float parametricSegmentCount = s.parametricSegmentCount;
    float radsPerPolarSegment = s.radsPerPolarSegment;
    uint32_t flags = flagsIn;
    float mergedSegmentCount = __fsub_rn(s.totalVertexCount, s.joinSegmentCount);
    float mergedVertexID = vertexIdx;
    if (mergedVertexID <= mergedSegmentCount)
    {
        flags &= ~JOIN_TYPE_MASK;
    }
    else
    {
        p0 = p1 = p2 = p3;
        tan0 = tan1;
        tan1 = s.joinTangent;
        parametricSegmentCount = 1.f;
        mergedVertexID = __fsub_rn(mergedVertexID, mergedSegmentCount);
        mergedSegmentCount = s.joinSegmentCount;
        radsPerPolarSegment = s.radsPerJoinSegment;
        if ((flags & JOIN_TYPE_MASK) > ROUND_JOIN_CONTOUR_FLAG)
        {
            if (mergedVertexID < 2.5f)
                flags |= JOIN_TANGENT_0_CONTOUR_FLAG;
            if (mergedVertexID > 1.5f && mergedVertexID < 3.5f)
                flags |= JOIN_TANGENT_INNER_CONTOUR_FLAG;
        }
        else if ((flags & EMULATED_STROKE_CAP_CONTOUR_FLAG) ||
                 (flags & JOIN_TYPE_MASK) == FEATHER_JOIN_CONTOUR_FLAG)
        {
            mergedSegmentCount = __fsub_rn(mergedSegmentCount, 2.f);
            mergedVertexID = __fsub_rn(mergedVertexID, 1.f);
        }
        flags |= radsPerPolarSegment < 0.f ? LEFT_JOIN_CONTOUR_FLAG
                                           : RIGHT_JOIN_CONTOUR_FLAG;
    }

    float2 coord;
    float theta = 0.f;
    if (mergedVertexID == 0.f || mergedVertexID == mergedSegmentCount ||
        (flags & JOIN_TYPE_MASK) > ROUND_JOIN_CONTOUR_FLAG)
    {
        bool isTan0 = mergedVertexID < __fmul_rn(mergedSegmentCount, .5f);
        coord = isTan0 ? p0 : p3;
        theta = rive_atan2(isTan0 ? tan0 : tan1);
    }
    else if (flags & RETROFIT_TRI_STRIP_CONTOUR_FLAG)
    {
        coord = p0;
        if (mergedVertexID >= 8.f)
            coord = p1;
        if (mergedVertexID >= 12.f)
            coord = p2;
        if (mergedVertexID >= 14.f)
            coord = s.joinTangent;
    }
    else
    {
        float T, polarT;
        if (parametricSegmentCount == mergedSegmentCount)
        {
            T = __fdiv_rn(mergedVertexID, parametricSegmentCount);
            polarT = 0.f;
        }
        else
        {
            float2 C = f2sub(p1, p0);
            float2 D = f2sub(p3, p0);
            float2 E = f2sub(p2, p1);
            float2 B = f2sub(E, C);
            float2 A = f2add(f2scale(E, -3.f), D);
            float2 B_ = f2scale(B, __fmul_rn(parametricSegmentCount, 2.f));
            float2 C_ = f2scale(C, __fmul_rn(parametricSegmentCount, parametricSegmentCount));
            float lastParametricID = 0.f;
            float maxParametricID =
                fminf(__fsub_rn(parametricSegmentCount, 1.f), mergedVertexID);
            float2 tan0norm = f2normalize(tan0);
            float absRads = fabsf(radsPerPolarSegment);
            float maxRotation0 = __fmul_rn(__fadd_rn(1.f, mergedVertexID), absRads);
#pragma unroll
            for (int p = 9; p >= 0; --p)
            {
                float testID = __fadd_rn(lastParametricID, (float)(1 << p));
                if (testID <= maxParametricID)
                {
                    float2 testTan = f2add(f2scale(A, testID), B_);
                    testTan = f2add(f2scale(testTan, testID), C_);
                    float cosRotation = f2dot(f2normalize(testTan), tan0norm);
                    float maxRotation =
                        __fadd_rn(__fmul_rn(testID, -absRads), maxRotation0);
                    maxRotation = fminf(maxRotation, kPi);
                    if (cosRotation >= rc_cosf(maxRotation))
                        lastParametricID = testID;
                }
            }
            float parametricT = __fdiv_rn(lastParametricID, parametricSegmentCount);
            float lastPolarID = __fsub_rn(mergedVertexID, lastParametricID);
            float theta0 = rc_acosf(fminf(fmaxf(tan0norm.x, -1.f), 1.f));
            theta0 = tan0norm.y >= 0.f ? theta0 : -theta0;
            theta = __fadd_rn(__fmul_rn(lastPolarID, radsPerPolarSegment), theta0);
            float sn, cs;
            rc_sincosf(theta, &sn, &cs);
            float2 norm = make_float2(sn, -cs);
            float a = f2dot(norm, A), bHalf = f2dot(norm, B), c = f2dot(norm, C);
            float disc = fmaxf(__fsub_rn(__fmul_rn(bHalf, bHalf), __fmul_rn(a, c)), 0.f);
            float q = __fsqrt_rn(disc);
            if (bHalf > 0.f)
                q = -q;
            q = __fsub_rn(q, bHalf);
            float qa5 = __fmul_rn(__fmul_rn(-.5f, q), a);
            float rs, rt;
            if (fabsf(__fadd_rn(__fmul_rn(q, q), qa5)) < fabsf(__fadd_rn(__fmul_rn(a, c), qa5)))
            {
                rs = q;
                rt = a;
            }
            else
            {
                rs = c;
                rt = q;
            }
            polarT = (rt != 0.f) ? __fdiv_rn(rs, rt) : 0.f;
            polarT = fminf(fmaxf(polarT, 0.f), 1.f);
            if (lastPolarID == 0.f)
                polarT = 0.f;
            T = fmaxf(parametricT, polarT);
        }
        float2 abc, bcd;
        coord = eval_cubic_mix(p0, p1, p2, p3, T, abc, bcd);
        if (T != polarT)
            theta = rive_atan2(f2sub(bcd, abc));
    }
    // GLSL mod(theta, 2pi) = theta - 2pi * floor(theta / 2pi)
    uint32_t z;
    if (kFeather && (flags & JOIN_TYPE_MASK) == FEATHER_JOIN_CONTOUR_FLAG)
    {
        // tessellate.glsl:551-559: a feather join leaves its stepping to the
        // draw pass, which needs the join's vertex and segment counts.
        z = ((uint32_t)mergedSegmentCount << 16) | (uint32_t)mergedVertexID;
    }
    else
    {
        z = __float_as_uint(
            __fsub_rn(theta, __fmul_rn(k2Pi, floorf(__fdiv_rn(theta, k2Pi)))));
    }
    return make_uint4(__float_as_uint(coord.x), __float_as_uint(coord.y), z, flags);
}
} // namespace

// One block of 128 threads per GradientSpan of the batch; each thread owns 4
// of the 512 texel columns.
__global__ void __launch_bounds__(128) color_ramp_kernel(BatchTables B)
{
    const uint32_t g = blockIdx.x;
    if (g >= B.totalGradSpans)
        return;
    const uint32_t scene = find_range(B.gradSpanBase, B.sceneCount, g);
    const FlushParams& P = B.scenes[scene];
    const uint32_t s = g - B.gradSpanBase[scene];
    uint4 sp = P.gradSpans[P.firstGradSpan + s];
    uint32_t y = sp.y & ~GRAD_SPAN_FLAGS_MASK;
    if (y >= P.gradDataHeight)
        return;
    float x0 = (float)(sp.x & 0xffffu) * (1.f / 65536.f);
    float x1 = (float)(sp.x >> 16) * (1.f / 65536.f);
    float cx0 = x0, cx3 = x1;
    if (sp.y & GRAD_SPAN_FLAG_LEFT_BORDER)
        cx0 = (sp.y & GRAD_SPAN_FLAG_COMPLEX_BORDER) ? 0.f : x0 - 1.f / kGradTextureWidth;
    if (sp.y & GRAD_SPAN_FLAG_RIGHT_BORDER)
        cx3 = (sp.y & GRAD_SPAN_FLAG_COMPLEX_BORDER) ? 1.f : x1 + 1.f / kGradTextureWidth;
    // Quad edges in texel units (exact: the texture width is a power of two).
    float e0 = cx0 * kGradTextureWidth, e1 = x0 * kGradTextureWidth;
    float e2 = x1 * kGradTextureWidth, e3 = cx3 * kGradTextureWidth;
    float c0[4] = {(float)((sp.z >> 16) & 0xffu) / 255.f, (float)((sp.z >> 8) & 0xffu) / 255.f,
                   (float)(sp.z & 0xffu) / 255.f, (float)(sp.z >> 24) / 255.f};
    float c1[4] = {(float)((sp.w >> 16) & 0xffu) / 255.f, (float)((sp.w >> 8) & 0xffu) / 255.f,
                   (float)(sp.w & 0xffu) / 255.f, (float)(sp.w >> 24) / 255.f};
    uchar4* row = P.grad + (size_t)y * kGradTextureWidth;
    for (int i = threadIdx.x; i < kGradTextureWidth; i += blockDim.x)
    {
        float pc = (float)i + .5f;
        float t;
        if (pc >= e0 && pc < e1)
            t = 0.f;
        else if (pc >= e1 && pc < e2)
            t = (pc - e1) / (e2 - e1);
        else if (pc >= e2 && pc < e3)
            t = 1.f;
        else
            continue;
        float v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            float x = t == 0.f ? c0[k] : (t == 1.f ? c1[k] : c0[k] + (c1[k] - c0[k]) * t);
            v[k] = fminf(fmaxf(x, 0.f), 1.f);
        }
        row[i] = make_uchar4((unsigned char)__float2int_rn(v[0] * 255.f),
                             (unsigned char)__float2int_rn(v[1] * 255.f),
                             (unsigned char)__float2int_rn(v[2] * 255.f),
                             (unsigned char)__float2int_rn(v[3] * 255.f));
    }
}

// One warp per TessVertexSpan of the batch (both its forward and mirrored
// rectangles).
template <bool kFeather>
__device__ __forceinline__ void tessellate(const BatchTables& B)
{
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (gw >= B.totalTessSpans)
        return;
    const uint32_t scene = find_range(B.tessSpanBase, B.sceneCount, gw);
    const FlushParams& P = B.scenes[scene];
    const uint32_t warp = gw - B.tessSpanBase[scene];
    const uint4* sp = P.tessSpans + 4 * (size_t)(P.firstTessSpan + warp);
    SpanSetup s = span_setup<kFeather>(P, sp);
    if (!s.valid)
        return;
    uint4 q2 = sp[2], q3 = sp[3];
    for (int second = 0; second < 2; ++second)
    {
        float y = __uint_as_float(second ? q2.w : q2.z);
        int32_t x0x1 = (int32_t)(second ? q3.y : q3.x);
        int x0 = (int32_t)((uint32_t)x0x1 << 16) >> 16;
        int x1 = x0x1 >> 16;
        if (isnan(y) || x0 == x1 || y < 0.f || y >= (float)P.tessDataHeight)
            continue;
        int rowIdx = (int)y;
        int lo = max(min(x0, x1), 0), hi = min(max(x0, x1), kTessTextureWidth);
        uint32_t flags = s.contourIDWithFlags;
        if (x1 < x0)
            flags |= MIRRORED_CONTOUR_CONTOUR_FLAG;
        uint4* row = P.tess + (size_t)rowIdx * kTessTextureWidth;
        for (int px = lo + lane; px < hi; px += 32)
        {
            float vertexIdx = __fsub_rn(s.totalVertexCount,
                                        fabsf(__fsub_rn((float)x1, __fadd_rn((float)px, .5f))));
            row[px] = tess_vertex<kFeather>(s, vertexIdx, flags);
        }
    }
}

// Resident 256-thread CTAs per SM the tessellation's registers are bounded
// for: 4 (64 registers, a few bytes spilled) tessellates the full-feature
// frame in 0.93 ms against 1.03 ms at the compiler's 74 registers (3 CTAs).
#ifndef RIVE_TESS_MIN_BLOCKS
#define RIVE_TESS_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(256, RIVE_TESS_MIN_BLOCKS) tessellate_kernel(BatchTables B)
{
    tessellate<false>(B);
}

// With feathered-fill softening and feather-join texels.
__global__ void __launch_bounds__(256) tessellate_feather_kernel(BatchTables B)
{
    tessellate<true>(B);
}
// The tessellation pass's device functions on n items, for the parity tests
// (the layouts of oracle_cubic_eval and oracle_math_eval): fn 0..5 the cubic
// functions, 10..13 sin, cos, acos and the cube root.
__global__ void __launch_bounds__(128) tess_math_kernel(int fn, const float* __restrict__ in,
                                                        float* __restrict__ out, uint32_t n)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    constexpr int kIn[6] = {2, 8, 10, 9, 12, 8}, kOut[6] = {1, 2, 1, 2, 1, 4};
    if (fn >= 10)
    {
        const float v = in[i];
        out[i] = fn == 10 ? rc_sinf(v) : fn == 11 ? rc_cosf(v) : fn == 12 ? rc_acosf(v)
                                                                         : rc_cbrtf(v);
        return;
    }
    const float* x = in + (size_t)i * kIn[fn];
    float* y = out + (size_t)i * kOut[fn];
    const float2 p0 = make_float2(x[0], x[1]), p1 = make_float2(x[2], x[3]);
    const float2 p2 = make_float2(x[4], x[5]), p3 = make_float2(x[6], x[7]);
    switch (fn)
    {
        case 0: y[0] = clamped_divide(x[0], x[1]); break;
        case 1: y[0] = cubic_max_height(p0, p1, p2, p3, y[1]); break;
        case 2: y[0] = cubic_local_curvature(p0, p1, p2, p3, x[8], x[9]); break;
        case 3:
        {
            float2 abc, bcd;
            const float2 q = eval_cubic_mix(p0, p1, p2, p3, x[8], abc, bcd);
            y[0] = q.x;
            y[1] = q.y;
            break;
        }
        case 4: y[0] = wang_cubic_segments(p0, p1, p2, p3, make_float4(x[8], x[9], x[10], x[11])); break;
        default:
        {
            float2 t0, t1;
            cubic_tangents(p0, p1, p2, p3, t0, t1);
            y[0] = t0.x;
            y[1] = t0.y;
            y[2] = t1.x;
            y[3] = t1.y;
            break;
        }
    }
}

cudaError_t run_tess_math(int fn, const float* in, float* out, size_t n)
{
    static const int kIn[6] = {2, 8, 10, 9, 12, 8}, kOut[6] = {1, 2, 1, 2, 1, 4};
    if (n == 0)
        return cudaSuccess;
    const size_t inN = n * (fn >= 10 ? 1 : kIn[fn]), outN = n * (fn >= 10 ? 1 : kOut[fn]);
    float *dIn = nullptr, *dOut = nullptr;
    cudaError_t e = cudaMalloc(&dIn, inN * 4);
    if (e == cudaSuccess)
        e = cudaMalloc(&dOut, outN * 4);
    if (e == cudaSuccess)
        e = cudaMemcpy(dIn, in, inN * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
    {
        tess_math_kernel<<<(unsigned)((n + 127) / 128), 128>>>(fn, dIn, dOut, (uint32_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(out, dOut, outN * 4, cudaMemcpyDeviceToHost);
    cudaFree(dIn);
    cudaFree(dOut);
    return e;
}

cudaError_t upload_inverse_feather_lut(const float table[kGaussianTableSize])
{
    return cudaMemcpyToSymbol(g_inverseFeatherLUT, table, sizeof(float) * kGaussianTableSize);
}
} // namespace rivecuda
