// Draw pass of a rasterOrdering flush: patch expansion, triangle set-up, tile
// binning and the raster-ordered pixel resolve.
//
// Reference semantics:
//  * patch expansion: renderer/src/shaders/draw_path.vert:96-422 with
//    unpack_tessellated_path_vertex (draw_path_common.glsl:275-789) over the
//    midpointFan patch (gpu.cpp:446-687: 42 vertices, 72 indices);
//  * rasterisation: Vulkan rules of the reference backend -- pixel centres,
//    top-left ties, clockwise front faces, counterclockwise culled
//    (gpu.cpp:1552-1567, vulkan/draw_pipeline_vulkan.cpp:333-334);
//  * resolve: draw_raster_order_path.frag:14-238 (fp16 coverage keyed by
//    path ID, nonzero/even-odd, nested clip, clip rect, paint colour,
//    advanced blend, src-over, dither).
// The vertex shading takes sin and cos from rive_fp32_math.h, as the
// tessellation does: the sign of an AA outset depends on the last bit of a
// near-zero normal component, so the C restatement of these passes and this
// kernel must evaluate them to the same bits to place the same triangles.
//
// GB300 design: instead of a hardware rasteriser with fragment interlock, the
// flush is tiled. Each triangle is set up once (edge functions with canonical
// anchors, coverage planes) into a 96-byte record; (tile, triangle) pairs are
// radix-sorted by tile, which keeps primitive order inside each tile; then one
// 256-thread CTA per 16x16 tile walks its triangles in order with each thread
// owning one pixel and its pixel-local-storage planes in registers. Raster
// order therefore holds by construction, with no interlock and no atomics.
#include "rive_cuda_internal.cuh"
#include "rive_fp32_math.h"

#include <cuda_fp16.h>

#include <mutex>
#include <type_traits>

namespace rivecuda
{
namespace
{
struct PatchVertexDesc
{
    float localVertexID, outset, fillCoverage;
    float mLocalVertexID, mOutset, mFillCoverage;
    int vertexType;
};

// The midpointFan patch vertex table of gpu.cpp:446-560, by vertex index.
__device__ __forceinline__ PatchVertexDesc patch_vertex_desc(int v)
{
    PatchVertexDesc d;
    if (v < 32)
    {
        int seg = v >> 2, k = v & 3;
        float l = (float)seg, r = l + 1.f;
        d.vertexType = STROKE_VERTEX;
        switch (k)
        {
            case 0:
                d.localVertexID = l; d.outset = -1.f; d.fillCoverage = 1.f;
                d.mLocalVertexID = r - 1.f; d.mOutset = -1.f; d.mFillCoverage = 1.f;
                break;
            case 1:
                d.localVertexID = l; d.outset = 1.f; d.fillCoverage = 0.f;
                d.mLocalVertexID = l - 1.f; d.mOutset = -1.f; d.mFillCoverage = 1.f;
                break;
            case 2:
                d.localVertexID = r; d.outset = -1.f; d.fillCoverage = 1.f;
                d.mLocalVertexID = r - 1.f; d.mOutset = 1.f; d.mFillCoverage = 0.f;
                break;
            default:
                d.localVertexID = r; d.outset = 1.f; d.fillCoverage = 0.f;
                d.mLocalVertexID = l - 1.f; d.mOutset = 1.f; d.mFillCoverage = 0.f;
                break;
        }
    }
    else if (v < 41)
    {
        float i = (float)(v - 32);
        d.vertexType = FAN_VERTEX;
        d.localVertexID = i; d.outset = -1.f; d.fillCoverage = 1.f;
        d.mLocalVertexID = i - 1.f; d.mOutset = -1.f; d.mFillCoverage = 1.f;
    }
    else
    {
        d.vertexType = FAN_MIDPOINT_VERTEX;
        d.localVertexID = 0.f; d.outset = 0.f; d.fillCoverage = 1.f;
        d.mLocalVertexID = 0.f; d.mOutset = 0.f; d.mFillCoverage = 1.f;
    }
    return d;
}

// The midpointFan index table (gpu.cpp:600-680), by triangle index.
__device__ __forceinline__ void patch_triangle(int t, int& a, int& b, int& c)
{
    if (t < 16)
    {
        int e = (t >> 1) * 4;
        if ((t & 1) == 0) { a = e; b = e + 1; c = e + 2; }
        else { a = e + 2; b = e + 1; c = e + 3; }
        return;
    }
    // Middle-out fan over the 9 fan vertices (32..40), then the triangle to
    // the contour midpoint (41).
    switch (t)
    {
        case 16: a = 32; b = 33; c = 34; return;
        case 17: a = 34; b = 35; c = 36; return;
        case 18: a = 36; b = 37; c = 38; return;
        case 19: a = 38; b = 39; c = 40; return;
        case 20: a = 32; b = 34; c = 36; return;
        case 21: a = 36; b = 38; c = 40; return;
        case 22: a = 32; b = 36; c = 40; return;
        default: a = 32; b = 40; c = 41; return;
    }
}

// The outerCurves patch vertex table (gpu.cpp:446-560, PatchType::outerCurves):
// 17 segments (16 curve segments and a zero-length bowtie join), a centred
// AA ramp on each side of the curve (coverage 1/2 on the curve), and a fan
// over the 16 curve segments; no midpoint vertex.
__device__ __forceinline__ PatchVertexDesc outer_vertex_desc(int v)
{
    PatchVertexDesc d;
    if (v < 2 * 4 * kOuterPatchSegmentSpan)
    {
        const bool bottom = v >= 4 * kOuterPatchSegmentSpan;
        const int u = bottom ? v - 4 * kOuterPatchSegmentSpan : v;
        const float l = (float)(u >> 2), r = l + 1.f;
        d.vertexType = STROKE_VERTEX;
        if (!bottom)
        {
            switch (u & 3)
            {
                case 0:
                    d.localVertexID = l; d.outset = 0.f; d.fillCoverage = .5f;
                    d.mLocalVertexID = r; d.mOutset = 0.f; d.mFillCoverage = .5f;
                    break;
                case 1:
                    d.localVertexID = l; d.outset = 1.f; d.fillCoverage = 0.f;
                    d.mLocalVertexID = l; d.mOutset = 0.f; d.mFillCoverage = .5f;
                    break;
                case 2:
                    d.localVertexID = r; d.outset = 0.f; d.fillCoverage = .5f;
                    d.mLocalVertexID = r; d.mOutset = 1.f; d.mFillCoverage = 0.f;
                    break;
                default:
                    d.localVertexID = r; d.outset = 1.f; d.fillCoverage = 0.f;
                    d.mLocalVertexID = l; d.mOutset = 1.f; d.mFillCoverage = 0.f;
                    break;
            }
        }
        else
        {
            switch (u & 3)
            {
                case 0:
                    d.localVertexID = l; d.outset = -0.f; d.fillCoverage = .5f;
                    d.mLocalVertexID = r; d.mOutset = -0.f; d.mFillCoverage = .5f;
                    break;
                case 1:
                    d.localVertexID = r; d.outset = -0.f; d.fillCoverage = .5f;
                    d.mLocalVertexID = r; d.mOutset = -1.f; d.mFillCoverage = 0.f;
                    break;
                case 2:
                    d.localVertexID = l; d.outset = -1.f; d.fillCoverage = 0.f;
                    d.mLocalVertexID = l; d.mOutset = -0.f; d.mFillCoverage = .5f;
                    break;
                default:
                    d.localVertexID = r; d.outset = -1.f; d.fillCoverage = 0.f;
                    d.mLocalVertexID = l; d.mOutset = -1.f; d.mFillCoverage = 0.f;
                    break;
            }
        }
    }
    else
    {
        const float i = (float)(v - 2 * 4 * kOuterPatchSegmentSpan);
        d.vertexType = FAN_VERTEX;
        d.localVertexID = i; d.outset = 0.f; d.fillCoverage = 1.f;
        d.mLocalVertexID = i; d.mOutset = 0.f; d.mFillCoverage = 1.f;
    }
    return d;
}

// The outerCurves index table, by triangle index: the top ramp (pattern
// 0,1,2 / 2,1,3), the bottom ramp (0,2,1 / 1,2,3), then the middle-out fan.
__device__ __forceinline__ void outer_triangle(int t, int& a, int& b, int& c)
{
    constexpr int kRamp = 2 * kOuterPatchSegmentSpan;
    if (t < kRamp)
    {
        const int e = (t >> 1) * 4;
        if ((t & 1) == 0) { a = e; b = e + 1; c = e + 2; }
        else { a = e + 2; b = e + 1; c = e + 3; }
        return;
    }
    if (t < 2 * kRamp)
    {
        const int u = t - kRamp;
        const int e = 4 * kOuterPatchSegmentSpan + (u >> 1) * 4;
        if ((u & 1) == 0) { a = e; b = e + 2; c = e + 1; }
        else { a = e + 1; b = e + 2; c = e + 3; }
        return;
    }
    // Middle-out fan over the 17 fan vertices: steps 1, 2, 4, 8.
    const int fan = 8 * kOuterPatchSegmentSpan;
    const int u = t - 2 * kRamp;
    const int step = u < 8 ? 1 : (u < 12 ? 2 : (u < 14 ? 4 : 8));
    const int first = u < 8 ? 0 : (u < 12 ? 8 : (u < 14 ? 12 : 14));
    const int i = (u - first) * 2 * step;
    a = fan + i;
    b = fan + i + step;
    c = fan + i + 2 * step;
}

// The midpointFanCenterAA patch vertex table (gpu.cpp:446-560,
// PatchType::midpointFanCenterAA), by vertex index: an AA ramp centred on the
// curve on each side (coverage 1/2 on the curve), the 9-vertex fan and the
// contour midpoint. Feathered fills draw with it.
__device__ __forceinline__ PatchVertexDesc center_vertex_desc(int v)
{
    constexpr int kRampVerts = 4 * kPatchSegmentSpan;
    PatchVertexDesc d;
    auto set = [&d](float l, float o, float c, float ml, float mo, float mc) {
        d.localVertexID = l; d.outset = o; d.fillCoverage = c;
        d.mLocalVertexID = ml; d.mOutset = mo; d.mFillCoverage = mc;
    };
    if (v < 2 * kRampVerts)
    {
        const bool bottom = v >= kRampVerts;
        const int u = bottom ? v - kRampVerts : v;
        const float l = (float)(u >> 2), r = l + 1.f;
        d.vertexType = STROKE_VERTEX;
        if (!bottom)
        {
            switch (u & 3)
            {
                case 0: set(l, 0.f, .5f, r - 1.f, 0.f, .5f); break;
                case 1: set(l, 1.f, 0.f, l - 1.f, 0.f, .5f); break;
                case 2: set(r, 0.f, .5f, r - 1.f, 1.f, 0.f); break;
                default: set(r, 1.f, 0.f, l - 1.f, 1.f, 0.f); break;
            }
        }
        else
        {
            switch (u & 3)
            {
                case 0: set(l, -0.f, .5f, r - 1.f, -0.f, .5f); break;
                case 1: set(r, -0.f, .5f, r - 1.f, -1.f, 0.f); break;
                case 2: set(l, -1.f, 0.f, l - 1.f, -0.f, .5f); break;
                default: set(r, -1.f, 0.f, l - 1.f, -1.f, 0.f); break;
            }
        }
    }
    else if (v < 2 * kRampVerts + kPatchSegmentSpan + 1)
    {
        const float i = (float)(v - 2 * kRampVerts);
        d.vertexType = FAN_VERTEX;
        set(i, 0.f, 1.f, i - 1.f, 0.f, 1.f);
    }
    else
    {
        d.vertexType = FAN_MIDPOINT_VERTEX;
        set(0.f, 0.f, 1.f, 0.f, 0.f, 1.f);
    }
    return d;
}

// The midpointFanCenterAA index table, by triangle index: the top ramp
// (0,1,2 / 2,1,3 per segment), the bottom ramp (0,2,1 / 1,2,3), the
// middle-out fan (steps 1, 2, 4) and the triangle to the midpoint.
__device__ __forceinline__ void center_triangle(int t, int& a, int& b, int& c)
{
    constexpr int kRamp = 2 * kPatchSegmentSpan;
    if (t < kRamp)
    {
        const int e = (t >> 1) * 4;
        if ((t & 1) == 0) { a = e; b = e + 1; c = e + 2; }
        else { a = e + 2; b = e + 1; c = e + 3; }
        return;
    }
    if (t < 2 * kRamp)
    {
        const int u = t - kRamp;
        const int e = 4 * kPatchSegmentSpan + (u >> 1) * 4;
        if ((u & 1) == 0) { a = e; b = e + 2; c = e + 1; }
        else { a = e + 1; b = e + 2; c = e + 3; }
        return;
    }
    const int fan = 8 * kPatchSegmentSpan;
    const int u = t - 2 * kRamp;
    if (u == 7)
    {
        a = fan;
        b = fan + kPatchSegmentSpan;
        c = fan + kPatchSegmentSpan + 1;
        return;
    }
    const int step = u < 4 ? 1 : (u < 6 ? 2 : 4);
    const int first = u < 4 ? 0 : (u < 6 ? 4 : 6);
    const int i = (u - first) * 2 * step;
    a = fan + i;
    b = fan + i + step;
    c = fan + i + 2 * step;
}

__device__ __forceinline__ float2 mat_mul(float4 m, float2 v)
{
    // float2x2 columns (m.x, m.y) and (m.z, m.w).
    return make_float2(__fadd_rn(__fmul_rn(m.x, v.x), __fmul_rn(m.z, v.y)),
                       __fadd_rn(__fmul_rn(m.y, v.x), __fmul_rn(m.w, v.y)));
}

// draw_path_common.glsl:267-274
__device__ __forceinline__ float manhattan_pixel_width(float4 M, float2 n)
{
    float2 v = mat_mul(M, n);
    return __fmul_rn(__fadd_rn(fabsf(v.x), fabsf(v.y)),
                     __fdiv_rn(1.f, __fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y))));
}

__device__ __forceinline__ float signf(float x)
{
    return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f);
}

struct VertexOut
{
    float2 pos;
    float2 cov;
    uint32_t pathID;
    bool discard;
};

// GLSL mod(x, y) = x - y * floor(x / y)
__device__ __forceinline__ float glsl_mod(float x, float y)
{
    return __fsub_rn(x, __fmul_rn(y, floorf(__fdiv_rn(x, y))));
}

// pack_feathered_fill_coverages (draw_path_common.glsl:107-149): a spoke of a
// feather join carries the corner's angle as (cotTheta, y0) and its position
// in the corner's local frame as (x, y).
__device__ void pack_feathered_fill_coverages(float cornerTheta, float2 spokeNorm, float outset,
                                              float2& cov, float2& cov2)
{
    const float ao = fabsf(outset);
    const float cx = __fmul_rn(__fsub_rn(1.f, __fmul_rn(spokeNorm.x, ao)), .5f);
    const float cy = __fmul_rn(__fsub_rn(1.f, __fmul_rn(spokeNorm.y, ao)), .5f);
    float cotTheta = 0.f, y0 = 0.f;
    if (!(fabsf(__fsub_rn(cornerTheta, kPi * .5f)) < 1.f / kHorizontalCotangentThreshold))
    {
        const float tanTheta = tanf(cornerTheta);
        cotTheta = __fdiv_rn(signf(__fsub_rn(kPi * .5f, cornerTheta)),
                             fmaxf(fabsf(tanTheta), 1.f / kHorizontalCotangentValue));
        y0 = cotTheta >= 0.f ? __fsub_rn(cy, __fmul_rn(__fsub_rn(1.f, cx), tanTheta))
                             : __fadd_rn(cy, __fmul_rn(cx, tanTheta));
    }
    cov = make_float2(__fadd_rn(fmaxf(cx, 0.f), kFeatherXCoordBias),
                      __fadd_rn(-cy, kFeatherCoverageBias));
    cov2 = make_float2(cotTheta, y0);
}

__device__ __forceinline__ bool tess_fetch(const FlushParams& P, long long idx, uint4& out)
{
    if (idx < 0 || idx >= (long long)P.tessDataHeight * kTessTextureWidth)
    {
        atomicOr(P.error, ERR_BAD_TESS_INDEX);
        return false;
    }
    out = P.tess[idx];
    return true;
}

// unpack_tessellated_path_vertex for a midpointFan patch vertex, plus the
// position math of @drawVertexMain. Returns false on a malformed input.
// kFeather: compiled with the feather paths (ENABLE_FEATHER); without it a
// path's feather radius is ignored.
template <bool kFeather>
__device__ bool shade_patch_vertex(const FlushParams& P,
                                   const PatchVertexDesc& pv,
                                   int span,
                                   uint32_t instanceID,
                                   VertexOut& o,
                                   float2& cov2) // feathered fills: the corner's cotTheta, y0
{
    int localVertexID = (int)pv.localVertexID;
    float outset = pv.outset;
    float fillCoverage = pv.fillCoverage;
    int vertexIDOnContour = min(localVertexID, span - 1);
    long long tessVertexIdx = (long long)instanceID * span + vertexIDOnContour;
    uint4 tv;
    if (!tess_fetch(P, tessVertexIdx, tv))
        return false;
    uint32_t flags = tv.w;
    uint32_t contourID = max(flags & CONTOUR_ID_MASK, 1u);
    if (contourID > P.contourCount)
    {
        atomicOr(P.error, ERR_BAD_CONTOUR);
        return false;
    }
    uint4 cd = P.contours[P.firstContour + contourID - 1];
    float2 midpoint = make_float2(__uint_as_float(cd.x), __uint_as_float(cd.y));
    uint32_t pathID = cd.z & 0xffffu;
    uint32_t vertexIndex0 = cd.w;
    if (pathID >= P.pathCount)
    {
        atomicOr(P.error, ERR_BAD_PATH);
        return false;
    }
    const uint4* path = P.paths + 4 * (size_t)(P.firstPath + pathID);
    uint4 r0 = path[0], r1 = path[1];
    float4 M = make_float4(__uint_as_float(r0.x), __uint_as_float(r0.y),
                           __uint_as_float(r0.z), __uint_as_float(r0.w));
    float2 translate = make_float2(__uint_as_float(r1.x), __uint_as_float(r1.y));
    float strokeRadius = __uint_as_float(r1.z);
    float featherRadius = kFeather ? __uint_as_float(r1.w) : 0.f;
    uint32_t mirrored = flags & MIRRORED_CONTOUR_CONTOUR_FLAG;
    if (mirrored)
    {
        localVertexID = (int)pv.mLocalVertexID;
        outset = pv.mOutset;
        fillCoverage = pv.mFillCoverage;
    }
    if (localVertexID != vertexIDOnContour)
    {
        long long repl = tessVertexIdx + localVertexID - vertexIDOnContour;
        uint4 rv;
        if (!tess_fetch(P, repl, rv))
            return false;
        if ((rv.w & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)) !=
            (flags & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)))
        {
            bool isClosed = strokeRadius == 0.f || midpoint.x != 0.f;
            if (isClosed)
            {
                tessVertexIdx = vertexIndex0;
                if (!tess_fetch(P, tessVertexIdx, tv))
                    return false;
            }
        }
        else
        {
            tessVertexIdx = repl;
            tv = rv;
        }
        flags = (tv.w & ~MIRRORED_CONTOUR_CONTOUR_FLAG) | mirrored;
    }
    float theta;
    float joinEdge0Theta = 0.f, joinCornerTheta = 0.f;
    const bool featherJoin = kFeather && (flags & JOIN_TYPE_MASK) == FEATHER_JOIN_CONTOUR_FLAG &&
                             pv.vertexType == STROKE_VERTEX;
    if (featherJoin)
    {
        // draw_path_common.glsl:372-468: a feather join steps between the
        // tangents of the tessellation vertices just before and after it:
        // backward segments first (erasing coverage outside the corner), one
        // zero-width helper, then forward segments.
        float joinVertexID = (float)(tv.z & 0xffffu);
        float joinSegmentCount = (float)(tv.z >> 16);
        int off0 = (int)(-joinVertexID - 1.f);
        int off1 = (int)(__fadd_rn(__fsub_rn(joinSegmentCount, joinVertexID), 1.f));
        if (flags & MIRRORED_CONTOUR_CONTOUR_FLAG)
        {
            off0 = -off0;
            off1 = -off1;
        }
        uint4 before, after;
        if (!tess_fetch(P, tessVertexIdx + off0, before) ||
            !tess_fetch(P, tessVertexIdx + off1, after))
            return false;
        if ((after.w & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)) !=
            (before.w & (MIRRORED_CONTOUR_CONTOUR_FLAG | 0xffffu)))
        {
            if (!tess_fetch(P, vertexIndex0, after))
                return false;
        }
        joinEdge0Theta = __uint_as_float(before.z);
        const float joinEdge1Theta = __uint_as_float(after.z);
        joinCornerTheta = __fsub_rn(joinEdge1Theta, joinEdge0Theta);
        if (fabsf(joinCornerTheta) > kPi)
            joinCornerTheta = __fsub_rn(joinCornerTheta, __fmul_rn(k2Pi, signf(joinCornerTheta)));
        const float nonHelper =
            __fsub_rn(__fadd_rn(joinSegmentCount, 1.f), kFeatherJoinHelperVertexCount);
        const float forward =
            fminf(fmaxf(rintf(__fmul_rn(__fdiv_rn(fabsf(joinCornerTheta), kPi), nonHelper)), 1.f),
                  __fsub_rn(nonHelper, 1.f));
        const float backward = __fsub_rn(nonHelper, forward);
        if (joinVertexID <= backward)
        {
            joinCornerTheta = -__fsub_rn(__fmul_rn(kPi, signf(joinCornerTheta)), joinCornerTheta);
            joinSegmentCount = backward;
            if (joinVertexID == backward)
                outset = -outset;
        }
        else if (joinVertexID == __fadd_rn(backward, 1.f))
        {
            joinVertexID = 0.f;
            joinSegmentCount = 0.f;
            outset = 0.f;
        }
        else
        {
            joinVertexID = __fsub_rn(joinVertexID, __fadd_rn(backward, 2.f));
            joinSegmentCount = forward;
        }
        theta = joinVertexID == joinSegmentCount
                    ? joinEdge1Theta
                    : __fadd_rn(joinEdge0Theta,
                                __fmul_rn(joinCornerTheta, __fdiv_rn(joinVertexID, joinSegmentCount)));
    }
    else
    {
        theta = __uint_as_float(tv.z);
    }
    float sn, cs;
    rc_sincosf(theta, &sn, &cs);
    float2 norm = make_float2(sn, -cs);
    float2 origin = make_float2(__uint_as_float(tv.x), __uint_as_float(tv.y));
    float2 offset = make_float2(0.f, 0.f);
    float2 cov;
    cov2 = make_float2(0.f, 0.f);
    o.discard = false;
    if (featherRadius != 0.f)
    {
        // draw_path_common.glsl:474-485: never feather harder than 1.5
        // standard deviations across half a pixel.
        const float2 mn = mat_mul(M, norm);
        const float len = __fsqrt_rn(__fadd_rn(__fmul_rn(mn.x, mn.x), __fmul_rn(mn.y, mn.y)));
        featherRadius = fmaxf(featherRadius, __fdiv_rn(kGaussianStddevs / 3.f, len));
    }
    if (strokeRadius != 0.f)
    {
        float detM = __fsub_rn(__fmul_rn(M.x, M.w), __fmul_rn(M.z, M.y));
        outset = __fmul_rn(outset, signf(detM));
        if (flags & LEFT_JOIN_CONTOUR_FLAG)
            outset = fminf(outset, 0.f);
        if (flags & RIGHT_JOIN_CONTOUR_FLAG)
            outset = fmaxf(outset, 0.f);
        float aaRadius = featherRadius != 0.f ? featherRadius
                                              : __fmul_rn(manhattan_pixel_width(M, norm), kAARadius);
        float globalCoverage = 1.f;
        if (aaRadius > strokeRadius && featherRadius == 0.f)
        {
            globalCoverage = __fdiv_rn(strokeRadius, aaRadius);
            strokeRadius = aaRadius;
        }
        float sr = __fadd_rn(strokeRadius, aaRadius);
        float2 vertexOffset = make_float2(__fmul_rn(norm.x, sr), __fmul_rn(norm.y, sr));
        float x = __fmul_rn(outset, sr);
        float k = __fdiv_rn(1.f, __fmul_rn(aaRadius, 2.f));
        cov.x = __fadd_rn(__fmul_rn(k, __fadd_rn(x, strokeRadius)), .5f);
        cov.y = __fadd_rn(__fmul_rn(k, __fadd_rn(-x, strokeRadius)), .5f);
        uint32_t joinType = flags & JOIN_TYPE_MASK;
        if (joinType > ROUND_JOIN_CONTOUR_FLAG)
        {
            int peekDir = 2;
            if (!(flags & JOIN_TANGENT_0_CONTOUR_FLAG))
                peekDir = -peekDir;
            if (flags & MIRRORED_CONTOUR_CONTOUR_FLAG)
                peekDir = -peekDir;
            uint4 ov;
            if (!tess_fetch(P, tessVertexIdx + peekDir, ov))
                return false;
            float otherTheta = __uint_as_float(ov.z);
            float joinAngle = fabsf(__fsub_rn(otherTheta, theta));
            if (joinAngle > kPi)
                joinAngle = __fsub_rn(k2Pi, joinAngle);
            bool isTan0 = (flags & JOIN_TANGENT_0_CONTOUR_FLAG) != 0;
            bool isLeft = (flags & LEFT_JOIN_CONTOUR_FLAG) != 0;
            float bisectTheta =
                __fadd_rn(__fmul_rn(joinAngle, isTan0 == isLeft ? -.5f : .5f), theta);
            float bs, bc;
            rc_sincosf(bisectTheta, &bs, &bc);
            float2 bisector = make_float2(bs, -bc);
            float bisectPixelWidth = manhattan_pixel_width(M, bisector);
            float miterRatio = rc_cosf(__fmul_rn(joinAngle, .5f));
            float clipRadius;
            if (joinType == MITER_CLIP_JOIN_CONTOUR_FLAG ||
                (joinType == MITER_REVERT_JOIN_CONTOUR_FLAG && miterRatio >= .25f))
            {
                float inverseLimit = (flags & EMULATED_STROKE_CAP_CONTOUR_FLAG) ? 1.f : .25f;
                clipRadius = __fmul_rn(strokeRadius,
                                       __fdiv_rn(1.f, fmaxf(miterRatio, inverseLimit)));
            }
            else
            {
                clipRadius = __fadd_rn(__fmul_rn(strokeRadius, miterRatio),
                                       __fmul_rn(bisectPixelWidth, .5f));
            }
            float clipAARadius = __fadd_rn(clipRadius, __fmul_rn(bisectPixelWidth, kAARadius));
            if (flags & JOIN_TANGENT_INNER_CONTOUR_FLAG)
            {
                float strokeAARadius = __fadd_rn(strokeRadius, aaRadius);
                float slop = __fmul_rn(aaRadius, .125f);
                if (strokeAARadius <= __fadd_rn(__fmul_rn(clipAARadius, miterRatio), slop))
                {
                    float miterAARadius = __fmul_rn(strokeAARadius, __fdiv_rn(1.f, miterRatio));
                    vertexOffset = make_float2(__fmul_rn(bisector.x, miterAARadius),
                                               __fmul_rn(bisector.y, miterAARadius));
                }
                else
                {
                    float2 bo = make_float2(__fmul_rn(bisector.x, clipAARadius),
                                            __fmul_rn(bisector.y, clipAARadius));
                    float kx = __fadd_rn(__fmul_rn(vertexOffset.x, vertexOffset.x),
                                         __fmul_rn(vertexOffset.y, vertexOffset.y));
                    float ky = __fadd_rn(__fmul_rn(bo.x, bo.x), __fmul_rn(bo.y, bo.y));
                    // Row vector k times inverse of the matrix with columns
                    // vertexOffset and bo; inverse() as the reference's own
                    // polyfills define it, the adjoint times 1 / determinant.
                    float det = __fsub_rn(__fmul_rn(vertexOffset.x, bo.y),
                                          __fmul_rn(bo.x, vertexOffset.y));
                    float invDet = __fdiv_rn(1.f, det);
                    float i00 = __fmul_rn(bo.y, invDet), i01 = __fmul_rn(-vertexOffset.y, invDet);
                    float i10 = __fmul_rn(-bo.x, invDet), i11 = __fmul_rn(vertexOffset.x, invDet);
                    vertexOffset = make_float2(__fadd_rn(__fmul_rn(kx, i00), __fmul_rn(ky, i01)),
                                               __fadd_rn(__fmul_rn(kx, i10), __fmul_rn(ky, i11)));
                }
            }
            float ao = fabsf(outset);
            float2 pt = make_float2(__fmul_rn(vertexOffset.x, ao), __fmul_rn(vertexOffset.y, ao));
            float clipDistance =
                __fdiv_rn(__fsub_rn(clipAARadius,
                                    __fadd_rn(__fmul_rn(pt.x, bisector.x), __fmul_rn(pt.y, bisector.y))),
                          __fmul_rn(bisectPixelWidth, kAARadius * 2.f));
            if (flags & LEFT_JOIN_CONTOUR_FLAG)
                cov.y = clipDistance;
            else
                cov.x = clipDistance;
        }
        cov.x = __fmul_rn(cov.x, globalCoverage);
        cov.y = __fmul_rn(cov.y, globalCoverage);
        cov.y = fmaxf(cov.y, 1e-4f);
        if (featherRadius != 0.f)
            cov.x = __fsub_rn(kFeatherCoverageBias, cov.x); // marks a feathered stroke
        offset = mat_mul(M, make_float2(__fmul_rn(vertexOffset.x, outset),
                                        __fmul_rn(vertexOffset.y, outset)));
        if (pv.vertexType != STROKE_VERTEX)
            o.discard = true;
    }
    else
    {
        cov = make_float2(fillCoverage, -1.f);
        if (featherRadius != 0.f)
        {
            // draw_path_common.glsl:659-741: a feathered edge; the spokes of a
            // feather join carry their corner.
            cov.y = kFeatherCoverageBias;
            cov2 = make_float2(kHorizontalCotangentValue, fillCoverage);
            if (featherJoin)
            {
                if (joinCornerTheta < 0.f)
                {
                    joinEdge0Theta = __fadd_rn(joinEdge0Theta, joinCornerTheta);
                    joinCornerTheta = -joinCornerTheta;
                }
                float spoke = __fsub_rn(theta, joinEdge0Theta);
                spoke = __fsub_rn(glsl_mod(__fadd_rn(spoke, kPi * .5f), k2Pi), kPi * .5f);
                spoke = fminf(fmaxf(spoke, 0.f), joinCornerTheta);
                if (spoke > __fmul_rn(joinCornerTheta, .5f))
                    spoke = __fsub_rn(joinCornerTheta, spoke);
                float ss, sc;
                rc_sincosf(spoke, &ss, &sc);
                pack_feathered_fill_coverages(joinCornerTheta, make_float2(ss, sc), outset, cov,
                                              cov2);
            }
            const float r = __fmul_rn(outset, featherRadius);
            offset = mat_mul(M, make_float2(__fmul_rn(norm.x, r), __fmul_rn(norm.y, r)));
        }
        else
        {
            // sign(MUL(outset * norm, inverse(M))) with inverse() as the
            // reference's own polyfills define it, the adjoint times
            // 1 / determinant: where the product cancels to within a
            // rounding step, the form decides the sign (and so which side of
            // the vertex the AA ramp goes), so it is the same form, rounded
            // the same way, as the C restatement of this pass.
            float2 on = make_float2(__fmul_rn(norm.x, outset), __fmul_rn(norm.y, outset));
            float det = __fsub_rn(__fmul_rn(M.x, M.w), __fmul_rn(M.z, M.y));
            float invDet = __fdiv_rn(1.f, det);
            float i00 = __fmul_rn(M.w, invDet), i01 = __fmul_rn(-M.y, invDet);
            float i10 = __fmul_rn(-M.z, invDet), i11 = __fmul_rn(M.x, invDet);
            float rx = __fadd_rn(__fmul_rn(on.x, i00), __fmul_rn(on.y, i01));
            float ry = __fadd_rn(__fmul_rn(on.x, i10), __fmul_rn(on.y, i11));
            offset = make_float2(signf(rx) * kAARadius, signf(ry) * kAARadius);
        }
        if (((flags & MIRRORED_CONTOUR_CONTOUR_FLAG) != 0) !=
            ((flags & NEGATE_PATH_FILL_COVERAGE_FLAG) != 0))
            cov.x = -cov.x;
        if (pv.vertexType == FAN_MIDPOINT_VERTEX)
            origin = midpoint;
        if ((flags & RETROFIT_TRI_STRIP_CONTOUR_FLAG) && pv.vertexType != FAN_VERTEX)
            o.discard = true;
    }
    if (P.wireframe)
        cov = make_float2(1.f, -1.f);
    float2 mo = mat_mul(M, origin);
    o.pos = make_float2(__fadd_rn(__fadd_rn(mo.x, offset.x), translate.x),
                        __fadd_rn(__fadd_rn(mo.y, offset.y), translate.y));
    if (kFeather && P.atlasMode)
    {
        // render_atlas.glsl:30-35: into the feather atlas by the path's atlas
        // transform (PathData words 9-11: scale, translate x, translate y).
        const uint4 r2 = path[2];
        const float sc = __uint_as_float(r2.y);
        o.pos = make_float2(__fadd_rn(__fmul_rn(o.pos.x, sc), __uint_as_float(r2.z)),
                            __fadd_rn(__fmul_rn(o.pos.y, sc), __uint_as_float(r2.w)));
    }
    o.cov = cov;
    o.pathID = pathID;
    return true;
}

// E(p) = A * (p.x - ax) + B * (p.y - ay), evaluated identically by the binner
// and the raster so their tile/pixel decisions agree.
__device__ __forceinline__ float edge_eval(float4 e, float px, float py)
{
    return __fmaf_rn(e.z, __fsub_rn(px, e.x), __fmul_rn(e.w, __fsub_rn(py, e.y)));
}

// Builds the oriented, canonically-anchored edge P->Q of a triangle.
__device__ __forceinline__ float4 make_edge(float2 P, float2 Q)
{
    bool pFirst = P.y < Q.y || (P.y == Q.y && P.x < Q.x);
    float2 a = pFirst ? P : Q, b = pFirst ? Q : P;
    float A = -(b.y - a.y), B = b.x - a.x; // exact: snapped coordinates
    if (!pFirst)
    {
        A = -A;
        B = -B;
    }
    return make_float4(a.x, a.y, A, B);
}

// Tile-local edge functions. The raster tests pixel (lx, ly) of a tile (lx,
// ly = 0..15 pixel offsets from the tile's first pixel centre) as
//   E = fma(A, lx, fma(B, ly, C)),  C = edge_eval at the tile's first centre.
// The two triangles sharing an edge hold bitwise-negated (A, B, C), so their
// E values are exact negations and the fill stays watertight. Tile counting,
// binning and the raster's block masks all use this same expression; float
// rounding is monotone in lx and ly, so testing the corner of a rectangle
// that maximises E never rejects a pixel the raster would accept.
__device__ __forceinline__ float tile_edge_origin(float4 e, int tx, int ty, int tileLog2)
{
    return edge_eval(e, (float)(tx << tileLog2) + .5f, (float)(ty << tileLog2) + .5f);
}

__device__ __forceinline__ float local_edge(float c, float a, float b, float lx, float ly)
{
    return __fmaf_rn(a, lx, __fmaf_rn(b, ly, c));
}

__device__ __forceinline__ bool local_inside(float a, float b, float E)
{
    // Top-left tie rule for clockwise (y-down) triangles: edge direction
    // (dx, dy) = (B, -A); inclusive when dy < 0, or dy == 0 and dx > 0.
    return E > 0.f || (E == 0.f && (a > 0.f || (a == 0.f && b > 0.f)));
}

// Can any pixel of the tile-local rectangle [x0, x1) x [y0, y1) lie inside
// all three edges (tile constants c[k], slopes e[k].z, e[k].w)?
__device__ __forceinline__ bool local_rect_overlaps(const float* c, const float4* e, int x0, int x1,
                                                    int y0, int y1)
{
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        const float lx = (float)(e[k].z > 0.f ? x1 - 1 : x0);
        const float ly = (float)(e[k].w > 0.f ? y1 - 1 : y0);
        if (local_edge(c[k], e[k].z, e[k].w, lx, ly) < 0.f)
            return false;
    }
    return true;
}

__device__ __forceinline__ bool tile_overlaps(const float4* e, int4 bb, int tx, int ty,
                                              int tileLog2)
{
    const int ts = 1 << tileLog2;
    const int ox = tx << tileLog2, oy = ty << tileLog2;
    const float c[3] = {tile_edge_origin(e[0], tx, ty, tileLog2),
                        tile_edge_origin(e[1], tx, ty, tileLog2),
                        tile_edge_origin(e[2], tx, ty, tileLog2)};
    return local_rect_overlaps(c, e, max(ox, bb.x) - ox, min(ox + ts, bb.z) - ox,
                               max(oy, bb.y) - oy, min(oy + ts, bb.w) - oy);
}

__device__ __forceinline__ int4 unpack_bbox(uint4 meta)
{
    return make_int4((int)(meta.y & 0xffffu), (int)(meta.z & 0xffffu), (int)(meta.y >> 16),
                     (int)(meta.z >> 16));
}
} // namespace

// Sets up one triangle for the tile raster: snaps the vertices to the
// 1/256-pixel grid, culls counterclockwise and degenerate triangles (exact
// integer area), clips the pixel box to the target, and builds the edge
// functions and coverage planes. Returns false for a triangle that draws
// nothing (bb stays empty).
// `clip` bounds the pixels (an atlas batch's scissor; the canvas always).
// `twoSided` keeps counterclockwise triangles (the atlas fill pipeline culls
// nothing, gpu.hpp:2076-2077): they are turned clockwise and marked
// FEATURE_ATLAS_NEGATE, since a back-facing atlas fill subtracts coverage.
__device__ bool setup_triangle(const FlushParams& P,
                               const VertexOut& A,
                               const VertexOut& Bv,
                               const VertexOut& Cv,
                               uint32_t features,
                               uint32_t scene,
                               TriRecord& T,
                               int4& bb,
                               float4* featherPlanes = nullptr,
                               float2 zwA = {}, float2 zwB = {}, float2 zwC = {},
                               int4 clip = make_int4(0, 0, 0x7fffffff, 0x7fffffff),
                               bool twoSided = false)
{
    bb = make_int4(0, 0, 0, 0);
    if (A.discard || Bv.discard || Cv.discard)
        return false;
    float m = fmaxf(fmaxf(fmaxf(fabsf(A.pos.x), fabsf(A.pos.y)), fmaxf(fabsf(Bv.pos.x), fabsf(Bv.pos.y))),
                    fmaxf(fabsf(Cv.pos.x), fabsf(Cv.pos.y)));
    if (!(m < 32768.f)) // NaN or outside the exact snapping range
    {
        if (!isnan(m))
            atomicOr(P.error, ERR_COORD_RANGE);
        return false;
    }
    const VertexOut* pB = &Bv;
    const VertexOut* pC = &Cv;
    int X1 = __float2int_rn(Bv.pos.x * 256.f), Y1 = __float2int_rn(Bv.pos.y * 256.f);
    int X2 = __float2int_rn(Cv.pos.x * 256.f), Y2 = __float2int_rn(Cv.pos.y * 256.f);
    const int X0 = __float2int_rn(A.pos.x * 256.f), Y0 = __float2int_rn(A.pos.y * 256.f);
    // Exact twice-area in 1/65536 px^2: counterclockwise culled (or turned,
    // when two-sided), degenerate dropped.
    long long area2 = (long long)(X1 - X0) * (Y2 - Y0) - (long long)(X2 - X0) * (Y1 - Y0);
    if (area2 < 0 && twoSided)
    {
        int t = X1;
        X1 = X2;
        X2 = t;
        t = Y1;
        Y1 = Y2;
        Y2 = t;
        pB = &Cv;
        pC = &Bv;
        const float2 z = zwB;
        zwB = zwC;
        zwC = z;
        area2 = -area2;
        features |= FEATURE_ATLAS_NEGATE;
    }
    if (area2 <= 0)
        return false;
    const VertexOut& B = *pB;
    const VertexOut& C = *pC;
    const int mnx = min(min(X0, X1), X2), mxx = max(max(X0, X1), X2);
    const int mny = min(min(Y0, Y1), Y2), mxy = max(max(Y0, Y1), Y2);
    // Pixels k whose centres (256 k + 128) lie in [min, max].
    const int bx0 = max(max(-((-(mnx - 128)) >> 8), 0), clip.x);
    const int bx1 = min(min(((mxx - 128) >> 8) + 1, (int)P.width), clip.z);
    const int by0 = max(max(-((-(mny - 128)) >> 8), 0), clip.y);
    const int by1 = min(min(((mxy - 128) >> 8) + 1, (int)P.height), clip.w);
    if (bx0 >= bx1 || by0 >= by1)
        return false;
    const float s = 1.f / 256.f;
    const float2 p0 = make_float2(X0 * s, Y0 * s), p1 = make_float2(X1 * s, Y1 * s);
    const float2 p2 = make_float2(X2 * s, Y2 * s);
    T.e0 = make_edge(p0, p1);
    T.e1 = make_edge(p1, p2);
    T.e2 = make_edge(p2, p0);
    const float d1x = p1.x - p0.x, d1y = p1.y - p0.y;
    const float d2x = p2.x - p0.x, d2y = p2.y - p0.y;
    const float inv = 1.f / ((float)area2 * (s * s));
    const float ax = T.e0.x - p0.x, ay = T.e0.y - p0.y;
    const float cxgx = ((B.cov.x - A.cov.x) * d2y - (C.cov.x - A.cov.x) * d1y) * inv;
    const float cxgy = ((C.cov.x - A.cov.x) * d1x - (B.cov.x - A.cov.x) * d2x) * inv;
    const float cygx = ((B.cov.y - A.cov.y) * d2y - (C.cov.y - A.cov.y) * d1y) * inv;
    const float cygy = ((C.cov.y - A.cov.y) * d1x - (B.cov.y - A.cov.y) * d2x) * inv;
    const uint2 paint = P.paints[P.firstPaint + A.pathID];
    T.cov0 = make_float4(A.cov.x + cxgx * ax + cxgy * ay, cxgx, cxgy, A.cov.y + cygx * ax + cygy * ay);
    T.cov1 = make_float4(cygx, cygy, __uint_as_float(paint.x), __uint_as_float(paint.y));
    if (featherPlanes)
    {
        // The third and fourth coverage components of a feathered fill, as
        // planes anchored at the first (snapped) vertex.
        const float zgx = ((zwB.x - zwA.x) * d2y - (zwC.x - zwA.x) * d1y) * inv;
        const float zgy = ((zwC.x - zwA.x) * d1x - (zwB.x - zwA.x) * d2x) * inv;
        const float wgx = ((zwB.y - zwA.y) * d2y - (zwC.y - zwA.y) * d1y) * inv;
        const float wgy = ((zwC.y - zwA.y) * d1x - (zwB.y - zwA.y) * d2x) * inv;
        featherPlanes[0] = make_float4(zwA.x, zgx, zgy, zwA.y);
        featherPlanes[1] = make_float4(wgx, wgy, p0.x, p0.y);
    }
    // The fp16 coverage key of the path (draw_raster_order_path.frag: pathID
    // bits, sign bit flipped for even-odd fills).
    uint32_t key = A.pathID == 0 ? 0u : ((A.pathID + MAX_DENORM_F16) * P.pathIDGranularity) & 0xffffu;
    if (paint.x & PAINT_FLAG_EVEN_ODD_FILL)
        key ^= 0x8000u;
    bb = make_int4(bx0, by0, bx1, by1);
    T.meta = make_uint4((A.pathID & 0xffffu) | (features << 16), (uint32_t)bx0 | ((uint32_t)bx1 << 16),
                        (uint32_t)by0 | ((uint32_t)by1 << 16), key | (scene << 16));
    return true;
}

// Tiles a set-up triangle touches (the same tile test as the binner's).
__device__ __forceinline__ void tile_span(int4 bb, int tileLog2, int& tx0, int& ty0, int& ntx,
                                          int& nty)
{
    tx0 = bb.x >> tileLog2;
    ty0 = bb.y >> tileLog2;
    ntx = ((bb.z - 1) >> tileLog2) - tx0 + 1;
    nty = ((bb.w - 1) >> tileLog2) - ty0 + 1;
}

constexpr int kLaneTiles = 8;

// Counts the tiles of the warp's triangles: a lane counts its own triangle
// when its box spans at most kLaneTiles tiles; the whole warp walks larger
// ones in turn. `has` marks lanes holding a triangle; e/bb its edges and box.
__device__ __forceinline__ void count_tiles(bool has,
                                            int tileLog2,
                                            const float4* e,
                                            int4 bb,
                                            uint32_t* __restrict__ countOut,
                                            uint8_t* __restrict__ maskOut,
                                            const float4 (*warpEdges)[3],
                                            const int4* warpBoxes,
                                            uint32_t* const* warpOuts)
{
    const int lane = threadIdx.x & 31;
    bool big = false;
    if (has)
    {
        if (bb.z > bb.x)
        {
            int tx0, ty0, ntx, nty;
            tile_span(bb, tileLog2, tx0, ty0, ntx, nty);
            if (ntx * nty <= kLaneTiles)
            {
                // The tiles it overlaps, as bits in row-major order over its
                // tile box, so the binner need not test them again.
                uint32_t count = 0, mask = 0;
                int i = 0;
                for (int ty = ty0; ty < ty0 + nty; ++ty)
                    for (int tx = tx0; tx < tx0 + ntx; ++tx, ++i)
                        if (tile_overlaps(e, bb, tx, ty, tileLog2))
                        {
                            ++count;
                            mask |= 1u << i;
                        }
                *countOut = count;
                *maskOut = (uint8_t)mask;
            }
            else
            {
                big = true;
            }
        }
        else
        {
            *countOut = 0;
        }
    }
    uint32_t bigs = __ballot_sync(0xffffffffu, big);
    while (bigs)
    {
        const int t = __ffs(bigs) - 1;
        bigs &= bigs - 1;
        const int4 tb = warpBoxes[t];
        const float4 te[3] = {warpEdges[t][0], warpEdges[t][1], warpEdges[t][2]};
        int tx0, ty0, ntx, nty;
        tile_span(tb, tileLog2, tx0, ty0, ntx, nty);
        const int n = ntx * nty;
        uint32_t count = 0;
        for (int i = lane; i < n; i += 32)
            count += tile_overlaps(te, tb, tx0 + i % ntx, ty0 + i / ntx, tileLog2) ? 1u : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            count += __shfl_xor_sync(0xffffffffu, count, o);
        if (lane == 0)
            *warpOuts[t] = count;
    }
}

// ---- Interior tiles as winding records -----------------------------------
//
// Inside a fill, the midpoint fan's triangles overlap a tile many times, yet
// every one of them has coverage +1 or -1, so at a pixel the path's count is
// their signed sum: the winding number of the fan's boundary (the contour
// polygon inset by the AA ramp) around the pixel. On a tile that no contour
// edge, AA ramp or contour midpoint comes near, that sum is one integer for
// every pixel, and the raster can add it once instead of walking the fan.
//
//  * patch_setup marks the path's edge tiles (within kWindingEdgeMargin of a
//    contour edge or midpoint) and defers the counting of its fan triangles;
//  * fan_filter_kernel adds each deferred fan triangle's coverage, row by
//    row, into the path's grid of winding deltas and counts its tiles,
//    keeping edge tiles only;
//  * path_winding_kernel turns each grid row's deltas into windings and
//    counts the interior tiles whose winding is not zero;
//  * bin_scatter writes one winding entry per counted interior tile, at the
//    path's place in primitive order (its first patch's winding slot);
//  * the raster stages a winding entry as a tile-wide "triangle" of constant
//    coverage W.
// Integers are exact in the fp16 coverage plane, and integer sums do not
// depend on their order, so the image is the one the fan gives.

// clamp(floor(n / d), qmin, qmax) for d > 0 (|n| < 2^50, d < 2^38,
// |qmin|, |qmax| < 2^13), without a 64-bit division: exact products decide
// the clamped cases; inside the range a float estimate is off by at most one
// and is corrected with exact products.
__device__ __forceinline__ long long floor_div_clamped(long long n, long long d, long long qmin,
                                                       long long qmax)
{
    if (n < qmin * d)
        return qmin;
    if (n >= (qmax + 1) * d)
        return qmax;
    long long q = (long long)floorf(__fdiv_rn((float)n, (float)d));
    q = min(max(q, qmin), qmax);
    while (q > qmin && q * d > n)
        --q;
    while (q < qmax && (q + 1) * d <= n)
        ++q;
    return q;
}

// The grid of a path whose interior tiles are winding records, or null.
__device__ __forceinline__ PathGrid* winding_grid(const BatchTables& B, uint32_t scene,
                                                  uint32_t pathID)
{
    if (!B.grids)
        return nullptr;
    PathGrid* g = B.grids + B.pathBase[scene] + pathID;
    const uint32_t f = g->flags;
    return (f & (PATH_GRID_ELIGIBLE | PATH_GRID_PLACED | PATH_GRID_UNSAFE)) ==
                   (PATH_GRID_ELIGIBLE | PATH_GRID_PLACED)
               ? g
               : nullptr;
}

// Whether a deferred fan triangle keeps tile (tx, ty): every tile when its
// path has no usable grid, else the edge tiles (and, defensively, tiles
// outside the grid box, which the box's margin keeps from happening).
__device__ __forceinline__ bool keep_fan_tile(const PathGrid* g, const uint8_t* __restrict__ edge,
                                              int tx, int ty)
{
    if (!g || tx < g->tx0 || tx >= g->tx1 || ty < g->ty0 || ty >= g->ty1)
        return true;
    return edge[g->offset + (size_t)(ty - g->ty0) * (g->tx1 - g->tx0) + (tx - g->tx0)] != 0;
}

// Adds a kept fan triangle's coverage (+-1) into its path's winding deltas.
// A tile's winding is evaluated at its reference pixel, its first pixel
// centre (ox + 1/2, oy + 1/2): for each tile row whose reference line the
// triangle crosses, the columns whose reference pixel lies inside it are
// found exactly, in 64-bit integers of 1/256 px, from the snapped edges with
// the raster's tie rule, and the row's deltas get +c at the first and -c
// past the last.
__device__ void fan_winding_deltas(const TriRecord& T, int4 bb, int c, const PathGrid& G,
                                   int32_t* __restrict__ W, int tileLog2)
{
    const int ts = 1 << tileLog2;
    int r0 = (bb.y + ts - 1) >> tileLog2, r1 = (bb.w - 1) >> tileLog2;
    r0 = max(r0, G.ty0);
    r1 = min(r1, G.ty1 - 1);
    if (r0 > r1)
        return;
    const float4 e[3] = {T.e0, T.e1, T.e2};
    long long A[3], Bc[3], AX[3], AY[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        // Snapped coordinates and their differences are exact multiples of
        // 1/256 below 2^16 px: exact integers after scaling.
        AX[k] = (long long)__fmul_rn(e[k].x, 256.f);
        AY[k] = (long long)__fmul_rn(e[k].y, 256.f);
        A[k] = (long long)__fmul_rn(e[k].z, 256.f);
        Bc[k] = (long long)__fmul_rn(e[k].w, 256.f);
    }
    const int gw = G.tx1 - G.tx0;
    for (int r = r0; r <= r1; ++r)
    {
        const long long PY = (long long)(r << tileLog2) * 256 + 128;
        long long lo = G.tx0, hi = G.tx1 - 1;
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            // E(col) = alpha * col + beta, in (1/256 px)^2.
            const long long alpha = A[k] * (long long)(ts * 256);
            const long long beta = A[k] * (128 - AX[k]) + Bc[k] * (PY - AY[k]);
            if (A[k] > 0) // inside where E >= 0 (ties belong to this edge): col >= -beta/alpha
                lo = max(lo, -floor_div_clamped(beta, alpha, -hi - 1, -lo));
            else if (A[k] < 0) // inside where E > 0: col <= floor((beta - 1) / -alpha)
                hi = min(hi, floor_div_clamped(beta - 1, -alpha, lo - 1, hi));
            else if (!(beta > 0 || (beta == 0 && Bc[k] > 0)))
                hi = lo - 1;
            if (lo > hi)
                break;
        }
        if (lo > hi)
            continue;
        int32_t* row = W + G.offset + (size_t)(r - G.ty0) * gw;
        atomicAdd(row + (lo - G.tx0), c);
        if (hi + 1 < G.tx1)
            atomicAdd(row + (hi + 1 - G.tx0), -c);
    }
}

// Marks the grid's tiles whose pixel centres, widened by kWindingEdgeMargin
// px, meet the segment a-b (a point when a == b). Finite inputs.
__device__ void mark_edge_tiles(float2 a, float2 b, const PathGrid& G, uint8_t* __restrict__ edge,
                                int tileLog2)
{
    const float ts = (float)(1 << tileLog2);
    const float m = kWindingEdgeMargin - .5f; // tile t's widened span: [t ts - m, (t+1) ts + m]
    const float y0 = fminf(a.y, b.y), y1 = fmaxf(a.y, b.y);
    const int gw = G.tx1 - G.tx0;
    int t0 = (int)ceilf((y0 - m) / ts - 1.f), t1 = (int)floorf((y1 + m) / ts);
    t0 = max(t0, G.ty0);
    t1 = min(t1, G.ty1 - 1);
    const float dy = b.y - a.y, dx = b.x - a.x;
    for (int ty = t0; ty <= t1; ++ty)
    {
        // The part of the segment inside the row's widened band.
        const float ylo = fmaxf((float)ty * ts - m, y0), yhi = fminf((float)(ty + 1) * ts + m, y1);
        float xa, xb;
        if (fabsf(dy) < 1e-6f)
        {
            xa = fminf(a.x, b.x);
            xb = fmaxf(a.x, b.x);
        }
        else
        {
            const float u0 = fminf(fmaxf((ylo - a.y) / dy, 0.f), 1.f);
            const float u1 = fminf(fmaxf((yhi - a.y) / dy, 0.f), 1.f);
            const float xu0 = a.x + dx * u0, xu1 = a.x + dx * u1;
            // A little slack for the rounding of the clip.
            xa = fminf(xu0, xu1) - 1e-2f;
            xb = fmaxf(xu0, xu1) + 1e-2f;
        }
        int c0 = (int)ceilf((xa - m) / ts - 1.f), c1 = (int)floorf((xb + m) / ts);
        c0 = max(c0, G.tx0);
        c1 = min(c1, G.tx1 - 1);
        uint8_t* row = edge + G.offset + (size_t)(ty - G.ty0) * gw;
        for (int tx = c0; tx <= c1; ++tx)
            row[tx - G.tx0] = 1;
    }
}

// Patch set-up, one warp per patch instance of the batch: shade the patch's
// vertices, assemble and set up its triangles, then count the tiles each one
// touches. kList selects the patch: 0 the midpoint fan, 1 the outer-curve
// patch (interior triangulation), 3 the center-AA midpoint fan (feathered
// fills). Triangle slot order is primitive order (flush, draw batch,
// instance, triangle-in-patch).
template <int kList, bool kFeather, bool kWinding = false>
__device__ __forceinline__ void patch_setup(const BatchTables& B,
                                            TriRecord* __restrict__ tris,
                                            uint32_t* __restrict__ tileCounts,
                                            uint8_t* __restrict__ tileMasks)
{
    constexpr bool kOuter = kList == 1, kCenter = kList == 3;
    constexpr int kVerts =
        kOuter ? kOuterPatchVertexCount : (kCenter ? kCenterPatchVertexCount : kPatchVertexCount);
    constexpr int kTris = kOuter ? kOuterPatchTriangleCount
                                 : (kCenter ? kCenterPatchTriangleCount : kPatchTriangleCount);
    constexpr int kSpan = kOuter ? kOuterPatchSegmentSpan : kPatchSegmentSpan;
    constexpr int kTriPasses = (kTris + 31) / 32;
    __shared__ VertexOut sv[4][kVerts];
    // The feathered-fill coverage components, kept only for feathered draws.
    __shared__ float2 sZW[4][kFeather ? kVerts : 1];
    __shared__ float4 sEdges[4][kTriPasses * 32][3];
    __shared__ int4 sBox[4][kTriPasses * 32];
    __shared__ uint32_t* sOut[4][kTriPasses * 32];
    __shared__ bool sok[4];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t gi = blockIdx.x * 4 + w;
    if (gi >= B.totalItems[kList])
        return; // whole warp exits together
    const uint32_t seg = find_range(B.segBase[kList], B.segCount[kList], gi);
    const PatchSegment S = B.segments[kList][seg];
    const FlushParams& P = B.scenes[S.scene];
    const uint32_t local = gi - B.segBase[kList][seg];
    const uint32_t instance = S.baseElement + local;
    // Feathered draws keep their fills' extra coverage planes per slot.
    float4* const planes = (kFeather && (S.features & SF_FEATHER)) ? B.featherPlanes : nullptr;
    if (lane == 0)
        sok[w] = true;
    __syncwarp();
    for (int v = lane; v < kVerts; v += 32)
    {
        VertexOut o;
        const PatchVertexDesc pv = kOuter    ? outer_vertex_desc(v)
                                   : kCenter ? center_vertex_desc(v)
                                             : patch_vertex_desc(v);
        float2 zw;
        if (!shade_patch_vertex<kFeather>(P, pv, kSpan, instance, o, zw))
        {
            sok[w] = false;
            o.discard = true;
        }
        sv[w][v] = o;
        if (kFeather && planes)
            sZW[w][v] = zw;
    }
    __syncwarp();
    // The path's image slot, for the raster's image paint (every patch of
    // the path writes the same value).
    if (S.image != kNoImage && lane == 0 && sok[w] && P.pathImage)
    {
        const uint32_t pid = sv[w][kVerts - 1].pathID;
        if (pid < P.pathCount)
            P.pathImage[pid] = S.image;
    }
    // With interior tiles as winding records, each midpoint-fan patch also
    // owns a winding slot after its triangles.
    const uint32_t stride = (kList == 0 && B.fanSlotStride) ? B.fanSlotStride : (uint32_t)kTris;
    const uint32_t slot0 = S.slotBase + local * stride;
    PathGrid* wg = nullptr; // the path's winding grid, when this patch feeds it
    if (kWinding && kList == 0 && !kFeather && B.grids)
    {
        if (lane == 0)
        {
            tileCounts[slot0 + kTris] = 0; // path_winding_kernel fills the path's anchor
            tileMasks[slot0 + kTris] = 0;
        }
        if (sok[w])
        {
            const uint32_t pid = sv[w][kVerts - 1].pathID;
            PathGrid* g = pid < P.pathCount ? winding_grid(B, S.scene, pid) : nullptr;
            if (g)
            {
                // A discarded or non-finite vertex would leave a hole in the
                // fan: such a path keeps its fan triangles everywhere.
                bool bad = false;
                for (int v = lane; v < kVerts; v += 32)
                {
                    const VertexOut& o = sv[w][v];
                    bad = bad || o.discard ||
                          !(fabsf(o.pos.x) < 32768.f && fabsf(o.pos.y) < 32768.f);
                }
                if (__any_sync(0xffffffffu, bad))
                {
                    if (lane == 0)
                        atomicOr(&g->flags, PATH_GRID_UNSAFE);
                }
                else
                {
                    wg = g;
                }
            }
        }
        if (wg)
        {
            const PathGrid G = *wg;
            // Edge tiles: near the inset contour's edges (fan vertices 32..40,
            // shared by the AA ramps) or its midpoint (vertex 41).
            if (lane < kPatchSegmentSpan)
                mark_edge_tiles(sv[w][32 + lane].pos, sv[w][33 + lane].pos, G, B.gridEdge,
                                B.tileLog2);
            else if (lane == kPatchSegmentSpan)
                mark_edge_tiles(sv[w][41].pos, sv[w][41].pos, G, B.gridEdge, B.tileLog2);
            if (lane == 0)
            {
                // The winding slot's record: the path's paint, coverage key
                // and grid, for the raster to stage a winding entry from.
                const uint32_t pid = sv[w][kVerts - 1].pathID;
                atomicMin(&wg->anchor, slot0 + kTris);
                const uint2 paint = P.paints[P.firstPaint + pid];
                uint32_t key = pid == 0 ? 0u
                                        : ((pid + MAX_DENORM_F16) * P.pathIDGranularity) & 0xffffu;
                if (paint.x & PAINT_FLAG_EVEN_ODD_FILL)
                    key ^= 0x8000u;
                TriRecord R;
                R.e0 = make_float4(__uint_as_float(G.offset), __int_as_float(G.tx0),
                                   __int_as_float(G.ty0), __int_as_float(G.tx1 - G.tx0));
                R.e1 = make_float4(__int_as_float(G.ty1 - G.ty0), 0.f, 0.f, 0.f);
                R.e2 = make_float4(0.f, 0.f, 0.f, 0.f);
                R.cov0 = make_float4(0.f, 0.f, 0.f, 0.f);
                R.cov1 = make_float4(0.f, 0.f, __uint_as_float(paint.x), __uint_as_float(paint.y));
                R.meta = make_uint4((pid & 0xffffu) | ((S.features | FEATURE_WINDING_SLOT) << 16), 0u,
                                    0u, key | (S.scene << 16));
                tris[slot0 + kTris] = R;
            }
        }
    }
    for (int pass = 0; pass < kTriPasses; ++pass)
    {
        const int t = pass * 32 + lane;
        const bool has = t < kTris;
        bool deferred = false;
        int4 bb = make_int4(0, 0, 0, 0);
        float4 e[3];
        if (has)
        {
            int ia, ib, ic;
            if (kOuter)
                outer_triangle(t, ia, ib, ic);
            else if (kCenter)
                center_triangle(t, ia, ib, ic);
            else
                patch_triangle(t, ia, ib, ic);
            // Fan triangles (16..23) of a path with a winding grid: their
            // tiles are counted once the grid knows its edge tiles.
            const bool fan = kWinding && kList == 0 && wg && t >= 16;
            TriRecord T;
            const int4 clip = make_int4((int)(S.scissorLT & 0xffffu), (int)(S.scissorLT >> 16),
                                        (int)(S.scissorRB & 0xffffu), (int)(S.scissorRB >> 16));
            if (sok[w] && setup_triangle(P, sv[w][ia], sv[w][ib], sv[w][ic],
                                         S.features | (fan ? FEATURE_FAN_DEFERRED : 0u), S.scene,
                                         T, bb, planes ? planes + 2 * (size_t)(slot0 + t) : nullptr,
                                         planes ? sZW[w][kFeather ? ia : 0] : float2{},
                                         planes ? sZW[w][kFeather ? ib : 0] : float2{},
                                         planes ? sZW[w][kFeather ? ic : 0] : float2{}, clip,
                                         kCenter && P.atlasMode))
            {
                tris[slot0 + t] = T;
                e[0] = T.e0;
                e[1] = T.e1;
                e[2] = T.e2;
                sEdges[w][t][0] = T.e0;
                sEdges[w][t][1] = T.e1;
                sEdges[w][t][2] = T.e2;
                deferred = fan;
            }
            sBox[w][t] = bb;
            sOut[w][t] = tileCounts + slot0 + t;
        }
        __syncwarp();
        count_tiles(has && !deferred, B.tileLog2, e, bb, tileCounts + slot0 + t,
                    tileMasks + slot0 + t, sEdges[w] + pass * 32, sBox[w] + pass * 32,
                    sOut[w] + pass * 32);
        if (deferred)
            tileCounts[slot0 + t] = kDeferredCount;
        __syncwarp();
    }
}

// Resident 128-thread CTAs per SM the midpoint-fan set-up's registers are
// bounded for.
#ifndef RIVE_SETUP_MIN_BLOCKS
#define RIVE_SETUP_MIN_BLOCKS 9
#endif
__global__ void __launch_bounds__(128, RIVE_SETUP_MIN_BLOCKS) patch_setup_kernel(BatchTables B,
                                                          TriRecord* __restrict__ tris,
                                                          uint32_t* __restrict__ tileCounts,
                                                          uint8_t* __restrict__ tileMasks)
{
    patch_setup<0, false>(B, tris, tileCounts, tileMasks);
}

// Midpoint-fan set-up for batches that draw interior tiles as winding records
// (its own kernel, so the plain one keeps its register budget).
__global__ void __launch_bounds__(128) patch_setup_winding_kernel(BatchTables B,
                                                                  TriRecord* __restrict__ tris,
                                                                  uint32_t* __restrict__ tileCounts,
                                                                  uint8_t* __restrict__ tileMasks)
{
    patch_setup<0, false, true>(B, tris, tileCounts, tileMasks);
}

// Midpoint-fan set-up with the feather paths, for batches that feather.
__global__ void __launch_bounds__(128) patch_setup_feather_kernel(BatchTables B,
                                                                  TriRecord* __restrict__ tris,
                                                                  uint32_t* __restrict__ tileCounts,
                                                                  uint8_t* __restrict__ tileMasks)
{
    patch_setup<0, true>(B, tris, tileCounts, tileMasks);
}

__global__ void __launch_bounds__(128) outer_setup_kernel(BatchTables B,
                                                          TriRecord* __restrict__ tris,
                                                          uint32_t* __restrict__ tileCounts,
                                                          uint8_t* __restrict__ tileMasks)
{
    patch_setup<1, false>(B, tris, tileCounts, tileMasks);
}

__global__ void __launch_bounds__(128) center_setup_kernel(BatchTables B,
                                                           TriRecord* __restrict__ tris,
                                                           uint32_t* __restrict__ tileCounts,
                                                           uint8_t* __restrict__ tileMasks)
{
    patch_setup<3, true>(B, tris, tileCounts, tileMasks);
}

// The mip level of an image-mesh triangle. draw_mesh.frag samples with the
// implicit level of detail plus FlushUniforms::mipMapLODBias
// (TEXTURE_SAMPLE_DYNAMIC_LODBIAS); under the Vulkan rules the reference
// backend follows, lambda = log2(rho) + bias with rho the larger of the
// texel-space lengths of d(uv)/dx and d(uv)/dy, clamped to [0, levels - 1],
// and the nearest mip level ceil(lambda + 1/2) - 1
// (VK_SAMPLER_MIPMAP_MODE_NEAREST). Texture coordinates are affine over a
// triangle, so rho is the triangle's constant. Level k is reached when
// lambda > k - 1/2, i.e. rho^2 > 2^(2k - 1 - 2 bias): a comparison with a
// power of two, exact for the reference's bias of -1/2 (other biases are
// taken to the nearest half-integer).
__device__ __forceinline__ uint32_t mesh_mip_level(float rho2, float bias, uint32_t levels)
{
    const int twoBias = (int)rintf(__fmul_rn(2.f, bias));
    uint32_t level = 0;
    for (uint32_t k = 1; k < levels; ++k)
    {
        if (!(rho2 > ldexpf(1.f, 2 * (int)k - 1 - twoBias)))
            break;
        level = k;
    }
    return level;
}

// One triangle of an image mesh (draw_image_mesh.vert): the vertices of its
// three indices, each the view matrix times the local position plus the
// translate (ImageDrawInstance), with its texture coordinates; no face is
// culled (get_cull_face, gpu.cpp:1552-1593). The texture coordinates become
// exact planes in the slot's feather-plane pair; the record carries the
// ImageDrawInstance index and the image slot with the triangle's mip level
// where paths keep their paint words, and the coverage key of path 0.
__device__ bool mesh_triangle(const BatchTables& B, const FlushParams& P, const PatchSegment& S,
                              uint32_t local, uint32_t slot, TriRecord& T, int4& bb)
{
    bb = make_int4(0, 0, 0, 0);
    const MeshDesc& M = B.meshes[S.mesh];
    const float4* inst = P.imageDraws + 4 * (size_t)M.imageDraw;
    const float4 vm = inst[0], tr = inst[2];
    VertexOut v[3];
    float2 uv[3];
    for (int k = 0; k < 3; ++k)
    {
        const uint32_t vi = M.indices[3 * local + k];
        if (vi >= M.vertexCount)
        {
            atomicOr(P.error, ERR_BAD_MESH_INDEX);
            return false;
        }
        const float2 p = M.positions[vi];
        uv[k] = M.uvs[vi];
        v[k].pos = make_float2(__fadd_rn(__fadd_rn(__fmul_rn(vm.x, p.x), __fmul_rn(vm.z, p.y)), tr.x),
                               __fadd_rn(__fadd_rn(__fmul_rn(vm.y, p.x), __fmul_rn(vm.w, p.y)), tr.y));
        v[k].cov = uv[k];
        v[k].pathID = 0;
        v[k].discard = false;
    }
    float4* planes = B.featherPlanes + 2 * (size_t)slot;
    if (!setup_triangle(P, v[0], v[1], v[2], S.features, S.scene, T, bb, planes, uv[0], uv[1], uv[2],
                        make_int4(0, 0, 0x7fffffff, 0x7fffffff), true))
        return false;
    const float4 f0 = planes[0], f1 = planes[1];
    const ImageTex& tex = P.images[M.image];
    const float W = (float)tex.width, H = (float)tex.height;
    const float ux = __fmul_rn(f0.y, W), vx = __fmul_rn(f1.x, H);
    const float uy = __fmul_rn(f0.z, W), vy = __fmul_rn(f1.y, H);
    const float rho2 = fmaxf(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(vx, vx)),
                             __fadd_rn(__fmul_rn(uy, uy), __fmul_rn(vy, vy)));
    const uint32_t level = mesh_mip_level(rho2, P.mipLodBias, tex.levels);
    T.cov1.z = __uint_as_float(M.imageDraw);
    T.cov1.w = __uint_as_float(M.image | (level << 24));
    T.meta.w = S.scene << 16;
    return true;
}

// Interior triangulation (DrawType::interiorTriangulation): one thread per
// triangle of the batch's TriangleVertex records. A vertex is the path-space
// point mapped by the path's matrix, and its coverage is the triangle's
// winding weight (unpack_interior_triangle_vertex,
// draw_path_common.glsl:792-819); the raster adds it like a fill's constant
// coverage.
__global__ void __launch_bounds__(256) interior_setup_kernel(BatchTables B,
                                                             TriRecord* __restrict__ tris,
                                                             uint32_t* __restrict__ tileCounts,
                                                             uint8_t* __restrict__ tileMasks)
{
    __shared__ float4 sEdges[8][32][3];
    __shared__ int4 sBox[8][32];
    __shared__ uint32_t* sOut[8][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t first = (blockIdx.x * blockDim.x) & ~31u;
    if (first >= B.totalItems[2])
        return; // whole warp exits together
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    const bool has = gi < B.totalItems[2];
    int4 bb = make_int4(0, 0, 0, 0);
    float4 e[3];
    uint32_t slot = 0;
    if (has)
    {
        const uint32_t seg = find_range(B.segBase[2], B.segCount[2], gi);
        const PatchSegment S = B.segments[2][seg];
        const FlushParams& P = B.scenes[S.scene];
        const uint32_t local = gi - B.segBase[2][seg];
        slot = S.slotBase + local;
        VertexOut v[3];
        bool ok = true;
        if (S.features & FEATURE_IMAGE_MESH)
        {
            TriRecord T;
            if (mesh_triangle(B, P, S, local, slot, T, bb))
            {
                tris[slot] = T;
                e[0] = T.e0;
                e[1] = T.e1;
                e[2] = T.e2;
                sEdges[w][lane][0] = T.e0;
                sEdges[w][lane][1] = T.e1;
                sEdges[w][lane][2] = T.e2;
            }
            ok = false; // set up already
        }
        for (int k = 0; k < 3 && ok; ++k)
        {
            const uint32_t vi = S.baseElement + 3 * local + k;
            if (vi >= P.triangleVertexCount)
            {
                atomicOr(P.error, ERR_BAD_TESS_INDEX);
                ok = false;
                break;
            }
            const uint32_t* r = P.triangleVertices + 3 * (size_t)vi;
            const uint32_t pathID = r[2] & 0xffffu;
            if (pathID >= P.pathCount)
            {
                atomicOr(P.error, ERR_BAD_PATH);
                ok = false;
                break;
            }
            const uint4* path = P.paths + 4 * (size_t)(P.firstPath + pathID);
            if (S.features & FEATURE_ATLAS_BLIT)
            {
                // unpack_atlas_coverage_vertex (draw_path_common.glsl:822-844):
                // a screen-space rectangle corner, carrying its atlas position
                // (screen * scale + translate by the path's atlas transform)
                // for the raster to sample.
                const uint4 r2 = path[2];
                const float sc = __uint_as_float(r2.y);
                const float x = __uint_as_float(r[0]), y = __uint_as_float(r[1]);
                v[k].pos = make_float2(x, y);
                v[k].cov = make_float2(__fadd_rn(__fmul_rn(x, sc), __uint_as_float(r2.z)),
                                       __fadd_rn(__fmul_rn(y, sc), __uint_as_float(r2.w)));
                v[k].pathID = pathID;
                v[k].discard = false;
                continue;
            }
            const uint4 r0 = path[0], r1 = path[1];
            const float4 M = make_float4(__uint_as_float(r0.x), __uint_as_float(r0.y),
                                         __uint_as_float(r0.z), __uint_as_float(r0.w));
            const float2 p = mat_mul(M, make_float2(__uint_as_float(r[0]), __uint_as_float(r[1])));
            v[k].pos = make_float2(__fadd_rn(p.x, __uint_as_float(r1.x)),
                                   __fadd_rn(p.y, __uint_as_float(r1.y)));
            v[k].cov = make_float2((float)((int32_t)r[2] >> 16), -1.f);
            v[k].pathID = pathID;
            v[k].discard = false;
        }
        if (ok && S.image != kNoImage && P.pathImage)
            P.pathImage[v[0].pathID] = S.image;
        TriRecord T;
        if (ok && setup_triangle(P, v[0], v[1], v[2], S.features, S.scene, T, bb))
        {
            tris[slot] = T;
            e[0] = T.e0;
            e[1] = T.e1;
            e[2] = T.e2;
            sEdges[w][lane][0] = T.e0;
            sEdges[w][lane][1] = T.e1;
            sEdges[w][lane][2] = T.e2;
        }
        sBox[w][lane] = bb;
        sOut[w][lane] = tileCounts + slot;
    }
    __syncwarp();
    count_tiles(has, B.tileLog2, e, bb, tileCounts + slot, tileMasks + slot, sEdges[w], sBox[w], sOut[w]);
}

// ---- Winding grids: the per-path passes ------------------------------------

// One thread per path of the batch: an empty grid box, and whether the path's
// interior tiles may become winding records. Eligible: a fill (no stroke
// radius) without a feather, not the clear colour's path 0, not drawn as
// wireframe, and not a nested clip update (its stash of the outer clip keeps
// an RGBA8 rounding when a pixel saw more than one fragment of it, which a
// single winding entry cannot reproduce).
__global__ void __launch_bounds__(256) path_init_kernel(BatchTables B)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.pathBase[B.sceneCount])
        return;
    const uint32_t scene = find_range(B.pathBase, B.sceneCount, i);
    const FlushParams& P = B.scenes[scene];
    const uint32_t pid = i - B.pathBase[scene];
    PathGrid g;
    g.tx0 = g.ty0 = 0x7fffffff;
    g.tx1 = g.ty1 = -0x7fffffff;
    g.offset = 0;
    g.anchor = 0xffffffffu;
    g.entries = 0;
    g.flags = 0;
    g.length = 0.f;
    if (pid != 0 && !P.wireframe)
    {
        const uint4 r1 = P.paths[4 * (size_t)(P.firstPath + pid) + 1];
        const uint2 paint = P.paints[P.firstPaint + pid];
        const bool nestedClip = (paint.x & 0xfu) == CLIP_UPDATE_PAINT_TYPE && (paint.x >> 16) != 0;
        if (__uint_as_float(r1.z) == 0.f && __uint_as_float(r1.w) == 0.f && !nestedClip)
            g.flags = PATH_GRID_ELIGIBLE;
    }
    B.grids[i] = g;
}

// One thread per tessellation span of the batch: grows its path's grid box by
// the span's control points and its contour's midpoint, mapped to pixels by
// the path's matrix (curves stay inside their control points' hull), widened
// by the AA offset (1/2 px) and the edge margin, in tiles clipped to the
// canvas.
__global__ void __launch_bounds__(256) path_bounds_kernel(BatchTables B)
{
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= B.totalTessSpans)
        return;
    const uint32_t scene = find_range(B.tessSpanBase, B.sceneCount, gi);
    const FlushParams& P = B.scenes[scene];
    const uint4* sp = P.tessSpans + 4 * (size_t)(P.firstTessSpan + gi - B.tessSpanBase[scene]);
    const uint32_t contourID = sp[3].w & CONTOUR_ID_MASK;
    if (contourID == 0 || contourID > P.contourCount)
        return;
    const uint4 cd = P.contours[P.firstContour + contourID - 1];
    const uint32_t pid = cd.z & 0xffffu;
    if (pid >= P.pathCount)
        return;
    PathGrid* g = B.grids + B.pathBase[scene] + pid;
    if (!(g->flags & PATH_GRID_ELIGIBLE))
        return;
    const uint4* path = P.paths + 4 * (size_t)(P.firstPath + pid);
    const uint4 r0 = path[0], r1 = path[1];
    const float4 M = make_float4(__uint_as_float(r0.x), __uint_as_float(r0.y),
                                 __uint_as_float(r0.z), __uint_as_float(r0.w));
    const float2 tr = make_float2(__uint_as_float(r1.x), __uint_as_float(r1.y));
    const uint4 q0 = sp[0], q1 = sp[1];
    const float2 pts[5] = {make_float2(__uint_as_float(q0.x), __uint_as_float(q0.y)),
                           make_float2(__uint_as_float(q0.z), __uint_as_float(q0.w)),
                           make_float2(__uint_as_float(q1.x), __uint_as_float(q1.y)),
                           make_float2(__uint_as_float(q1.z), __uint_as_float(q1.w)),
                           make_float2(__uint_as_float(cd.x), __uint_as_float(cd.y))};
    float x0 = 3e38f, y0 = 3e38f, x1 = -3e38f, y1 = -3e38f, len = 0.f;
    float2 prev = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 5; ++k)
    {
        const float2 q = mat_mul(M, pts[k]);
        const float x = q.x + tr.x, y = q.y + tr.y;
        if (!(fabsf(x) < 1e9f && fabsf(y) < 1e9f))
            return; // non-finite: the set-up marks the path unsafe
        x0 = fminf(x0, x);
        x1 = fmaxf(x1, x);
        y0 = fminf(y0, y);
        y1 = fmaxf(y1, y);
        if (k > 0 && k < 4) // the control polygon p0-p1-p2-p3
            len += sqrtf((x - prev.x) * (x - prev.x) + (y - prev.y) * (y - prev.y));
        prev = make_float2(x, y);
    }
    atomicAdd(&g->length, len);
    const float pad = kAARadius + kWindingEdgeMargin + 1.f;
    const float ts = (float)(1 << B.tileLog2);
    const int tilesY = (int)((P.height + (1u << B.tileLog2) - 1) >> B.tileLog2);
    const int tx0 = max((int)floorf((x0 - pad) / ts), 0);
    const int ty0 = max((int)floorf((y0 - pad) / ts), 0);
    const int tx1 = min((int)floorf((x1 + pad) / ts), (int)P.tilesX - 1) + 1;
    const int ty1 = min((int)floorf((y1 + pad) / ts), tilesY - 1) + 1;
    if (tx0 >= tx1 || ty0 >= ty1)
        return;
    atomicMin(&g->tx0, tx0);
    atomicMin(&g->ty0, ty0);
    atomicMax(&g->tx1, tx1);
    atomicMax(&g->ty1, ty1);
}

// One thread per path: places an eligible path's grid in the pool (one cell
// per tile of its box), unless its contour is long enough to make most of
// those tiles edge tiles. gridCounters[0] ends as the cells the batch asked
// for; a grid past the pool's capacity is not placed, and that path keeps its
// fan triangles on every tile.
__global__ void __launch_bounds__(256) path_alloc_kernel(BatchTables B)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B.pathBase[B.sceneCount])
        return;
    PathGrid& g = B.grids[i];
    if (!(g.flags & PATH_GRID_ELIGIBLE) || g.tx0 >= g.tx1 || g.ty0 >= g.ty1)
        return;
    const uint32_t cells = (uint32_t)(g.tx1 - g.tx0) * (uint32_t)(g.ty1 - g.ty0);
    // Too little interior to pay for the grid: keep the plain fan.
    if (1.5f * g.length * (1.f / (float)(1 << B.tileLog2)) >= kWindingMaxEdgeShare * (float)cells)
        return;
    const uint32_t off = atomicAdd(&B.gridCounters[0], cells);
    if ((uint64_t)off + cells <= B.gridCapacity)
    {
        g.offset = off;
        g.flags |= PATH_GRID_PLACED;
    }
}

// One warp per path, after fan_filter_kernel: each grid row's deltas become the
// windings of its tiles (a warp scan, 32 columns at a time), and the path's
// interior tiles with a nonzero winding are counted into its anchor slot.
__global__ void __launch_bounds__(256) path_winding_kernel(BatchTables B,
                                                           uint32_t* __restrict__ tileCounts)
{
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= B.pathBase[B.sceneCount])
        return;
    PathGrid* g = B.grids + i;
    const uint32_t flags = g->flags;
    if ((flags & (PATH_GRID_ELIGIBLE | PATH_GRID_PLACED)) != (PATH_GRID_ELIGIBLE | PATH_GRID_PLACED))
        return;
    const int gw = g->tx1 - g->tx0, gh = g->ty1 - g->ty0;
    const uint32_t anchor = g->anchor;
    const bool counted = !(flags & PATH_GRID_UNSAFE) && anchor != 0xffffffffu;
    uint32_t n = 0;
    for (int r = 0; r < gh; ++r)
    {
        int32_t* row = B.gridWinding + g->offset + (size_t)r * gw;
        const uint8_t* edge = B.gridEdge + g->offset + (size_t)r * gw;
        int32_t carry = 0;
        for (int c0 = 0; c0 < gw; c0 += 32)
        {
            const int c = c0 + lane;
            int32_t v = c < gw ? row[c] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int32_t y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o)
                    v += y;
            }
            v += carry;
            if (c < gw)
            {
                row[c] = v;
                n += (counted && !edge[c] && v != 0) ? 1u : 0u;
            }
            carry = __shfl_sync(0xffffffffu, v, 31);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        n += __shfl_xor_sync(0xffffffffu, n, o);
    if (lane == 0)
    {
        g->entries = counted ? n : 0u;
        if (counted && n)
        {
            tileCounts[anchor] = n;
            atomicAdd(&B.gridCounters[1], n);
        }
    }
}

// One thread per fan triangle (16..23) of every midpoint-fan patch, after the
// set-up: a deferred one adds its coverage into its path's winding deltas and
// counts its tiles, now that the path's edge tiles are known (only edge
// tiles, when the path's grid is usable), with the per-slot tile mask for
// small boxes, as count_tiles does.
__global__ void __launch_bounds__(256) fan_filter_kernel(BatchTables B,
                                                         const TriRecord* __restrict__ tris,
                                                         uint32_t* __restrict__ tileCounts,
                                                         uint8_t* __restrict__ tileMasks)
{
    __shared__ float4 sEdges[8][32][3];
    __shared__ int4 sBox[8][32];
    __shared__ const PathGrid* sGrid[8][32];
    __shared__ uint32_t sSlot[8][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t total = B.totalItems[0] * 8u;
    const uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x;
    if ((gi & ~31u) >= total)
        return; // whole warp exits together
    const int tileLog2 = B.tileLog2;
    bool big = false;
    if (gi < total)
    {
        const uint32_t patch = gi >> 3;
        const uint32_t seg = find_range(B.segBase[0], B.segCount[0], patch);
        const PatchSegment S = B.segments[0][seg];
        const uint32_t slot =
            S.slotBase + (patch - B.segBase[0][seg]) * B.fanSlotStride + 16u + (gi & 7u);
        if (tileCounts[slot] == kDeferredCount)
        {
            const TriRecord& T = tris[slot];
            const uint4 meta = T.meta;
            const int4 bb = unpack_bbox(meta);
            const float4 e[3] = {T.e0, T.e1, T.e2};
            const PathGrid* g = winding_grid(B, meta.w >> 16, meta.x & 0xffffu);
            // A fan triangle's coverage is +-1 everywhere (its three vertices
            // carry the same fill coverage): its share of the path's windings.
            if (g)
                fan_winding_deltas(T, bb, T.cov0.x > 0.f ? 1 : -1, *g, B.gridWinding, tileLog2);
            int tx0, ty0, ntx, nty;
            tile_span(bb, tileLog2, tx0, ty0, ntx, nty);
            if (ntx * nty <= kLaneTiles)
            {
                uint32_t count = 0, mask = 0;
                int k = 0;
                for (int ty = ty0; ty < ty0 + nty; ++ty)
                    for (int tx = tx0; tx < tx0 + ntx; ++tx, ++k)
                        if (tile_overlaps(e, bb, tx, ty, tileLog2) &&
                            keep_fan_tile(g, B.gridEdge, tx, ty))
                        {
                            ++count;
                            mask |= 1u << k;
                        }
                tileCounts[slot] = count;
                tileMasks[slot] = (uint8_t)mask;
            }
            else
            {
                big = true;
                sEdges[w][lane][0] = e[0];
                sEdges[w][lane][1] = e[1];
                sEdges[w][lane][2] = e[2];
                sBox[w][lane] = bb;
                sGrid[w][lane] = g;
                sSlot[w][lane] = slot;
            }
        }
    }
    __syncwarp();
    uint32_t bigs = __ballot_sync(0xffffffffu, big);
    while (bigs)
    {
        const int t = __ffs(bigs) - 1;
        bigs &= bigs - 1;
        const int4 tb = sBox[w][t];
        const float4 te[3] = {sEdges[w][t][0], sEdges[w][t][1], sEdges[w][t][2]};
        const PathGrid* tg = sGrid[w][t];
        int tx0, ty0, ntx, nty;
        tile_span(tb, tileLog2, tx0, ty0, ntx, nty);
        const int n = ntx * nty;
        uint32_t count = 0;
        for (int i = lane; i < n; i += 32)
        {
            const int tx = tx0 + i % ntx, ty = ty0 + i / ntx;
            count += (tile_overlaps(te, tb, tx, ty, tileLog2) && keep_fan_tile(tg, B.gridEdge, tx, ty))
                         ? 1u
                         : 0u;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            count += __shfl_xor_sync(0xffffffffu, count, o);
        if (lane == 0)
            tileCounts[sSlot[w][t]] = count;
    }
}

// FlushUniforms fields the passes use (gpu.hpp:1466-1537: pathIDGranularity
// at byte 72, ditherScale at 88, ditherBias at 92), read on the device so no
// pass waits for the host. One thread per flush of the batch.
__global__ void scene_uniforms_kernel(FlushParams* __restrict__ scenes, uint32_t sceneCount)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= sceneCount)
        return;
    const uint8_t* u = scenes[i].uniforms;
    const uint32_t granularity = *reinterpret_cast<const uint32_t*>(u + 72);
    scenes[i].pathIDGranularity = granularity ? granularity : 1u;
    scenes[i].ditherScale = *reinterpret_cast<const float*>(u + 88);
    scenes[i].ditherBias = *reinterpret_cast<const float*>(u + 92);
    scenes[i].mipLodBias = *reinterpret_cast<const float*>(u + 80);
}

// Fixed-capacity binning: entries [total, capacity) get the sentinel key (one
// past the batch's last tile) so a sort over the whole capacity leaves them
// at the end, where tile_ranges_kernel ignores them.
template <typename K>
__device__ __forceinline__ void bin_fill(const uint32_t* __restrict__ pairTotal, uint32_t capacity,
                                         uint32_t sentinel, K* __restrict__ keys)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < capacity && i >= *pairTotal)
        keys[i] = (K)sentinel;
}
__global__ void bin_fill_kernel(const uint32_t* __restrict__ pairTotal,
                                uint32_t capacity,
                                uint32_t sentinel,
                                uint32_t* __restrict__ keys)
{
    bin_fill(pairTotal, capacity, sentinel, keys);
}
// 16-bit tile keys (batches of at most 65,535 tiles): the sort moves 6 bytes
// per entry and pass instead of 8.
__global__ void bin_fill16_kernel(const uint32_t* __restrict__ pairTotal,
                                  uint32_t capacity,
                                  uint32_t sentinel,
                                  uint16_t* __restrict__ keys)
{
    bin_fill(pairTotal, capacity, sentinel, keys);
}

// Writes the (tile, slot) pairs of each triangle at its scanned offset. One
// warp per 32 consecutive slots: a lane writes its own triangle's pairs when
// its box spans few tiles; larger triangles are walked by the whole warp with
// a ballot assigning output positions. Pairs at or past `capacity` are
// dropped and flagged (ERR_BIN_OVERFLOW). With kWinding (interior tiles as
// winding records), a deferred fan triangle's large box keeps its path's
// edge tiles only, and an anchor winding slot writes one entry per interior
// tile of its path with a nonzero winding.
template <bool kWinding, typename K>
__device__ __forceinline__ void bin_scatter(const BatchTables* __restrict__ Bw,
                                            uint32_t slotCount,
                                            int tileLog2,
                                            const uint2* __restrict__ sceneTiles,
                                            const TriRecord* __restrict__ tris,
                                            const uint32_t* __restrict__ tileCounts,
                                            const uint8_t* __restrict__ tileMasks,
                                            const uint32_t* __restrict__ offsets,
                                            uint32_t capacity,
                                            uint32_t* __restrict__ error,
                                            K* __restrict__ keys,
                                            uint32_t* __restrict__ vals)
{
    constexpr int kLaneTiles = 8;
    const uint32_t warpId = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const uint32_t first = warpId * 32;
    if (first >= slotCount)
        return;
    const uint32_t mySlot = first + lane;
    const uint32_t myCount = mySlot < slotCount ? tileCounts[mySlot] : 0u;
    bool isBig = false;
    if (myCount)
    {
        const uint4 meta = tris[mySlot].meta;
        const int4 bb = unpack_bbox(meta);
        int tx0, ty0, ntx, nty;
        tile_span(bb, tileLog2, tx0, ty0, ntx, nty);
        if (kWinding && (meta.x & (FEATURE_WINDING_SLOT << 16)))
        {
            isBig = true; // the warp writes a path's winding entries
        }
        else if (ntx * nty <= kLaneTiles)
        {
            // The set-up already tested these tiles: walk its mask.
            const uint2 st = sceneTiles[meta.w >> 16]; // (tileBase, tilesX)
            uint32_t mask = tileMasks[mySlot];
            uint32_t o = offsets[mySlot];
            while (mask)
            {
                const int i = __ffs(mask) - 1;
                mask &= mask - 1;
                const int tx = tx0 + i % ntx, ty = ty0 + i / ntx;
                if (o < capacity)
                {
                    keys[o] = (K)(st.x + (uint32_t)ty * st.y + (uint32_t)tx);
                    vals[o] = mySlot;
                }
                else
                {
                    atomicOr(error, ERR_BIN_OVERFLOW);
                }
                ++o;
            }
        }
        else
        {
            isBig = true;
        }
    }
    uint32_t pending = __ballot_sync(0xffffffffu, isBig);
    while (pending)
    {
        const int t = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t slot = first + t;
        const TriRecord* T = tris + slot;
        const uint4 meta = T->meta;
        const uint2 st = sceneTiles[meta.w >> 16];
        uint32_t o = offsets[slot];
        if (kWinding && (meta.x & (FEATURE_WINDING_SLOT << 16)))
        {
            // The path's grid, from its winding slot's record.
            const uint32_t goff = __float_as_uint(T->e0.x);
            const int gx0 = __float_as_int(T->e0.y), gy0 = __float_as_int(T->e0.z);
            const int gw = __float_as_int(T->e0.w), gh = __float_as_int(T->e1.x);
            const uint32_t cells = (uint32_t)gw * (uint32_t)gh;
            for (uint32_t base = 0; base < cells; base += 32)
            {
                const uint32_t c = base + lane;
                const bool hit =
                    c < cells && !Bw->gridEdge[goff + c] && Bw->gridWinding[goff + c] != 0;
                const uint32_t mask = __ballot_sync(0xffffffffu, hit);
                if (hit)
                {
                    const uint32_t pos = o + __popc(mask & ((1u << lane) - 1u));
                    const int tx = gx0 + (int)(c % (uint32_t)gw), ty = gy0 + (int)(c / (uint32_t)gw);
                    if (pos < capacity)
                    {
                        keys[pos] = (K)(st.x + (uint32_t)ty * st.y + (uint32_t)tx);
                        vals[pos] = BIN_WINDING_ENTRY | slot;
                    }
                    else
                    {
                        atomicOr(error, ERR_BIN_OVERFLOW);
                    }
                }
                o += __popc(mask);
            }
            continue;
        }
        const int4 bb = unpack_bbox(meta);
        const float4 e[3] = {T->e0, T->e1, T->e2};
        const PathGrid* g = (kWinding && (meta.x & (FEATURE_FAN_DEFERRED << 16)))
                                ? winding_grid(*Bw, meta.w >> 16, meta.x & 0xffffu)
                                : nullptr;
        int tx0, ty0, ntx, nty;
        tile_span(bb, tileLog2, tx0, ty0, ntx, nty);
        const int n = ntx * nty;
        for (int base = 0; base < n; base += 32)
        {
            const int i = base + lane;
            bool hit = false;
            int tx = 0, ty = 0;
            if (i < n)
            {
                tx = tx0 + i % ntx;
                ty = ty0 + i / ntx;
                hit = tile_overlaps(e, bb, tx, ty, tileLog2) &&
                      (!kWinding || keep_fan_tile(g, kWinding ? Bw->gridEdge : nullptr, tx, ty));
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, hit);
            if (hit)
            {
                const uint32_t pos = o + __popc(mask & ((1u << lane) - 1u));
                if (pos < capacity)
                {
                    keys[pos] = (K)(st.x + (uint32_t)ty * st.y + (uint32_t)tx);
                    vals[pos] = slot;
                }
                else
                {
                    atomicOr(error, ERR_BIN_OVERFLOW);
                }
            }
            o += __popc(mask);
        }
    }
}

// Resident 256-thread CTAs per SM the binner's registers are bounded for: 6
// (no spills) bins the full-feature frame in 0.98 ms against 1.10 ms at the
// compiler's 45 registers (5 CTAs).
#ifndef RIVE_BIN_MIN_BLOCKS
#define RIVE_BIN_MIN_BLOCKS 6
#endif
__global__ void __launch_bounds__(256, RIVE_BIN_MIN_BLOCKS) bin_scatter_kernel(uint32_t slotCount,
                                                          int tileLog2,
                                                          const uint2* __restrict__ sceneTiles,
                                                          const TriRecord* __restrict__ tris,
                                                          const uint32_t* __restrict__ tileCounts,
                                                          const uint8_t* __restrict__ tileMasks,
                                                          const uint32_t* __restrict__ offsets,
                                                          uint32_t capacity,
                                                          uint32_t* __restrict__ error,
                                                          uint32_t* __restrict__ keys,
                                                          uint32_t* __restrict__ vals)
{
    bin_scatter<false>(nullptr, slotCount, tileLog2, sceneTiles, tris, tileCounts, tileMasks,
                       offsets, capacity, error, keys, vals);
}
__global__ void __launch_bounds__(256, RIVE_BIN_MIN_BLOCKS) bin_scatter16_kernel(uint32_t slotCount,
                                                          int tileLog2,
                                                          const uint2* __restrict__ sceneTiles,
                                                          const TriRecord* __restrict__ tris,
                                                          const uint32_t* __restrict__ tileCounts,
                                                          const uint8_t* __restrict__ tileMasks,
                                                          const uint32_t* __restrict__ offsets,
                                                          uint32_t capacity,
                                                          uint32_t* __restrict__ error,
                                                          uint16_t* __restrict__ keys,
                                                          uint32_t* __restrict__ vals)
{
    bin_scatter<false>(nullptr, slotCount, tileLog2, sceneTiles, tris, tileCounts, tileMasks,
                       offsets, capacity, error, keys, vals);
}

// The same, for batches that draw interior tiles as winding records.
__global__ void __launch_bounds__(256) bin_scatter_winding_kernel(BatchTables B,
                                                                  const TriRecord* __restrict__ tris,
                                                                  const uint32_t* __restrict__ tileCounts,
                                                                  const uint8_t* __restrict__ tileMasks,
                                                                  const uint32_t* __restrict__ offsets,
                                                                  uint32_t slotCount,
                                                                  uint32_t capacity,
                                                                  uint32_t* __restrict__ error,
                                                                  uint32_t* __restrict__ keys,
                                                                  uint32_t* __restrict__ vals)
{
    bin_scatter<true>(&B, slotCount, B.tileLog2, B.sceneTiles, tris, tileCounts, tileMasks,
                      offsets, capacity, error, keys, vals);
}

// A speculative pass whose scanned bin-entry total exceeds the capacity its
// bins were sized for has incomplete bins: every tile's range is emptied, so
// the raster leaves a loaded target as it was (a cleared one is cleared),
// until the back half runs again with exact bins.
__global__ void __launch_bounds__(256) ranges_guard_kernel(const uint32_t* __restrict__ pairTotal,
                                                           uint32_t capacity,
                                                           uint2* __restrict__ ranges,
                                                           uint32_t tiles)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tiles || *pairTotal <= capacity)
        return;
    ranges[i] = make_uint2(0u, 0u);
}

template <typename K>
__device__ __forceinline__ void tile_ranges(uint32_t pairCount, uint32_t tileCount,
                                            const K* __restrict__ keys, uint2* __restrict__ ranges)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pairCount)
        return;
    const uint32_t k = keys[i];
    if (k >= tileCount) // capacity padding
        return;
    if (i == 0 || keys[i - 1] != k)
        ranges[k].x = i;
    if (i == pairCount - 1 || keys[i + 1] != k)
        ranges[k].y = i + 1;
}
__global__ void __launch_bounds__(256) tile_ranges_kernel(uint32_t pairCount,
                                                          uint32_t tileCount,
                                                          const uint32_t* __restrict__ keys,
                                                          uint2* __restrict__ ranges)
{
    tile_ranges(pairCount, tileCount, keys, ranges);
}
__global__ void __launch_bounds__(256) tile_ranges16_kernel(uint32_t pairCount,
                                                            uint32_t tileCount,
                                                            const uint16_t* __restrict__ keys,
                                                            uint2* __restrict__ ranges)
{
    tile_ranges(pairCount, tileCount, keys, ranges);
}

namespace
{
__device__ __forceinline__ uint32_t id_bits_to_f16(uint32_t idBits, uint32_t granularity)
{
    return idBits == 0 ? 0u : ((idBits + MAX_DENORM_F16) * granularity) & 0xffffu;
}
__device__ __forceinline__ float h2f(uint32_t bits)
{
    return __half2float(__ushort_as_half((unsigned short)bits));
}
__device__ __forceinline__ uint32_t f2h(float f)
{
    return (uint32_t)__half_as_ushort(__float2half_rn(f));
}
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
__device__ __forceinline__ uint32_t unorm8(float x)
{
    return (uint32_t)__float2int_rn(clamp01(x) * 255.f);
}
__device__ __forceinline__ void unpack_rgba8(uint32_t c, float out[4])
{
    out[0] = (float)(c & 0xffu) / 255.f;
    out[1] = (float)((c >> 8) & 0xffu) / 255.f;
    out[2] = (float)((c >> 16) & 0xffu) / 255.f;
    out[3] = (float)(c >> 24) / 255.f;
}
__device__ __forceinline__ uint32_t pack_rgba8(const float c[4])
{
    return unorm8(c[0]) | (unorm8(c[1]) << 8) | (unorm8(c[2]) << 16) | (unorm8(c[3]) << 24);
}

__device__ __forceinline__ float min3f(float a, float b, float c) { return fminf(fminf(a, b), c); }
__device__ __forceinline__ float max3f(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }

// advanced_blend.glsl:94-154
__device__ void set_lum(const float base[3], const float lum[3], float out[3])
{
    float lumTarget = lum[0] * .30f + lum[1] * .59f + lum[2] * .11f;
    float lb = base[0] * .30f + base[1] * .59f + base[2] * .11f;
    float bi[3] = {base[0] - lb, base[1] - lb, base[2] - lb};
    float sx = lumTarget / fmaxf(EPSILON_FP16_NON_DENORM, -min3f(bi[0], bi[1], bi[2]));
    float sy = (1.f - lumTarget) / fmaxf(EPSILON_FP16_NON_DENORM, max3f(bi[0], bi[1], bi[2]));
    float s = fminf(1.f, fminf(sx, sy));
    for (int i = 0; i < 3; ++i)
        out[i] = bi[i] * s + lumTarget;
}
__device__ void set_lum_sat(const float hue[3], const float sat[3], const float lum[3], float out[3])
{
    float satTarget = max3f(sat[0], sat[1], sat[2]) - min3f(sat[0], sat[1], sat[2]);
    float mn = min3f(hue[0], hue[1], hue[2]);
    float h[3] = {hue[0] - mn, hue[1] - mn, hue[2] - mn};
    float scale = satTarget / fmaxf(EPSILON_FP16_NON_DENORM, max3f(h[0], h[1], h[2]));
    float hs[3] = {h[0] * scale, h[1] * scale, h[2] * scale};
    set_lum(hs, lum, out);
}

// advanced_color_blend (advanced_blend.glsl:156-327): src unmultiplied,
// dst premultiplied; returns mix(src, coeffs, dst.a).
__device__ __noinline__ void advanced_blend(float src[3], const float dp[4], uint32_t mode)
{
    float inv = dp[3] != 0.f ? 1.f / dp[3] : 0.f;
    float dst[3] = {dp[0] * inv, dp[1] * inv, dp[2] * inv};
    float co[3];
    switch (mode)
    {
        case 11: // multiply
            for (int i = 0; i < 3; ++i) co[i] = src[i] * dst[i];
            break;
        case 1: // screen
            for (int i = 0; i < 3; ++i) co[i] = src[i] + dst[i] - src[i] * dst[i];
            break;
        case 2: // overlay
            for (int i = 0; i < 3; ++i)
            {
                float sd = src[i] * dst[i];
                co[i] = 2.f * (dst[i] > .5f ? src[i] + dst[i] - sd - .5f : sd);
            }
            break;
        case 3: // darken
            for (int i = 0; i < 3; ++i) co[i] = fminf(src[i], dst[i]);
            break;
        case 4: // lighten
            for (int i = 0; i < 3; ++i) co[i] = fmaxf(src[i], dst[i]);
            break;
        case 5: // colordodge
            for (int i = 0; i < 3; ++i)
            {
                float d = fminf(fmaxf(dp[i], 0.f), dp[3]);
                float denom = clamp01(1.f - src[i]) * dp[3];
                co[i] = denom == 0.f ? signf(d) : fminf(1.f, d / denom);
            }
            break;
        case 6: // colorburn
        {
            float a = dp[3] == 0.f ? 1.f : dp[3];
            for (int i = 0; i < 3; ++i)
            {
                float s = clamp01(src[i]);
                float d = fminf(fmaxf(dp[i], 0.f), dp[3]);
                float numer = a - d;
                co[i] = 1.f - (s == 0.f ? signf(numer) : fminf(1.f, numer / (s * a)));
            }
            break;
        }
        case 7: // hardlight
            for (int i = 0; i < 3; ++i)
            {
                float sd = src[i] * dst[i];
                co[i] = 2.f * (src[i] > .5f ? src[i] + dst[i] - sd - .5f : sd);
            }
            break;
        case 8: // softlight
            for (int i = 0; i < 3; ++i)
            {
                float c;
                if (src[i] <= .5f)
                    c = 1.f - dst[i];
                else if (dst[i] <= .25f)
                    c = (16.f * dst[i] - 12.f) * dst[i] + 3.f;
                else
                    c = rsqrtf(dst[i]) - 1.f;
                co[i] = dst[i] + dst[i] * (2.f * src[i] - 1.f) * c;
            }
            break;
        case 9: // difference
            for (int i = 0; i < 3; ++i) co[i] = fabsf(dst[i] - src[i]);
            break;
        case 10: // exclusion
            for (int i = 0; i < 3; ++i) co[i] = src[i] + dst[i] - 2.f * src[i] * dst[i];
            break;
        case 12: case 13: case 14: case 15:
        {
            float s[3] = {clamp01(src[0]), clamp01(src[1]), clamp01(src[2])};
            if (mode == 12) set_lum_sat(s, dst, dst, co);
            else if (mode == 13) set_lum_sat(dst, s, dst, co);
            else if (mode == 14) set_lum(s, dst, co);
            else set_lum(dst, s, co);
            break;
        }
        default:
            co[0] = src[0]; co[1] = src[1]; co[2] = src[2];
            break;
    }
    float a = dp[3];
    for (int i = 0; i < 3; ++i)
        src[i] = src[i] * (1.f - a) + co[i] * a;
}

// Coordinate arithmetic here and in paint_color / clip_rect_distance is
// written with explicit round-to-nearest operations (no contraction into
// fused multiply-adds), in the oracle's order: a gradient coordinate is a
// difference of large terms, and a contracted evaluation lands on the other
// side of a hard colour step at a few pixels.
__device__ __noinline__ void sample_grad(const FlushParams& P, float u, float v, float out[4])
{
    float fx = __fsub_rn(__fmul_rn(u, (float)kGradTextureWidth), .5f);
    // The gradient texture always has at least one row allocated.
    const int H = max((int)P.gradDataHeight, 1);
    float fy = __fsub_rn(__fmul_rn(v, (float)P.gradTextureHeight), .5f);
    float x0f = floorf(fx), y0f = floorf(fy);
    float ax = __fsub_rn(fx, x0f), ay = __fsub_rn(fy, y0f);
    int x0 = (int)x0f, y0 = (int)y0f;
    out[0] = out[1] = out[2] = out[3] = 0.f;
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i)
        {
            int xi = min(max(x0 + i, 0), kGradTextureWidth - 1);
            int yj = min(max(y0 + j, 0), H - 1);
            float wgt = __fmul_rn(i ? ax : __fsub_rn(1.f, ax), j ? ay : __fsub_rn(1.f, ay));
            uchar4 t = P.grad[(size_t)yj * kGradTextureWidth + xi];
            out[0] = __fadd_rn(out[0], __fmul_rn(wgt, __fdiv_rn((float)t.x, 255.f)));
            out[1] = __fadd_rn(out[1], __fmul_rn(wgt, __fdiv_rn((float)t.y, 255.f)));
            out[2] = __fadd_rn(out[2], __fmul_rn(wgt, __fdiv_rn((float)t.z, 255.f)));
            out[3] = __fadd_rn(out[3], __fmul_rn(wgt, __fdiv_rn((float)t.w, 255.f)));
        }
}

// Pixel-local storage of one pixel (draw_raster_order_path.frag:7-12), plus
// the path whose fragments are still being accumulated.
struct Pixel
{
    uint32_t color;    // RGBA8, the colour before the pending path
    uint32_t clip;     // packHalf2x16(coverage, clipID)
    uint32_t scratch;  // RGBA8 scratch plane
    uint32_t key;      // coverage plane's path key (fp16 bits of the pathID)
    float count;       // coverage plane's count (always an fp16 value)
    uint32_t pendMeta; // pathAndFeatures of the pending path (0: none)
    uint32_t pendPaintX, pendPaintY;
    uint32_t pendFrags; // fragments of the pending path so far (saturating)
};

// min_component of find_clip_rect_coverage_distances (common.glsl:376-400)
// at the pixel centre, for the clip-rect inverse matrix cm (2x2) and its
// translate ct.xy.
__device__ __forceinline__ float clip_rect_distance_m(float4 cm, float4 ct, float fx, float fy)
{
    float awx = fabsf(cm.x) + fabsf(cm.z), awy = fabsf(cm.y) + fabsf(cm.w);
    float d0, d1, d2, d3;
    if (awx != 0.f && awy != 0.f)
    {
        float rx = __fdiv_rn(1.f, awx), ry = __fdiv_rn(1.f, awy);
        float cx = __fadd_rn(__fadd_rn(__fmul_rn(cm.x, fx), __fmul_rn(cm.z, fy)), ct.x);
        float cy = __fadd_rn(__fadd_rn(__fmul_rn(cm.y, fx), __fmul_rn(cm.w, fy)), ct.y);
        d0 = __fadd_rn(__fadd_rn(__fmul_rn(cx, rx), rx), .5f);
        d1 = __fadd_rn(__fadd_rn(__fmul_rn(cy, ry), ry), .5f);
        d2 = __fadd_rn(__fadd_rn(__fmul_rn(-cx, rx), rx), .5f);
        d3 = __fadd_rn(__fadd_rn(__fmul_rn(-cy, ry), ry), .5f);
    }
    else
    {
        d0 = d2 = ct.x;
        d1 = d3 = ct.y;
    }
    return fminf(fminf(d0, d1), fminf(d2, d3));
}

// A path's clip rect: the inverse matrix of its PaintAuxData (words 8-13).
__device__ __forceinline__ float clip_rect_distance(const FlushParams& P, uint32_t pathID, float fx,
                                                    float fy)
{
    const float4* aux = P.paintAux + 8 * (size_t)(P.firstPaintAux + pathID);
    return clip_rect_distance_m(aux[2], aux[3], fx, fy);
}

// find_paint_color (draw_path.vert:431-496, evaluated at the pixel): the
// paint's colour with its alpha multiplied by `coverage`, premultiplied
// unless advanced blending wants it straight.
__device__ __noinline__ void image_modulate(const FlushParams& P, uint32_t pathID, float fx,
                                            float fy, bool unmultiplied, float color[4]);

__device__ __forceinline__ void paint_color(const FlushParams& P, uint32_t paintX, uint32_t paintY,
                                            uint32_t pathID, float fx, float fy, float coverage,
                                            bool unmultiplied, float color[4],
                                            uint32_t features = 0)
{
    const uint32_t paintType = paintX & 0xfu;
    if (paintType == SOLID_COLOR_PAINT_TYPE)
    {
        unpack_rgba8(paintY, color);
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
    else if (paintType == LINEAR_GRADIENT_PAINT_TYPE || paintType == RADIAL_GRADIENT_PAINT_TYPE)
    {
        const float4* aux = P.paintAux + 8 * (size_t)(P.firstPaintAux + pathID);
        float4 pm = aux[0], pt = aux[1];
        float pcx = __fadd_rn(__fadd_rn(__fmul_rn(pm.x, fx), __fmul_rn(pm.z, fy)), pt.x);
        float pcy = __fadd_rn(__fadd_rn(__fmul_rn(pm.y, fx), __fmul_rn(pm.w, fy)), pt.y);
        float spanB = pt.z > .9f ? 2.f : pt.w;
        float t = paintType == LINEAR_GRADIENT_PAINT_TYPE
                      ? pcx
                      : __fsqrt_rn(__fadd_rn(__fmul_rn(pcx, pcx), __fmul_rn(pcy, pcy)));
        t = clamp01(t);
        float x = spanB > 1.f ? __fadd_rn(__fmul_rn(1.f - 1.f / kGradTextureWidth, t),
                                          .5f / kGradTextureWidth)
                              : __fadd_rn(__fmul_rn(1.f / kGradTextureWidth, t), spanB);
        sample_grad(P, x, __uint_as_float(paintY), color);
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
        color[0] = color[1] = color[2] = color[3] = 0.f;
    }
    if ((features & SF_MODULATED_IMAGE) && (paintX & PAINT_FLAG_HAS_IMAGE) && P.pathImage)
        image_modulate(P, pathID, fx, fy, unmultiplied, color);
}

// An image texel address under a wrap mode (the Vulkan sampler address modes
// the reference maps ImageWrap to, pipeline_manager_vulkan.cpp:25-38): clamp
// to edge, repeat, mirrored repeat.
__device__ __forceinline__ int wrap_texel(int i, int n, uint32_t wrap)
{
    if (wrap == 1)
    {
        i %= n;
        return i < 0 ? i + n : i;
    }
    if (wrap == 2)
    {
        int m = i % (2 * n);
        if (m < 0)
            m += 2 * n;
        const int a = m - n; // mirror(a) = a >= 0 ? a : -(1 + a)
        return (n - 1) - (a >= 0 ? a : -(1 + a));
    }
    return min(max(i, 0), n - 1);
}

// The image sampled at normalised coordinates (u, v) with an explicit level of
// detail (TEXTURE_SAMPLE_DYNAMIC_LOD): the sampler's filter within the level
// a nearest mip selection picks (VK_SAMPLER_MIPMAP_MODE_NEAREST,
// pipeline_manager_vulkan.cpp:13-23: level ceil(lod + 1/2) - 1 above 1/2,
// else 0), RGBA as floats.
__device__ void sample_image_level(const ImageTex& t, int level, float u, float v, float out[4])
{
    const uint32_t wrapX = t.sampler % 3u, wrapY = (t.sampler / 3u) % 3u;
    const bool nearest = t.sampler >= 9u;
    const int w = max((int)(t.width >> level), 1), h = max((int)(t.height >> level), 1);
    const uchar4* tex = t.texels + t.off[level];
    if (nearest)
    {
        const int x = wrap_texel((int)floorf(__fmul_rn(u, (float)w)), w, wrapX);
        const int y = wrap_texel((int)floorf(__fmul_rn(v, (float)h)), h, wrapY);
        const uchar4 c = tex[(size_t)y * w + x];
        out[0] = __fdiv_rn((float)c.x, 255.f);
        out[1] = __fdiv_rn((float)c.y, 255.f);
        out[2] = __fdiv_rn((float)c.z, 255.f);
        out[3] = __fdiv_rn((float)c.w, 255.f);
        return;
    }
    const float fx = __fsub_rn(__fmul_rn(u, (float)w), .5f);
    const float fy = __fsub_rn(__fmul_rn(v, (float)h), .5f);
    const float x0f = floorf(fx), y0f = floorf(fy);
    const float ax = __fsub_rn(fx, x0f), ay = __fsub_rn(fy, y0f);
    const int x0 = (int)x0f, y0 = (int)y0f;
    out[0] = out[1] = out[2] = out[3] = 0.f;
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int i = 0; i < 2; ++i)
        {
            const int xi = wrap_texel(x0 + i, w, wrapX), yj = wrap_texel(y0 + j, h, wrapY);
            const float wgt = __fmul_rn(i ? ax : __fsub_rn(1.f, ax), j ? ay : __fsub_rn(1.f, ay));
            const uchar4 c = tex[(size_t)yj * w + xi];
            out[0] = __fadd_rn(out[0], __fmul_rn(wgt, __fdiv_rn((float)c.x, 255.f)));
            out[1] = __fadd_rn(out[1], __fmul_rn(wgt, __fdiv_rn((float)c.y, 255.f)));
            out[2] = __fadd_rn(out[2], __fmul_rn(wgt, __fdiv_rn((float)c.z, 255.f)));
            out[3] = __fadd_rn(out[3], __fmul_rn(wgt, __fdiv_rn((float)c.w, 255.f)));
        }
}

__device__ void sample_image(const ImageTex& t, float u, float v, float lod, float out[4])
{
    int level = 0;
    if (lod > .5f)
        level = min((int)ceilf(__fadd_rn(lod, .5f)) - 1, (int)t.levels - 1);
    sample_image_level(t, level, u, v, out);
}

// One fragment of an image-mesh triangle (draw_mesh.frag:60-225 with
// DRAW_IMAGE_MESH), written at once: the image at the triangle's texture
// coordinates of the pixel (planes in the slot's feather-plane pair, exact
// per pixel), at the mip level the set-up chose for the triangle; coverage 1,
// cut by the clip rect and the clip, then times the draw's opacity; advanced
// blending unmultiplies the texel first; dither, then src-over onto the
// colour. The coverage plane keeps what it held (a mesh is no path).
__device__ __noinline__ void resolve_mesh(const FlushParams& P, Pixel& s, uint32_t meta,
                                          uint32_t imageDraw, uint32_t imageWord,
                                          const float4* __restrict__ planes, float fx, float fy,
                                          float dither)
{
    const uint32_t features = meta >> 16;
    const float4 f0 = planes[0], f1 = planes[1];
    const float dx = __fsub_rn(fx, f1.z), dy = __fsub_rn(fy, f1.w);
    const float u = __fadd_rn(__fadd_rn(f0.x, __fmul_rn(f0.y, dx)), __fmul_rn(f0.z, dy));
    const float v = __fadd_rn(__fadd_rn(f0.w, __fmul_rn(f1.x, dx)), __fmul_rn(f1.y, dy));
    float color[4];
    sample_image_level(P.images[imageWord & 0xffffffu], (int)(imageWord >> 24), u, v, color);
    const float4* inst = P.imageDraws + 4 * (size_t)imageDraw;
    const float4 packed = inst[3];
    float coverage = 1.f;
    if (features & SF_CLIP_RECT)
    {
        const float4 tr = inst[2];
        coverage = fminf(fmaxf(clip_rect_distance_m(inst[1], make_float4(tr.z, tr.w, 0.f, 0.f),
                                                    fx, fy),
                               0.f),
                         coverage);
    }
    if (features & SF_CLIPPING)
    {
        const uint32_t clipBits = id_bits_to_f16(__float_as_uint(packed.y), P.pathIDGranularity);
        if (clipBits != 0)
        {
            const float clipCoverage = (s.clip >> 16) == clipBits ? h2f(s.clip & 0xffffu) : 0.f;
            coverage = fminf(coverage, fmaxf(clipCoverage, 0.f));
        }
    }
    coverage = __fmul_rn(coverage, packed.x); // opacity, after clipping
    float dst[4];
    unpack_rgba8(s.color, dst);
    if (features & SF_ADVANCED_BLEND)
    {
        // unmultiply_rgb (common.glsl:210-216): images are premultiplied.
        const float r = color[3] != 0.f ? __fdiv_rn(1.f, color[3]) : 0.f;
        color[0] = __fmul_rn(color[0], r);
        color[1] = __fmul_rn(color[1], r);
        color[2] = __fmul_rn(color[2], r);
        const uint32_t mode = __float_as_uint(packed.z);
        if (mode != 0 && (mode < 12 || (features & SF_HSL_BLEND_MODES)))
            advanced_blend(color, dst, mode);
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
        color[0] += dither;
        color[1] += dither;
        color[2] += dither;
    }
    const float a = color[3];
    for (int k = 0; k < 4; ++k)
        color[k] = dst[k] * (1.f - a) + color[k];
    s.color = pack_rgba8(color);
}

// ENABLE_MODULATED_IMAGE (draw_path.vert:343-361, 478-493): the paint's
// colour times the image the path's batch binds, sampled at the image matrix
// applied to the pixel centre, at the level of detail the front end computed
// (PaintAuxData words 16-22: image matrix, translate, LOD). The texels are
// premultiplied; advanced blending wants them straight.
__device__ __noinline__ void image_modulate(const FlushParams& P, uint32_t pathID, float fx,
                                            float fy, bool unmultiplied, float color[4])
{
    const uint32_t slot = P.pathImage[pathID];
    if (slot == kNoImage)
        return;
    const float4* aux = P.paintAux + 8 * (size_t)(P.firstPaintAux + pathID);
    const float4 m = aux[4], tl = aux[5];
    const float u = __fadd_rn(__fadd_rn(__fmul_rn(m.x, fx), __fmul_rn(m.z, fy)), tl.x);
    const float v = __fadd_rn(__fadd_rn(__fmul_rn(m.y, fx), __fmul_rn(m.w, fy)), tl.y);
    // v_image.z = 1 + lod in the vertex shader, lod = v_image.z - 1 in the
    // fragment shader.
    const float lod = __fsub_rn(__fadd_rn(1.f, tl.z), 1.f);
    float img[4];
    sample_image(P.images[slot], u, v, lod, img);
    if (unmultiplied && img[3] != 0.f)
    {
        img[0] = __fdiv_rn(img[0], img[3]);
        img[1] = __fdiv_rn(img[1], img[3]);
        img[2] = __fdiv_rn(img[2], img[3]);
    }
    for (int k = 0; k < 4; ++k)
        color[k] = __fmul_rn(color[k], img[k]);
}

// The colour / clip write of the last fragment of a path at this pixel.
//
// draw_raster_order_path.frag writes the colour (or clip) plane on every
// fragment, each time from the path's accumulated coverage and the same dst
// colour (stashed at the path's first fragment); only the last write
// survives. Evaluating it once, when the next path arrives or the tile ends,
// gives the same result. The one value an earlier fragment feeds forward is
// the nested-clip stash, which the reference keeps in RGBA8: its
// quantisation is applied when the path had more than one fragment here.
// kImages: the image paint is compiled in (the raster's feather variants,
// which batches with images or feathers use); the plain variant's resolve
// stays without it.
template <bool kImages>
__device__ __noinline__ void resolve_path(const FlushParams& P, Pixel& s, float fx, float fy,
                                          float dither)
{
    const uint32_t meta = s.pendMeta;
    const uint32_t pathID = meta & 0xffffu, features = meta >> 16;
    const uint32_t paintX = s.pendPaintX, paintY = s.pendPaintY;
    const uint32_t paintType = paintX & 0xfu;
    const bool evenOdd = (paintX & PAINT_FLAG_EVEN_ODD_FILL) != 0;
    // draw_raster_order_path.frag:63-82: clockwise fills keep positive
    // windings only; otherwise nonzero or even-odd.
    float coverage;
    if (features & FEATURE_CLOCKWISE_FILL)
    {
        coverage = fminf(fmaxf(s.count, 0.f), 1.f);
    }
    else
    {
        coverage = fabsf(s.count);
        if ((features & SF_EVEN_ODD) && evenOdd)
            coverage = 1.f - fabsf((coverage * .5f - floorf(coverage * .5f)) * 2.f + -1.f);
        coverage = fminf(coverage, 1.f);
    }

    if (features & SF_CLIPPING)
    {
        const uint32_t clipBits = id_bits_to_f16(
            (paintType == CLIP_UPDATE_PAINT_TYPE ? paintY : paintX) >> 16, P.pathIDGranularity);
        if (paintType == CLIP_UPDATE_PAINT_TYPE && clipBits != 0)
        {
            if (features & SF_NESTED_CLIPPING)
            {
                const uint32_t outerBits = id_bits_to_f16(paintX >> 16, P.pathIDGranularity);
                if (outerBits != 0)
                {
                    const uint32_t contentID = s.clip >> 16;
                    float outer;
                    if (contentID != clipBits)
                    {
                        outer = contentID == outerBits ? h2f(s.clip & 0xffffu) : 0.f;
                        const uint32_t stash = unorm8(outer);
                        s.scratch = stash;
                        if (s.pendFrags > 1)
                            outer = (float)stash / 255.f;
                    }
                    else
                    {
                        outer = (float)(s.scratch & 0xffu) / 255.f;
                    }
                    coverage = fminf(coverage, outer);
                }
            }
            s.clip = (clipBits << 16) | f2h(coverage);
            return;
        }
        if (clipBits != 0)
            coverage = (s.clip >> 16) == clipBits ? fminf(h2f(s.clip & 0xffffu), coverage) : 0.f;
    }
    if (features & SF_CLIP_RECT)
        coverage = fminf(fmaxf(clip_rect_distance(P, pathID, fx, fy), 0.f), coverage);

    const bool unmultiplied = (features & SF_ADVANCED_BLEND) != 0;
    float color[4];
    paint_color(P, paintX, paintY, pathID, fx, fy, coverage, unmultiplied, color,
                kImages ? features : 0u);

    float dst[4];
    unpack_rgba8(s.color, dst);
    s.scratch = s.color;
    if (unmultiplied)
    {
        uint32_t mode = (paintX >> 4) & 0xfu;
        if (mode != 0 && (mode < 12 || (features & SF_HSL_BLEND_MODES)))
            advanced_blend(color, dst, mode);
        color[0] *= color[3];
        color[1] *= color[3];
        color[2] *= color[3];
    }
    const float paintAlpha = color[3];
    for (int k = 0; k < 4; ++k)
        color[k] += dst[k] * (1.f - paintAlpha);
    if ((features & SF_DITHER) && paintAlpha != 0.f)
    {
        color[0] += dither;
        color[1] += dither;
        color[2] += dither;
    }
    s.color = pack_rgba8(color);
}

// The feather atlas at atlas pixel coordinates (x, y): the atlas sampler's
// linear filter with clamp-to-edge addressing (draw_mesh.frag:89-97), texel
// centres at half-integers, addresses clamped to the atlas content; then
// clamped to [0, 1].
__device__ __noinline__ float atlas_coverage(const FlushParams& P, float x, float y)
{
    const uint16_t* __restrict__ a = P.atlas;
    const int W = (int)P.atlasW, H = (int)P.atlasH;
    if (!a || W <= 0 || H <= 0)
        return 0.f;
    const float u = __fsub_rn(x, .5f), v = __fsub_rn(y, .5f);
    if (!(u == u) || !(v == v))
        return 0.f;
    const float fu = floorf(u), fv = floorf(v);
    const float wu = __fsub_rn(u, fu), wv = __fsub_rn(v, fv);
    const int iu = (int)fminf(fmaxf(fu, -1.f), (float)W), iv = (int)fminf(fmaxf(fv, -1.f), (float)H);
    const int u0 = min(max(iu, 0), W - 1), u1 = min(max(iu + 1, 0), W - 1);
    const int v0 = min(max(iv, 0), H - 1), v1 = min(max(iv + 1, 0), H - 1);
    const float t00 = h2f(a[(size_t)v0 * W + u0]), t10 = h2f(a[(size_t)v0 * W + u1]);
    const float t01 = h2f(a[(size_t)v1 * W + u0]), t11 = h2f(a[(size_t)v1 * W + u1]);
    const float top = __fadd_rn(t00, __fmul_rn(__fsub_rn(t10, t00), wu));
    const float bot = __fadd_rn(t01, __fmul_rn(__fsub_rn(t11, t01), wu));
    const float c = __fadd_rn(top, __fmul_rn(__fsub_rn(bot, top), wv));
    return fminf(fmaxf(c, 0.f), 1.f);
}

// One fragment of a featherAtlasBlit draw (draw_mesh.frag:60-225 with
// FEATHER_ATLAS_BLIT), written at once: the blit's two triangles never
// overlap, so it is the path's only fragment at the pixel. The coverage is
// the atlas sample, cut by the clip rect and the clip; the paint blends
// straight into the colour (dither before the blend, as that shader does);
// the coverage plane keeps what it held.
__device__ __noinline__ void resolve_blit(const FlushParams& P, Pixel& s, uint32_t meta,
                                          uint32_t paintX, uint32_t paintY, float ax, float ay,
                                          float fx, float fy, float dither)
{
    const uint32_t pathID = meta & 0xffffu, features = meta >> 16;
    const uint32_t paintType = paintX & 0xfu;
    float coverage = atlas_coverage(P, ax, ay);
    if (features & SF_CLIP_RECT)
        coverage = fminf(fmaxf(clip_rect_distance(P, pathID, fx, fy), 0.f), coverage);
    if (features & SF_CLIPPING)
    {
        const uint32_t clipBits = id_bits_to_f16(
            (paintType == CLIP_UPDATE_PAINT_TYPE ? paintY : paintX) >> 16, P.pathIDGranularity);
        if (clipBits != 0)
        {
            float clipCoverage = (s.clip >> 16) == clipBits ? h2f(s.clip & 0xffffu) : 0.f;
            coverage = fminf(coverage, fmaxf(clipCoverage, 0.f));
        }
    }
    const bool unmultiplied = (features & SF_ADVANCED_BLEND) != 0;
    float color[4];
    paint_color(P, paintX, paintY, pathID, fx, fy, 1.f, unmultiplied, color, features);
    float dst[4];
    unpack_rgba8(s.color, dst);
    if (unmultiplied)
    {
        uint32_t mode = (paintX >> 4) & 0xfu;
        if (mode != 0 && (mode < 12 || (features & SF_HSL_BLEND_MODES)))
            advanced_blend(color, dst, mode);
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
        color[0] += dither;
        color[1] += dither;
        color[2] += dither;
    }
    const float a = color[3];
    for (int k = 0; k < 4; ++k)
        color[k] = dst[k] * (1.f - a) + color[k];
    s.color = pack_rgba8(color);
}
} // namespace

// One CTA per 16x16 tile, one thread per pixel; warp w owns the 8x4 block at
// (8 (w & 1), 4 (w >> 1)). The tile's bin entries (triangle slots in
// primitive order) are staged 256 at a time into shared memory in tile-local
// form, each with a mask of the warp blocks it may cover; warps then walk
// their own triangles in order and keep every pixel's planes in registers.
struct __align__(16) TileTri
{
    float4 v0; // coverage key (bits), C0, A0, B0
    float4 v1; // C1, A1, B1, C2
    float4 v2; // A2, B2, covx at the tile origin, d covx/dx
    float4 v3; // d covx/dy, covy at the tile origin, d covy/dx, d covy/dy
    uint4 v4;  // paint.x, paint.y, pathAndFeatures, triangle slot
};
static_assert(sizeof(TileTri) == 80, "TileTri layout");

// The 512-entry feather table (the integral of the normal distribution over
// -3..+3 standard deviations, fp16 values widened to float), written by the
// host once per device (ensure_feather_lut, end of this file) before any flush.
__device__ float g_featherLUT[kGaussianTableSize];

// FEATHER(x) (common.glsl:53-60): the table sampled at normalised x with a
// linear filter and clamp-to-edge addressing.
__device__ __noinline__ float feather_lut(float x)
{
    const float t = __fsub_rn(__fmul_rn(x, (float)kGaussianTableSize), .5f);
    if (!(t == t))
        return g_featherLUT[0];
    const float f = floorf(t);
    const float w = __fsub_rn(t, f);
    const float fc = fminf(fmaxf(f, -1.f), (float)kGaussianTableSize);
    const int i0 = (int)fc;
    const int a = min(max(i0, 0), kGaussianTableSize - 1);
    const int b = min(max(i0 + 1, 0), kGaussianTableSize - 1);
    const float va = g_featherLUT[a], vb = g_featherLUT[b];
    return __fadd_rn(va, __fmul_rn(__fsub_rn(vb, va), w));
}

// eval_feathered_stroke (draw_path_common.glsl:242-258):
// 1 - feather(1 - leftCoverage) - feather(1 - rightCoverage), the left
// coverage carried biased by the feather bias.
__device__ __forceinline__ float eval_feathered_stroke(float covx, float covy)
{
    float c = 1.f;
    c = __fsub_rn(c, feather_lut(__fadd_rn(1.f - kFeatherCoverageBias, covx)));
    c = __fsub_rn(c, feather_lut(__fsub_rn(1.f, covy)));
    return c;
}

// eval_feathered_fill (draw_path_common.glsl:152-240): the feather of a flat
// edge, or, at a feather join, of a corner: the coverage of the first edge
// plus a 4-sample Gaussian quadrature of the second edge's integral.
__device__ float eval_feathered_fill(float cx, float cy, float cotTheta, float y0)
{
    y0 = fmaxf(y0, 0.f);
    float featherCoverage = cotTheta >= 0.f ? feather_lut(y0) : 0.f;
    if (fabsf(cotTheta) < kHorizontalCotangentThreshold)
    {
        const float x = __fsub_rn(fabsf(cx), kFeatherXCoordBias);
        const float y = __fadd_rn(-cy, kFeatherCoverageBias);
        const float dt = __fmul_rn(__fsub_rn(y, y0), 0.5984134206f);
        const float k[4] = {0.20888568955f, 0.62665706865f, 1.04442844776f, 1.46219982687f};
        const float c = __fadd_rn(__fmul_rn(y, cotTheta), x);
        float sum = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            const float t = __fadd_rn(y0, __fmul_rn(dt, k[i]));
            const float u = __fadd_rn(__fmul_rn(t, -cotTheta), c);
            const float tt = __fadd_rn(__fmul_rn(t, 5.09593080173f), -2.54796540086f);
            sum = __fadd_rn(sum, __fmul_rn(feather_lut(u), exp2f(-__fmul_rn(tt, tt))));
        }
        featherCoverage = __fadd_rn(featherCoverage, __fmul_rn(sum, dt));
    }
    return __fmul_rn(featherCoverage, signf(cx));
}

// A feathered fragment: a stroke's (covy >= 0), or a fill's, whose third and
// fourth coverage components come from the slot's planes. One out-of-line
// call site keeps the raster loop's register allocation as it is without
// feathers.
__device__ __noinline__ float feathered_fragment(const float4* __restrict__ planes, uint32_t slot,
                                                 float fx, float fy, float covx, float covy)
{
    if (covy >= 0.f)
        return eval_feathered_stroke(covx, covy);
    if (!planes)
        return covx;
    const float4 f0 = planes[2 * (size_t)slot], f1 = planes[2 * (size_t)slot + 1];
    const float dx = fx - f1.z, dy = fy - f1.w;
    const float covz = f0.x + f0.y * dx + f0.z * dy;
    const float covw = f0.w + f1.x * dx + f1.y * dy;
    return eval_feathered_fill(covx, covy, covz, covw);
}

// Resident CTAs per SM the register allocation is bounded for (16x16 tiles).
#ifndef RIVE_RASTER_MIN_BLOCKS
#define RIVE_RASTER_MIN_BLOCKS 5
#endif
// Prefetch of the next chunk's records into L2 while a chunk is walked (off:
// measured slower, the staging's loads are not what the barrier waits for).
#ifndef RIVE_RASTER_PREFETCH
#define RIVE_RASTER_PREFETCH 0
#endif
// Bin entries each thread stages per chunk (8x8 and 16x16 tiles): a chunk of
// kStage x threads entries between two CTA barriers.
#ifndef RIVE_RASTER_STAGE
#define RIVE_RASTER_STAGE 1
#endif

// Tile geometry: a CTA of T x T threads, one per pixel; warp w owns the 8x4
// block at (8 (w % (T/8)), 4 (w / (T/8))).
template <int TL> struct RasterTile
{
    static constexpr int T = 1 << TL;
    static constexpr int kThreads = T * T;
    static constexpr int kWarpCols = T / 8;
    static constexpr int kBlocks = kThreads / 32;
    using Mask = typename std::conditional<(kBlocks <= 8), uint8_t, uint32_t>::type;
};

template <int TL, bool kFeather, int kStage>
__device__ __forceinline__ void raster_tile(const BatchTables& B,
                                            const TriRecord* __restrict__ tris,
                                            const uint32_t* __restrict__ sortedSlots,
                                            const uint2* __restrict__ ranges,
                                            TileTri* __restrict__ sTris,
                                            typename RasterTile<TL>::Mask* __restrict__ sMask,
                                            uint32_t gtile)
{
    using G = RasterTile<TL>;
    static_assert(sizeof(FlushParams) / 4 <= G::kThreads, "one word of FlushParams per thread");
    __shared__ FlushParams sP;
    const uint2 range = ranges[gtile];
    // The tile's scene: its parameters are staged once for the whole CTA.
    const uint32_t scene = find_range(B.tileBase, B.sceneCount, gtile);
    if (threadIdx.x < sizeof(FlushParams) / 4)
        reinterpret_cast<uint32_t*>(&sP)[threadIdx.x] =
            reinterpret_cast<const uint32_t*>(B.scenes + scene)[threadIdx.x];
    __syncthreads();
    const FlushParams& P = sP;
    uint32_t* __restrict__ fb = P.fb;
    const uint32_t tilesX = P.tilesX;
    const uint32_t tile = gtile - B.tileBase[scene];
    const int tx = (int)(tile % tilesX), ty = (int)(tile / tilesX);
    const int ox = tx * G::T, oy = ty * G::T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lxi = (warp % G::kWarpCols) * 8 + (lane & 7), lyi = (warp / G::kWarpCols) * 4 + (lane >> 3);
    const int px = ox + lxi, py = oy + lyi;
    const float lx = (float)lxi, ly = (float)lyi;
    const bool inBounds = px < (int)P.width && py < (int)P.height;
    if (range.y <= range.x && !P.loadClear)
        return;
    Pixel s;
    s.color = P.loadClear ? P.clearColorPremulRGBA : (inBounds ? fb[(size_t)py * P.width + px] : 0u);
    s.clip = 0;
    s.scratch = 0;
    s.key = 0;
    s.count = 0.f;
    s.pendMeta = 0;
    s.pendPaintX = s.pendPaintY = 0;
    s.pendFrags = 0;
    const float fx = (float)px + .5f, fy = (float)py + .5f;
    // common.glsl:269-274 interleaved gradient noise (depends on the pixel
    // only). Rounded step by step as the C restatement rounds it: the noise
    // wraps at fract(), where a fused multiply-add's last bit moves a pixel's
    // dither by a whole step, and chains of advanced blends amplify it.
    float v1 = __fadd_rn(__fmul_rn(0.06711056f, fx), __fmul_rn(0.00583715f, fy));
    v1 = __fsub_rn(v1, floorf(v1));
    float v2 = __fmul_rn(52.9829189f, v1);
    v2 = __fsub_rn(v2, floorf(v2));
    const float dither = __fadd_rn(__fmul_rn(v2, P.ditherScale), P.ditherBias);
    uint32_t streamPath = 0xffffffffu; // coverage key of the warp's current path

    constexpr uint32_t kChunk = (uint32_t)G::kThreads * kStage;
    for (uint32_t base = range.x; base < range.y; base += kChunk)
    {
        // Each thread stages kStage triangles in tile-local form and marks
        // which of the warp blocks may hold a pixel each covers.
#pragma unroll
        for (int j = 0; j < kStage; ++j)
        {
        const uint32_t si = (uint32_t)j * G::kThreads + threadIdx.x;
        const uint32_t k = base + si;
        uint32_t m = 0;
        const uint32_t entry = k < range.y ? sortedSlots[k] : 0u;
        if (k < range.y && (entry & BIN_WINDING_ENTRY))
        {
            // A winding entry: the path's winding W on this interior tile, as
            // a "triangle" covering every pixel with constant fill coverage W
            // (edge functions 1, coverage planes flat).
            const TriRecord& R = tris[entry & ~BIN_WINDING_ENTRY];
            const float4 ge = R.e0;
            const uint32_t cell = __float_as_uint(ge.x) +
                                  (uint32_t)(ty - __float_as_int(ge.z)) * (uint32_t)__float_as_int(ge.w) +
                                  (uint32_t)(tx - __float_as_int(ge.y));
            const float W = (float)B.gridWinding[cell];
            const uint4 meta = R.meta;
            const float4 cv = R.cov1;
            TileTri L;
            L.v0 = make_float4(__uint_as_float(meta.w & 0xffffu), 1.f, 0.f, 0.f);
            L.v1 = make_float4(1.f, 0.f, 0.f, 1.f);
            L.v2 = make_float4(0.f, 0.f, W, 0.f);
            L.v3 = make_float4(0.f, -1.f, 0.f, 0.f);
            L.v4 = make_uint4(__float_as_uint(cv.z), __float_as_uint(cv.w), meta.x, 0u);
            sTris[si] = L;
            m = G::kBlocks >= 32 ? 0xffffffffu : ((1u << (G::kBlocks & 31)) - 1u);
        }
        else if (k < range.y)
        {
            const TriRecord T = tris[entry];
            const float4 e[3] = {T.e0, T.e1, T.e2};
            const float c[3] = {tile_edge_origin(e[0], tx, ty, TL),
                                tile_edge_origin(e[1], tx, ty, TL),
                                tile_edge_origin(e[2], tx, ty, TL)};
            const float dx0 = (float)ox + .5f - T.e0.x, dy0 = (float)oy + .5f - T.e0.y;
            TileTri L;
            L.v0 = make_float4(__uint_as_float(T.meta.w & 0xffffu), c[0], e[0].z, e[0].w);
            L.v1 = make_float4(c[1], e[1].z, e[1].w, c[2]);
            L.v2 = make_float4(e[2].z, e[2].w, T.cov0.x + T.cov0.y * dx0 + T.cov0.z * dy0,
                               T.cov0.y);
            L.v3 = make_float4(T.cov0.z, T.cov0.w + T.cov1.x * dx0 + T.cov1.y * dy0, T.cov1.x,
                               T.cov1.y);
            L.v4 = make_uint4(__float_as_uint(T.cov1.z), __float_as_uint(T.cov1.w), T.meta.x,
                              entry);
            sTris[si] = L;
            const int4 bb = unpack_bbox(T.meta);
            const int bx0 = bb.x - ox, bx1 = bb.z - ox, by0 = bb.y - oy, by1 = bb.w - oy;
#pragma unroll
            for (int b = 0; b < G::kBlocks; ++b)
            {
                const int qx = (b % G::kWarpCols) * 8, qy = (b / G::kWarpCols) * 4;
                const int x0 = max(bx0, qx), x1 = min(bx1, qx + 8);
                const int y0 = max(by0, qy), y1 = min(by1, qy + 4);
                if (x0 < x1 && y0 < y1 && local_rect_overlaps(c, e, x0, x1, y0, y1))
                    m |= 1u << b;
            }
        }
        sMask[si] = (typename G::Mask)m;
        }
        __syncthreads();
#if RIVE_RASTER_PREFETCH
        // The next chunk's records are pulled into L2 while this one is
        // walked, so the staging after the next barrier does not wait on DRAM.
        if (kStage == 1)
        {
            const uint32_t kn = base + kChunk + threadIdx.x;
            if (kn < range.y)
            {
                const uint32_t en = __ldg(sortedSlots + kn) & ~BIN_WINDING_ENTRY;
                const char* a = reinterpret_cast<const char*>(tris + en);
                asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(a + sizeof(TriRecord) - 1));
            }
        }
#endif
        const uint32_t n = min(kChunk, range.y - base);
        for (uint32_t g = 0; g < n; g += 32)
        {
            // Triangles of this group touching this warp's block, in order.
            uint32_t bits = __ballot_sync(0xffffffffu, (sMask[g + lane] >> warp) & 1u);
            while (bits)
            {
                const uint32_t i = g + (uint32_t)(__ffs(bits) - 1);
                bits &= bits - 1;
                const TileTri& T = sTris[i];
                const float4 v0 = T.v0;
                const uint32_t vPathID = __float_as_uint(v0.x);
                // A path's triangles are contiguous in primitive order, so when
                // the warp's stream moves to another path every pixel still
                // holding the previous path's coverage has seen all of it:
                // resolve them together (one convergent call per path).
                if (vPathID != streamPath)
                {
                    if (s.pendMeta)
                    {
                        resolve_path<kFeather>(P, s, fx, fy, dither);
                        s.pendMeta = 0;
                    }
                    streamPath = vPathID;
                }
                const float4 v1 = T.v1, v2 = T.v2;
                const float E0 = local_edge(v0.y, v0.z, v0.w, lx, ly);
                const float E1 = local_edge(v1.x, v1.y, v1.z, lx, ly);
                const float E2 = local_edge(v1.w, v2.x, v2.y, lx, ly);
                const float emin = fminf(fminf(E0, E1), E2);
                if (!(emin > 0.f) &&
                    !(emin == 0.f && local_inside(v0.z, v0.w, E0) && local_inside(v1.y, v1.z, E1) &&
                      local_inside(v2.x, v2.y, E2)))
                    continue;
                if (!inBounds)
                    continue;
                const float4 v3 = T.v3;
                const float covx = __fmaf_rn(v2.w, lx, __fmaf_rn(v3.x, ly, v2.z));
                const float covy = __fmaf_rn(v3.z, lx, __fmaf_rn(v3.w, ly, v3.y));
                if (kFeather && ((T.v4.z >> 16) & FEATURE_IMAGE_MESH))
                {
                    // An image-mesh triangle blends at once, like a blit.
                    if (s.pendMeta)
                    {
                        resolve_path<kFeather>(P, s, fx, fy, dither);
                        s.pendMeta = 0;
                    }
                    const uint4 v4 = T.v4;
                    resolve_mesh(P, s, v4.z, v4.x, v4.y, B.featherPlanes + 2 * (size_t)v4.w, fx, fy,
                                 dither);
                    continue;
                }
                if (kFeather && ((T.v4.z >> 16) & FEATURE_ATLAS_BLIT))
                {
                    // A blit: the pending path is complete here; the blit
                    // writes its colour at once and leaves the coverage plane
                    // (key and count) to whichever path owns it.
                    if (s.pendMeta)
                    {
                        resolve_path<kFeather>(P, s, fx, fy, dither);
                        s.pendMeta = 0;
                    }
                    const uint4 v4 = T.v4;
                    resolve_blit(P, s, v4.z, v4.x, v4.y, covx, covy, fx, fy, dither);
                    continue;
                }
                float count;
                if (s.key != vPathID)
                {
                    if (s.pendMeta)
                        resolve_path<kFeather>(P, s, fx, fy, dither);
                    const uint4 v4 = T.v4;
                    s.pendMeta = v4.z;
                    s.pendPaintX = v4.x;
                    s.pendPaintY = v4.y;
                    s.pendFrags = 1;
                    s.key = vPathID;
                    count = 0.f;
                }
                else
                {
                    count = s.count;
                    s.pendFrags = 2;
                    if (!s.pendMeta) // the key's path came back after a resolve
                    {
                        const uint4 v4 = T.v4;
                        s.pendMeta = v4.z;
                        s.pendPaintX = v4.x;
                        s.pendPaintY = v4.y;
                    }
                }
                // Strokes (covy >= 0) keep the maximum coverage, fills add
                // (find_stroke_coverage / find_fill_coverage,
                // draw_path.vert:501-519); feathered ones are marked by a
                // coverage below the feather threshold.
                const bool stroke = covy >= 0.f;
                float frag = stroke ? fminf(covx, covy) : covx;
                // (s.pendMeta is this triangle's pathAndFeatures here.)
                if (kFeather && (stroke ? covx : covy) < kFeatherCoverageThreshold &&
                    ((s.pendMeta >> 16) & SF_FEATHER))
                    frag = feathered_fragment(B.featherPlanes, T.v4.w, fx, fy, covx, covy);
                count = stroke ? fmaxf(frag, count) : count + frag;
                s.count = h2f(f2h(count)); // the plane stores fp16
            }
        }
        __syncthreads();
    }
    if (s.pendMeta)
        resolve_path<kFeather>(P, s, fx, fy, dither);
    if (inBounds)
        fb[(size_t)py * P.width + px] = s.color;
}

// The raster kernels, each without and with the feather paths (the host
// launches the feather variant only for batches with ENABLE_FEATHER draws).
#define RIVE_RASTER_KERNELS(NAME, FEATHER)                                                        \
    __global__ void __launch_bounds__(256, RIVE_RASTER_MIN_BLOCKS) NAME(                           \
        BatchTables B, const TriRecord* __restrict__ tris,                                        \
        const uint32_t* __restrict__ sortedSlots, const uint2* __restrict__ ranges)               \
    {                                                                                             \
        __shared__ TileTri sTris[256 * RIVE_RASTER_STAGE];                                        \
        __shared__ uint8_t sMask[256 * RIVE_RASTER_STAGE];                                        \
        raster_tile<4, FEATHER, RIVE_RASTER_STAGE>(B, tris, sortedSlots, ranges, sTris, sMask,   \
                                                    blockIdx.x);                                  \
    }
RIVE_RASTER_KERNELS(raster_tile_kernel, false)
RIVE_RASTER_KERNELS(raster_tile_feather_kernel, true)
#undef RIVE_RASTER_KERNELS

// The work-queue form of the 16x16 raster: a persistent grid (as many CTAs
// as stay resident) in which each CTA takes its next tile from an atomic
// cursor over `order`, the batch's tiles sorted by bin entries, heaviest
// first, so the longest tiles start first and the last wave has no straggler
// behind it. The cursor starts at zero on every launch.
#define RIVE_RASTER_QUEUE_KERNELS(NAME, FEATHER)                                                  \
    __global__ void __launch_bounds__(256, RIVE_RASTER_MIN_BLOCKS) NAME(                           \
        BatchTables B, const TriRecord* __restrict__ tris,                                        \
        const uint32_t* __restrict__ sortedSlots, const uint2* __restrict__ ranges,               \
        const uint32_t* __restrict__ order, uint32_t* __restrict__ cursor, uint32_t tiles)        \
    {                                                                                             \
        __shared__ TileTri sTris[256];                                                            \
        __shared__ uint8_t sMask[256];                                                            \
        __shared__ uint32_t sNext;                                                                \
        for (;;)                                                                                  \
        {                                                                                         \
            __syncthreads(); /* the last tile is done with the shared state */                    \
            if (threadIdx.x == 0)                                                                 \
                sNext = atomicAdd(cursor, 1u);                                                    \
            __syncthreads();                                                                      \
            const uint32_t t = sNext;                                                             \
            if (t >= tiles)                                                                       \
                break;                                                                            \
            raster_tile<4, FEATHER, 1>(B, tris, sortedSlots, ranges, sTris, sMask, order[t]);     \
        }                                                                                         \
    }
RIVE_RASTER_QUEUE_KERNELS(raster_queue_kernel, false)
RIVE_RASTER_QUEUE_KERNELS(raster_queue_feather_kernel, true)
#undef RIVE_RASTER_QUEUE_KERNELS

// The feather atlas pass (render_atlas.glsl with the floating-point target
// and fixed-function blending; the atlas pipelines of gpu.hpp:2076-2080):
// one CTA of T x T threads per atlas tile, one thread per texel, walking the
// tile's bin entries in primitive order (fill batches, then stroke batches).
// A fill adds its feathered coverage, subtracted when the triangle faced
// away; a stroke keeps the maximum; every blend result rounds to fp16, as
// the R16F target stores it. Each texel is written, covered or not (the
// atlas starts cleared). Triangles arrive clipped to their batch's scissor
// through their pixel box, which the texel test applies exactly.
template <int TL>
__device__ __forceinline__ void raster_atlas_tile(const BatchTables& B,
                                                  const TriRecord* __restrict__ tris,
                                                  const uint32_t* __restrict__ sortedSlots,
                                                  const uint2* __restrict__ ranges,
                                                  uint32_t gtile)
{
    constexpr int T = 1 << TL;
    const uint32_t scene = find_range(B.tileBase, B.sceneCount, gtile);
    const FlushParams& P = B.scenes[scene];
    const uint32_t tilesX = P.tilesX;
    const uint32_t tile = gtile - B.tileBase[scene];
    const int tx = (int)(tile % tilesX), ty = (int)(tile / tilesX);
    const int ox = tx * T, oy = ty * T;
    const int lxi = (int)threadIdx.x & (T - 1), lyi = (int)threadIdx.x >> TL;
    const int px = ox + lxi, py = oy + lyi;
    const float lx = (float)lxi, ly = (float)lyi;
    const float fx = (float)px + .5f, fy = (float)py + .5f;
    const uint2 range = ranges[gtile];
    float acc = 0.f;
    for (uint32_t k = range.x; k < range.y; ++k)
    {
        const uint32_t slot = __ldg(sortedSlots + k);
        const TriRecord& R = tris[slot];
        const uint4 meta = R.meta;
        const int4 bb = unpack_bbox(meta);
        if (px < bb.x || px >= bb.z || py < bb.y || py >= bb.w)
            continue;
        const float4 e0 = R.e0, e1 = R.e1, e2 = R.e2;
        const float c0 = tile_edge_origin(e0, tx, ty, TL), c1 = tile_edge_origin(e1, tx, ty, TL),
                    c2 = tile_edge_origin(e2, tx, ty, TL);
        const float E0 = local_edge(c0, e0.z, e0.w, lx, ly);
        const float E1 = local_edge(c1, e1.z, e1.w, lx, ly);
        const float E2 = local_edge(c2, e2.z, e2.w, lx, ly);
        const float emin = fminf(fminf(E0, E1), E2);
        if (!(emin > 0.f) &&
            !(emin == 0.f && local_inside(e0.z, e0.w, E0) && local_inside(e1.z, e1.w, E1) &&
              local_inside(e2.z, e2.w, E2)))
            continue;
        const float4 cv0 = R.cov0, cv1 = R.cov1;
        const float dx0 = (float)ox + .5f - e0.x, dy0 = (float)oy + .5f - e0.y;
        const float cx0 = cv0.x + cv0.y * dx0 + cv0.z * dy0;
        const float cy0 = cv0.w + cv1.x * dx0 + cv1.y * dy0;
        const float covx = __fmaf_rn(cv0.y, lx, __fmaf_rn(cv0.z, ly, cx0));
        const float covy = __fmaf_rn(cv1.x, lx, __fmaf_rn(cv1.y, ly, cy0));
        float frag = feathered_fragment(B.featherPlanes, slot, fx, fy, covx, covy);
        if (covy >= 0.f)
        {
            acc = h2f(f2h(fmaxf(acc, frag)));
        }
        else
        {
            if ((meta.x >> 16) & FEATURE_ATLAS_NEGATE)
                frag = -frag;
            acc = h2f(f2h(acc + frag));
        }
    }
    if (px < (int)P.width && py < (int)P.height)
        P.atlas[(size_t)py * P.atlasW + px] = (uint16_t)f2h(acc);
}

#define RIVE_ATLAS_KERNEL(NAME, TL)                                                                \
    __global__ void __launch_bounds__(1 << (2 * TL)) NAME(                                          \
        BatchTables B, const TriRecord* __restrict__ tris,                                        \
        const uint32_t* __restrict__ sortedSlots, const uint2* __restrict__ ranges,               \
        uint32_t firstTile)                                                                       \
    {                                                                                             \
        raster_atlas_tile<TL>(B, tris, sortedSlots, ranges, firstTile + blockIdx.x);              \
    }
RIVE_ATLAS_KERNEL(raster_atlas8_kernel, 3)
RIVE_ATLAS_KERNEL(raster_atlas_kernel, 4)
RIVE_ATLAS_KERNEL(raster_atlas32_kernel, 5)
#undef RIVE_ATLAS_KERNEL

// Sort keys of the work queue: per tile, its bin entries inverted (a plain
// ascending sort then puts the heaviest tile first), and its index.
__global__ void __launch_bounds__(256) tile_order_keys_kernel(uint32_t tiles,
                                                              const uint2* __restrict__ ranges,
                                                              uint32_t* __restrict__ keys,
                                                              uint32_t* __restrict__ vals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tiles)
        return;
    const uint2 r = ranges[i];
    keys[i] = 0xffffffffu - (r.y > r.x ? r.y - r.x : 0u);
    vals[i] = i;
}

#define RIVE_RASTER8_KERNELS(NAME, FEATHER)                                                       \
    __global__ void __launch_bounds__(64) NAME(BatchTables B, const TriRecord* __restrict__ tris, \
                                               const uint32_t* __restrict__ sortedSlots,         \
                                               const uint2* __restrict__ ranges)                 \
    {                                                                                             \
        __shared__ TileTri sTris[64 * RIVE_RASTER_STAGE];                                         \
        __shared__ uint8_t sMask[64 * RIVE_RASTER_STAGE];                                         \
        raster_tile<3, FEATHER, RIVE_RASTER_STAGE>(B, tris, sortedSlots, ranges, sTris, sMask,   \
                                                    blockIdx.x);                                  \
    }
RIVE_RASTER8_KERNELS(raster_tile8_kernel, false)
RIVE_RASTER8_KERNELS(raster_tile8_feather_kernel, true)
#undef RIVE_RASTER8_KERNELS

// 32x32 tiles: 1,024 threads, the staged records in dynamic shared memory
// (kRaster32SmemBytes).
#define RIVE_RASTER32_KERNELS(NAME, FEATHER)                                                      \
    __global__ void __launch_bounds__(1024, 1) NAME(                                              \
        BatchTables B, const TriRecord* __restrict__ tris,                                        \
        const uint32_t* __restrict__ sortedSlots, const uint2* __restrict__ ranges)               \
    {                                                                                             \
        extern __shared__ uint4 dyn[];                                                            \
        TileTri* sTris = reinterpret_cast<TileTri*>(dyn);                                         \
        uint32_t* sMask = reinterpret_cast<uint32_t*>(sTris + 1024);                              \
        raster_tile<5, FEATHER, 1>(B, tris, sortedSlots, ranges, sTris, sMask, blockIdx.x);       \
    }
RIVE_RASTER32_KERNELS(raster_tile32_kernel, false)
RIVE_RASTER32_KERNELS(raster_tile32_feather_kernel, true)
#undef RIVE_RASTER32_KERNELS
} // namespace rivecuda

namespace rivecuda
{
namespace
{
// Generator of the feather table (renderer/src/gpu.cpp:1983-2062, restated):
// 7 samples per entry of the normal distribution, shifted so the middle entry
// pair averages 1/2, made monotonic and clamped to [0, 1], eased to 0 and 1
// over the 8 entries at each end, then rounded to fp16 as the R16F texture
// holds it.
float eval_normal_distribution(float x, float mu, float inverseSigma)
{
    const float kOneOverSqrt2Pi = 0.398942280401433f;
    float y = (x - mu) * inverseSigma;
    return expf(-.5 * y * y) * inverseSigma * kOneOverSqrt2Pi;
}

void build_feather_table(float out[kGaussianTableSize])
{
    float table[kGaussianTableSize];
    const float sigma = kGaussianTableSize / (kGaussianStddevs * 2);
    const float inverseSigma = 1 / sigma;
    const float mu = kGaussianTableSize * .5f;
    float integral = 0;
    for (int i = 0; i < kGaussianTableSize; ++i)
    {
        const int kSamples = 7;
        for (int sample = 0; sample < kSamples; ++sample)
        {
            float dx = (float)(sample - (kSamples >> 1)) / kSamples;
            integral += eval_normal_distribution((float)i + dx, mu, inverseSigma) / kSamples;
        }
        table[i] = integral;
    }
    const float shift =
        .5 - (table[kGaussianTableSize / 2 - 1] + table[kGaussianTableSize / 2]) / 2;
    table[0] = fminf(fmaxf(0, table[0] + shift), 1);
    for (int i = 1; i < kGaussianTableSize; ++i)
        table[i] = fminf(fmaxf(table[i - 1], table[i] + shift), 1);
    const int kEase = 8;
    for (int i = 0; i < kGaussianTableSize; ++i)
    {
        if (i < kEase)
            table[i] *= (float)i / (float)kEase;
        if (i > (kGaussianTableSize - kEase) - 1)
        {
            float diffToOne = 1.0 - table[i];
            float fi = (float)(i - (kGaussianTableSize - kEase) + 1) / (float)kEase;
            table[i] = table[i] + (diffToOne * fi);
        }
    }
    for (int i = 0; i < kGaussianTableSize; ++i)
        out[i] = __half2float(__float2half_rn(table[i]));
}
} // namespace

// Generator of the inverse feather table (renderer/src/gpu.cpp:2125-2190,
// restated): the running integral of the normal distribution sampled 32 times
// per entry; every cell whose centre the integral crosses gets the sample
// height interpolated at the crossing, the middle cell exactly 1/2, the end
// cells 0 and 1; then rounded to fp16.
void build_inverse_feather_table(float out[kGaussianTableSize])
{
    constexpr int kPerEntry = 32;
    constexpr int kSamples = kGaussianTableSize * kPerEntry;
    float table[kGaussianTableSize] = {};
    const float inverseSigma = 1 / (float)(kGaussianTableSize / (kGaussianStddevs * 2));
    const float mu = kGaussianTableSize * .5f;
    // Start the integral at -1/2 minus the left half, so it reaches 1/2 at mu.
    float integral = 0;
    for (int i = 0; i < (kSamples + 1) / 2; ++i)
        integral += eval_normal_distribution((float)i / kPerEntry, mu, inverseSigma) / kPerEntry;
    integral = .5 - integral;
    table[0] = 0;
    table[kGaussianTableSize - 1] = 1;
    float prevX = NAN, prevY = 0;
    for (int i = 0; i < kSamples; ++i)
    {
        integral += eval_normal_distribution((float)i / kPerEntry, mu, inverseSigma) / kPerEntry;
        const float x = fminf(fmaxf(0, integral), 1) * kGaussianTableSize;
        const float y = (i + .5f) / kSamples;
        const size_t cell = (size_t)x;
        const float centre = cell + .5f;
        if (centre == mu)
            table[cell] = .5f;
        else if (prevX <= centre && x >= centre && cell < kGaussianTableSize)
            table[cell] = prevY + (y - prevY) * ((centre - prevX) / (x - prevX));
        prevX = x;
        prevY = y;
    }
    for (int i = 0; i < kGaussianTableSize; ++i)
        out[i] = __half2float(__float2half_rn(table[i]));
}

// Uploads the feather tables to the current device (once per device).
cudaError_t ensure_feather_lut(int device)
{
    static std::mutex m;
    static bool done[64] = {};
    std::lock_guard<std::mutex> lock(m);
    if (device >= 0 && device < 64 && done[device])
        return cudaSuccess;
    float table[kGaussianTableSize];
    build_feather_table(table);
    cudaError_t e = cudaMemcpyToSymbol(g_featherLUT, table, sizeof(table));
    if (e == cudaSuccess)
    {
        build_inverse_feather_table(table);
        e = upload_inverse_feather_lut(table);
    }
    if (e == cudaSuccess && device >= 0 && device < 64)
        done[device] = true;
    return e;
}

// The fp16 bits of the feather table, for the C ABI.
void feather_table_f16(uint16_t out[kGaussianTableSize])
{
    float table[kGaussianTableSize];
    build_feather_table(table);
    for (int i = 0; i < kGaussianTableSize; ++i)
        out[i] = __half_as_ushort(__float2half_rn(table[i]));
}

// One mip level of an image from the level above it: each texel the rounded
// mean of the (up to) 2x2 texels it covers, edges clamped.
__global__ void __launch_bounds__(256) mip_level_kernel(const uchar4* __restrict__ src,
                                                        uint32_t sw, uint32_t sh,
                                                        uchar4* __restrict__ dst, uint32_t dw,
                                                        uint32_t dh)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dw * dh)
        return;
    const uint32_t x = i % dw, y = i / dw;
    const uint32_t x0 = min(2 * x, sw - 1), x1 = min(2 * x + 1, sw - 1);
    const uint32_t y0 = min(2 * y, sh - 1), y1 = min(2 * y + 1, sh - 1);
    const uchar4 a = src[(size_t)y0 * sw + x0], b = src[(size_t)y0 * sw + x1];
    const uchar4 c = src[(size_t)y1 * sw + x0], d = src[(size_t)y1 * sw + x1];
    dst[i] = make_uchar4((unsigned char)((a.x + b.x + c.x + d.x + 2u) >> 2),
                         (unsigned char)((a.y + b.y + c.y + d.y + 2u) >> 2),
                         (unsigned char)((a.z + b.z + c.z + d.z + 2u) >> 2),
                         (unsigned char)((a.w + b.w + c.w + d.w + 2u) >> 2));
}
} // namespace rivecuda
