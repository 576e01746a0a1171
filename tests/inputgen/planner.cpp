// TEST AND BENCH INFRASTRUCTURE -- not part of the product. A stand-in for
// rive-runtime's own CPU front end (RiveRenderer -> RenderContext), used to
// produce flush records from rive_scene.h recordings on machines where the
// reference sources cannot be built (the GPU machines the benchmark and the
// GPU tests run on). In a deployment the reference's front end produces the
// records and hands them to RenderContextCUDAImpl; where the reference is
// compiled (oracle/_ref), the goldens come from it and this stand-in is tested
// byte for byte against it (tests/test_planner.py, tests/test_sriv.py).
//
// It follows the reference's algorithms (Wang's formula, chops, polar counts,
// span layout, gradient allocation, logical-flush limits) step by step,
// because its output must be byte-identical to the reference's: for
// rasterOrdering with midpoint-fan tessellation. Floating-point expressions
// keep the reference's operation order so results are bit-identical when both
// are built without FMA contraction (-ffp-contract=off).
#include "rive_cuda.h"
#include "rive_planner.h" // this directory
#include "rive_scene.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace
{
// ---------------------------------------------------------------------------
// Constants (renderer/include/rive/renderer/gpu.hpp, shaders/constants.glsl).
constexpr int kParametricPrecision = 4;
constexpr int kPolarPrecision = 8;
constexpr uint32_t kMaxParametricSegments = 1023;
constexpr uint32_t kMaxPolarSegments = 1023;
constexpr uint32_t kTessTextureWidth = 2048;
constexpr uint32_t kGradTextureWidth = 512;
constexpr uint32_t kGradTextureWidthInSimpleRamps = kGradTextureWidth / 2;
constexpr uint32_t kMidpointFanPatchSegmentSpan = 8;
constexpr uint32_t kOuterCubicPatchSegmentSpanPlusJoin = 17;
constexpr uint32_t kMaxTextureHeight = 2048;
constexpr size_t kMaxTessellationVertexCount = kMaxTextureHeight * kTessTextureWidth;
constexpr size_t kMaxTessellationPaddingVertexCount = 8 + 16 + 1;
constexpr size_t kMaxTessellationVertexCountBeforePadding =
    kMaxTessellationVertexCount - kMaxTessellationPaddingVertexCount;
constexpr size_t kMaxContourID = 65535;
constexpr uint32_t kMaxPathID = (((0x1f << 10) - 1) / 1) - 1023; // granularity 1
constexpr int NUM_SEGMENTS_IN_MITER_OR_BEVEL_JOIN = 5;
constexpr float kPI = 3.14159265f;
constexpr float kSQRT2 = 1.41421356f;
constexpr float kEPSILON = 1.f / (1 << 12);
constexpr float kRiveMiterLimit = 4.f;

constexpr uint32_t GRAD_SPAN_FLAG_LEFT_BORDER = 0x80000000u;
constexpr uint32_t GRAD_SPAN_FLAG_RIGHT_BORDER = 0x40000000u;
constexpr uint32_t GRAD_SPAN_FLAG_COMPLEX_BORDER = 0x20000000u;
constexpr uint32_t MITER_CLIP_JOIN_CONTOUR_FLAG = 5u << 26;
constexpr uint32_t MITER_REVERT_JOIN_CONTOUR_FLAG = 4u << 26;
constexpr uint32_t BEVEL_JOIN_CONTOUR_FLAG = 3u << 26;
constexpr uint32_t ROUND_JOIN_CONTOUR_FLAG = 2u << 26;
constexpr uint32_t EMULATED_STROKE_CAP_CONTOUR_FLAG = 1u << 25;
constexpr uint32_t PAINT_FLAG_NON_ZERO_FILL = 0x100u;
constexpr uint32_t PAINT_FLAG_EVEN_ODD_FILL = 0x200u;

// gpu::DrawContents
constexpr uint32_t DC_OPAQUE = 1u << 0, DC_STROKE = 1u << 2, DC_CLOCKWISE = 1u << 3,
                   DC_NONZERO = 1u << 4, DC_EVENODD = 1u << 5, DC_ACTIVE_CLIP = 1u << 6,
                   DC_ADVANCED_BLEND = 1u << 7, DC_CLIP_UPDATE = 1u << 8;
constexpr uint32_t DC_ANY_FILL = DC_CLOCKWISE | DC_NONZERO | DC_EVENODD;
// gpu::ShaderFeatures
constexpr uint32_t SF_CLIPPING = 1u << 0, SF_CLIP_RECT = 1u << 1, SF_ADVANCED_BLEND = 1u << 2,
                   SF_EVEN_ODD = 1u << 4, SF_NESTED_CLIPPING = 1u << 5, SF_HSL = 1u << 6,
                   SF_DITHER = 1u << 7;
// gpu::ShaderMiscFlags::clockwiseFill
constexpr uint32_t MISC_CLOCKWISE_FILL = 1u << 1;
constexpr uint32_t PAINT_FLAG_HAS_CLIP_RECT = 0x400u;
constexpr uint32_t NEGATE_PATH_FILL_COVERAGE_FLAG = 1u << 24;
constexpr uint32_t FILL_RULE_CLOCKWISE = 2; // rive::FillRule::clockwise

enum PaintType : uint32_t
{
    PT_CLIP_UPDATE = 0,
    PT_SOLID = 1,
    PT_LINEAR = 2,
    PT_RADIAL = 3
};
enum Verb : uint8_t
{
    V_MOVE = 0,
    V_LINE = 1,
    V_QUAD = 2,
    V_CUBIC = 4,
    V_CLOSE = 5
};
enum Join : uint32_t
{
    J_MITER = 0,
    J_ROUND = 1,
    J_BEVEL = 2
};
enum Cap : uint32_t
{
    C_BUTT = 0,
    C_ROUND = 1,
    C_SQUARE = 2
};
enum ContourDirections
{
    CD_FORWARD,
    CD_REVERSE_THEN_FORWARD,
    CD_FORWARD_THEN_REVERSE
};

struct PlanError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// rive::simd min/max/clamp semantics (include/rive/math/simd.hpp:208-253):
// a NaN operand is ignored in favour of the other, and clamp(NaN) == lo.
inline float simd_min(float a, float b) { return (b < a || std::isnan(a)) ? b : a; }
inline float simd_max(float a, float b) { return (a < b || std::isnan(a)) ? b : a; }
inline float simd_clamp(float x, float lo, float hi) { return simd_min(simd_max(lo, x), hi); }

// ---------------------------------------------------------------------------
// Geometry.
struct V2
{
    float x = 0, y = 0;
};
inline V2 operator+(V2 a, V2 b) { return {a.x + b.x, a.y + b.y}; }
inline V2 operator-(V2 a, V2 b) { return {a.x - b.x, a.y - b.y}; }
inline V2 operator-(V2 a) { return {-a.x, -a.y}; }
inline V2 operator*(V2 a, float s) { return {a.x * s, a.y * s}; }
inline bool operator==(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }
inline bool operator!=(V2 a, V2 b) { return !(a == b); }
inline bool bits_equal(V2 a, V2 b) { return memcmp(&a, &b, sizeof(V2)) == 0; }
inline V2 mix(V2 a, V2 b, float t) { return (b - a) * t + a; } // simd::mix

struct IBox
{
    int32_t l, t, r, b;
    bool empty() const { return l >= r || t >= b; }
    IBox intersect(IBox o) const
    {
        return {std::max(l, o.l), std::max(t, o.t), std::min(r, o.r), std::min(b, o.b)};
    }
    IBox join(IBox o) const
    {
        return {std::min(l, o.l), std::min(t, o.t), std::max(r, o.r), std::max(b, o.b)};
    }
    static IBox maximal()
    {
        return {std::numeric_limits<int32_t>::min(), std::numeric_limits<int32_t>::min(),
                std::numeric_limits<int32_t>::max(), std::numeric_limits<int32_t>::max()};
    }
    static IBox maximallyNegative()
    {
        return {std::numeric_limits<int32_t>::max(), std::numeric_limits<int32_t>::max(),
                std::numeric_limits<int32_t>::min(), std::numeric_limits<int32_t>::min()};
    }
};

struct FBox
{
    float l, t, r, b;
    IBox roundOut() const
    {
        return {(int32_t)floorf(l), (int32_t)floorf(t), (int32_t)ceilf(r), (int32_t)ceilf(b)};
    }
    float width() const { return r - l; }
    float height() const { return b - t; }
    FBox outset(float dx, float dy) const { return {l - dx, t - dy, r + dx, b + dy}; }
};

// rive::Mat2D: [xx, xy, yx, yy, tx, ty].
struct M2
{
    float v[6] = {1, 0, 0, 1, 0, 0};
    // operator== (include/rive/math/mat2d.hpp): element-wise float equality.
    bool operator==(const M2& o) const
    {
        for (int i = 0; i < 6; ++i)
            if (!(v[i] == o.v[i]))
                return false;
        return true;
    }
    // Mat2D::multiply (src/math/mat2d.cpp:45-57)
    M2 operator*(const M2& b) const
    {
        const float* a = v;
        M2 r;
        r.v[0] = a[0] * b.v[0] + a[2] * b.v[1];
        r.v[1] = a[1] * b.v[0] + a[3] * b.v[1];
        r.v[2] = a[0] * b.v[2] + a[2] * b.v[3];
        r.v[3] = a[1] * b.v[2] + a[3] * b.v[3];
        r.v[4] = a[0] * b.v[4] + a[2] * b.v[5] + a[4];
        r.v[5] = a[1] * b.v[4] + a[3] * b.v[5] + a[5];
        return r;
    }
    // Mat2D::invert (src/math/mat2d.cpp:179-200)
    bool invert(M2* out) const
    {
        float aa = v[0], ab = v[1], ac = v[2], ad = v[3], atx = v[4], aty = v[5];
        float det = aa * ad - ab * ac;
        if (det == 0.0f)
            return false;
        det = 1.0f / det;
        out->v[0] = ad * det;
        out->v[1] = -ab * det;
        out->v[2] = -ac * det;
        out->v[3] = aa * det;
        out->v[4] = (ac * aty - ad * atx) * det;
        out->v[5] = (ab * atx - aa * aty) * det;
        return true;
    }
    // Mat2D::findMaxScale (src/math/mat2d_find_max_scale.cpp)
    float findMaxScale() const
    {
        float xx = v[0], xy = v[1], yx = v[2], yy = v[3];
        if (xy == 0 && yx == 0)
            return std::max(fabsf(xx), fabsf(yy));
        float a = xx * xx + xy * xy;
        float b = xx * yx + yy * xy;
        float c = yx * yx + yy * yy;
        float bSqd = b * b;
        float result;
        if (bSqd <= kEPSILON * kEPSILON)
        {
            result = std::max(a, c);
        }
        else
        {
            float aminusc = a - c;
            float apluscdiv2 = (a + c) * .5f;
            float x = sqrtf(aminusc * aminusc + 4 * bSqd) * .5f;
            result = apluscdiv2 + x;
        }
        if (!std::isfinite(result))
            result = 0;
        result = std::max(result, 0.f);
        return sqrtf(result);
    }
    // Mat2D::mapBoundingBox (src/math/mat2d.cpp:103-168)
    FBox mapBoundingBox(const V2* pts, size_t n) const
    {
        float inf = std::numeric_limits<float>::infinity();
        float mnx = inf, mny = inf, mxx = -inf, mxy = -inf;
        bool scaleOnly = v[1] == 0.f && v[2] == 0.f;
        for (size_t i = 0; i < n; ++i)
        {
            float px, py;
            if (scaleOnly)
            {
                px = v[0] * pts[i].x;
                py = v[3] * pts[i].y;
            }
            else
            {
                float sx = v[2] * pts[i].y, sy = v[1] * pts[i].x;
                px = v[0] * pts[i].x + sx;
                py = v[3] * pts[i].y + sy;
            }
            mnx = simd_min(px, mnx);
            mny = simd_min(py, mny);
            mxx = simd_max(px, mxx);
            mxy = simd_max(py, mxy);
        }
        FBox b{mnx, mny, mxx, mxy};
        if (!(b.r - b.l >= 0 && b.b - b.t >= 0))
            return {0, 0, 0, 0};
        b.l += v[4];
        b.t += v[5];
        b.r += v[4];
        b.b += v[5];
        return b;
    }
    FBox mapBoundingBox(FBox box) const
    {
        V2 p[4] = {{box.l, box.t}, {box.r, box.t}, {box.r, box.b}, {box.l, box.b}};
        return mapBoundingBox(p, 4);
    }
};

// wangs_formula::cubic_pow4 with a VectorXform (wangs_formula.hpp).
float cubic_pow4(const V2 p[4], const M2& m)
{
    const float* mv = m.v;
    float vx[2], vy[2];
    for (int k = 0; k < 2; ++k)
    {
        // -2 * p[k+1] + p[k] + p[k+2]
        float x = -2.f * p[k + 1].x + p[k].x + p[k + 2].x;
        float y = -2.f * p[k + 1].y + p[k].y + p[k + 2].y;
        // m_scale * v + m_skew * v.yx
        vx[k] = mv[0] * x + mv[2] * y;
        vy[k] = mv[3] * y + mv[1] * x;
    }
    constexpr float lengthTermPow2 =
        ((3 * 3) * ((3 - 1) * (3 - 1)) / 64.f) * (kParametricPrecision * kParametricPrecision);
    return std::max(vx[0] * vx[0] + vy[0] * vy[0], vx[1] * vx[1] + vy[1] * vy[1]) *
           lengthTermPow2;
}

// bezier_utils.hpp:109-113
float calc_polar_segments_per_radian(float r)
{
    float cosTheta = 1.f - (1.f / kPolarPrecision) / r;
    return .5f / acosf(std::max(cosTheta, -1.f));
}

// simd::fast_acos (simd.hpp:496-507)
float fast_acos(float x)
{
    const float a = -0.939115566365855f, b = 0.9217841528914573f;
    const float c = -1.2845906244690837f, d = 0.295624144969963174f;
    const float pi_over_2 = 1.5707963267948966f;
    float xx = x * x;
    float numer = b * xx + a;
    float denom = xx * (d * xx + c) + 1.f;
    return x * (numer / denom) + pi_over_2;
}

V2 find_cubic_tan0(const V2 p[4])
{
    return (p[0] != p[1] ? p[1] : p[1] != p[2] ? p[2] : p[3]) - p[0];
}
V2 find_cubic_tan1(const V2 p[4])
{
    return p[3] - (p[3] != p[2] ? p[2] : p[2] != p[1] ? p[1] : p[0]);
}

// bezier_utils.cpp:21-32
V2 eval_cubic_at(const V2 p[4], float t)
{
    V2 a = p[3] + (p[1] - p[2]) * 3.f - p[0];
    V2 b = (p[2] - p[1] * 2.f + p[0]) * 3.f;
    V2 c = (p[1] - p[0]) * 3.f;
    V2 d = p[0];
    return ((a * t + b) * t + c) * t + d;
}

// bezier_utils.cpp:34-62 (3 * 2 + 1 points)
void chop_cubic_at(const V2 srcIn[4], V2 dst[7], float t)
{
    // dst may alias src (chained chops): read every control point first.
    const V2 src[4] = {srcIn[0], srcIn[1], srcIn[2], srcIn[3]};
    if (t == 1)
    {
        memcpy(dst, src, sizeof(V2) * 4);
        dst[4] = dst[5] = dst[6] = src[3];
        return;
    }
    V2 ab = mix(src[0], src[1], t), bc = mix(src[1], src[2], t), cd = mix(src[2], src[3], t);
    V2 abc = mix(ab, bc, t), bcd = mix(bc, cd, t);
    V2 abcd = mix(abc, bcd, t);
    dst[0] = src[0];
    dst[1] = ab;
    dst[2] = abc;
    dst[3] = abcd;
    dst[4] = bcd;
    dst[5] = cd;
    dst[6] = src[3];
}

// bezier_utils.cpp:64-102 (two chops at once)
void chop_cubic_at(const V2 srcIn[4], V2 dst[10], float t0, float t1)
{
    const V2 src[4] = {srcIn[0], srcIn[1], srcIn[2], srcIn[3]};
    if (t1 == 1)
    {
        chop_cubic_at(src, dst, t0);
        dst[7] = dst[8] = dst[9] = src[3];
        return;
    }
    const float T[2] = {t0, t1};
    V2 ab[2], bc[2], cd[2], abc[2], bcd[2], abcd[2], middle[2];
    for (int k = 0; k < 2; ++k)
    {
        ab[k] = mix(src[0], src[1], T[k]);
        bc[k] = mix(src[1], src[2], T[k]);
        cd[k] = mix(src[2], src[3], T[k]);
        abc[k] = mix(ab[k], bc[k], T[k]);
        bcd[k] = mix(bc[k], cd[k], T[k]);
        abcd[k] = mix(abc[k], bcd[k], T[k]);
    }
    // middle = mix(abc, bcd, T.zwxy): lane 0 uses t1, lane 1 uses t0.
    middle[0] = mix(abc[0], bcd[0], T[1]);
    middle[1] = mix(abc[1], bcd[1], T[0]);
    dst[0] = src[0];
    dst[1] = ab[0];
    dst[2] = abc[0];
    dst[3] = abcd[0];
    dst[4] = middle[0];
    dst[5] = middle[1];
    dst[6] = abcd[1];
    dst[7] = bcd[1];
    dst[8] = cd[1];
    dst[9] = src[3];
}

float clamp01(float x) { return simd_clamp(x, 0.f, 1.f); }

// bezier_utils.cpp:104-157 (tValues != nullptr)
void chop_cubic_at(const V2 src[4], V2* dst, const float* tValues, int tCount)
{
    if (tCount == 0)
    {
        memcpy(dst, src, 4 * sizeof(V2));
        return;
    }
    int i = 0;
    float lastT = 0;
    for (; i < tCount - 1; i += 2)
    {
        float tt0 = clamp01((tValues[i] - lastT) / (1 - lastT));
        float tt1 = clamp01((tValues[i + 1] - lastT) / (1 - lastT));
        lastT = tValues[i + 1];
        chop_cubic_at(src, dst, tt0, tt1);
        src = dst = dst + 6;
    }
    if (i < tCount)
    {
        float t = clamp01((tValues[i] - lastT) / (1 - lastT));
        chop_cubic_at(src, dst, t);
    }
}

// bezier_utils.cpp:180-331
int find_cubic_convex_180_chops(const V2 pts[4], float T[2], bool* areCusps)
{
    constexpr float TESS_EPSILON = 1.f / (1 << 10);
    constexpr uint32_t kIEEE_one_minus_2_epsilon = (127 << 23) - 2 * (1 << (24 - 10));
    auto bits = [](float f) {
        uint32_t u;
        memcpy(&u, &f, 4);
        return u;
    };
    V2 p0 = pts[0], p1 = pts[1], p2 = pts[2], p3 = pts[3];
    // CubicCoeffs
    V2 C = p1 - p0;
    V2 D = p2 - p1;
    V2 E = p3 - p0;
    V2 B = D - C;
    V2 A = D * -3.f + E;
    auto cross = [](V2 a, V2 b) { return a.x * b.y - a.y * b.x; };
    float a = cross(A, B);
    float b = cross(A, C);
    float c = cross(B, C);
    float b_over_minus_2 = -.5f * b;
    float discr_over_4 = b_over_minus_2 * b_over_minus_2 - a * c;
    float cuspThreshold = a * (TESS_EPSILON / 2);
    cuspThreshold *= cuspThreshold;
    if (discr_over_4 < -cuspThreshold)
    {
        *areCusps = false;
        float root = c / b_over_minus_2;
        if (bits(root - TESS_EPSILON) < kIEEE_one_minus_2_epsilon)
        {
            T[0] = root;
            return 1;
        }
        return 0;
    }
    *areCusps = discr_over_4 <= cuspThreshold;
    if (*areCusps)
    {
        if (a != 0 || b_over_minus_2 != 0 || c != 0)
        {
            float root = b_over_minus_2 / a;
            if (bits(root - TESS_EPSILON) < kIEEE_one_minus_2_epsilon)
            {
                T[0] = root;
                return 1;
            }
            *areCusps = false;
            return 0;
        }
        V2 base = p3 - p0;
        float dp[4];
        for (int k = 0; k < 4; ++k)
            dp[k] = pts[k].x * base.x + pts[k].y * base.y;
        if (dp[1] > dp[0] && dp[2] > dp[1] && dp[3] > dp[2])
        {
            *areCusps = false;
            return 0;
        }
        V2 tan0 = (C.x != 0.f || C.y != 0.f) ? C : p2 - p0;
        a = tan0.x * A.x + tan0.y * A.y;
        b_over_minus_2 = -(tan0.x * B.x + tan0.y * B.y);
        c = tan0.x * C.x + tan0.y * C.y;
        discr_over_4 = std::max(b_over_minus_2 * b_over_minus_2 - a * c, 0.f);
    }
    float q = sqrtf(discr_over_4);
    q = copysignf(q, b_over_minus_2);
    q = q + b_over_minus_2;
    float roots[2] = {q / a, c / q};
    bool in0 = (roots[0] > TESS_EPSILON) && (roots[0] < (1 - TESS_EPSILON));
    bool in1 = (roots[1] > TESS_EPSILON) && (roots[1] < (1 - TESS_EPSILON));
    if (in0)
    {
        if (in1 && roots[0] != roots[1])
        {
            if (roots[0] > roots[1])
                std::swap(roots[0], roots[1]);
            T[0] = roots[0];
            T[1] = roots[1];
            return 2;
        }
        T[0] = roots[0];
        return 1;
    }
    if (in1)
    {
        T[0] = roots[1];
        return 1;
    }
    return 0;
}

// draw.cpp:139-174
void chop_cubic_around_cusps(const V2 p[4], V2 dst[], const float cuspT[], int n,
                             float matrixMaxScale)
{
    float t[4];
    for (int i = 0; i < n; ++i)
    {
        float minT = i == 0 ? 0.f : (cuspT[i - 1] + cuspT[i]) * .5f;
        float maxT = i + 1 == n ? 1.f : (cuspT[i + 1] + cuspT[i]) * .5f;
        t[i * 2 + 0] = fmaxf(cuspT[i] - kEPSILON, minT);
        t[i * 2 + 1] = fminf(cuspT[i] + kEPSILON, maxT);
    }
    chop_cubic_at(p, dst, t, n * 2);
    for (int i = 0; i < n; ++i)
    {
        V2* chops = dst + i * 6;
        V2 cusp = eval_cubic_at(p, cuspT[i]);
        chops[3] = chops[6] = cusp;
        V2 pivot = (chops[2] + chops[7]) * .5f;
        V2 d = cusp - pivot;
        // Vec2D::normalized(): v * (1 / length)
        float len = sqrtf(d.x * d.x + d.y * d.y);
        V2 nrm = len > 0 ? d * (1.f / len) : V2{0, 0};
        float s = matrixMaxScale * kPolarPrecision * 2;
        pivot = V2{nrm.x / s, nrm.y / s} + cusp;
        chops[4] = chops[5] = pivot;
    }
}

// draw.cpp:113-131 (convert_line_to_cubic)
void line_to_cubic(V2 p0, V2 p1, V2 out[4])
{
    // simd::mix(endPts, endPts.zwxy, 1/3)
    float t = 1 / 3.f;
    out[0] = p0;
    out[1] = mix(p0, p1, t);
    out[2] = mix(p1, p0, t);
    out[3] = p1;
}

// ---------------------------------------------------------------------------
// Scene objects.
struct Path
{
    std::vector<uint8_t> verbs;
    std::vector<V2> pts;
    uint32_t fillRule = 0; // 0 nonZero, 1 evenOdd
    uint32_t id = 0;       // stands in for the raw path mutation ID
    size_t countMoves() const
    {
        return (size_t)std::count(verbs.begin(), verbs.end(), (uint8_t)V_MOVE);
    }
};

// RawPath::pruneEmptySegments (src/math/raw_path.cpp:353-413).
void prune_empty_segments(Path& path)
{
    std::vector<uint8_t> vo;
    std::vector<V2> po;
    size_t pi = 0;
    for (uint8_t verb : path.verbs)
    {
        int adv = verb == V_CUBIC ? 3 : verb == V_QUAD ? 2 : verb == V_CLOSE ? 0 : 1;
        const V2* s = path.pts.data() + pi;
        bool keep = true;
        if (verb == V_CUBIC || verb == V_QUAD || verb == V_LINE)
        {
            bool empty = true;
            if (verb == V_CUBIC && s[2] != s[1])
                empty = false;
            else if ((verb == V_CUBIC || verb == V_QUAD) && s[1] != s[0])
                empty = false;
            else if (s[0] != (po.empty() ? s[-1] : po.back()))
                empty = false;
            keep = !empty;
        }
        if (keep)
        {
            vo.push_back(verb);
            po.insert(po.end(), s, s + adv);
        }
        pi += (size_t)adv;
    }
    path.verbs.swap(vo);
    path.pts.swap(po);
}

struct Gradient
{
    PaintType type;
    std::vector<uint32_t> colors;
    std::vector<float> stops;
    float coeffs[3];
    bool isOpaque() const
    {
        uint32_t all = ~0u;
        for (uint32_t c : colors)
            all &= c;
        return (all >> 24) == 0xff;
    }
};

bool validate_stops(const std::vector<float>& stops)
{
    if (stops.empty())
        return false;
    for (float s : stops)
        if (!(0 <= s && s <= 1))
            return false;
    for (size_t i = 1; i < stops.size(); ++i)
        if (!(stops[i - 1] <= stops[i]))
            return false;
    return true;
}

// Gradient::MakeLinear / MakeRadial (renderer/src/gradient.cpp).
std::shared_ptr<Gradient> make_gradient(const rive_scene_paint& sp, const rive_scene_stop* stopRecs)
{
    auto g = std::make_shared<Gradient>();
    size_t count = sp.stop_count;
    std::vector<float> stops(count);
    g->colors.resize(count);
    for (size_t i = 0; i < count; ++i)
    {
        stops[i] = stopRecs[sp.stop_offset + i].position;
        g->colors[i] = stopRecs[sp.stop_offset + i].color;
    }
    if (!validate_stops(stops))
        return nullptr;
    std::vector<float> newStops = stops;
    if (sp.shader == RIVE_SCENE_SHADER_LINEAR)
    {
        g->type = PT_LINEAR;
        V2 start{sp.g[0], sp.g[1]}, end{sp.g[2], sp.g[3]};
        float firstStop = stops[0], lastStop = stops[count - 1];
        if ((firstStop != 0 || lastStop != 1) && lastStop - firstStop > kEPSILON)
        {
            // simd::precise_mix(a, b, t) = a * (1 - t) + b * t
            V2 ns{start.x * (1.f - firstStop) + end.x * firstStop,
                  start.y * (1.f - firstStop) + end.y * firstStop};
            V2 ne{start.x * (1.f - lastStop) + end.x * lastStop,
                  start.y * (1.f - lastStop) + end.y * lastStop};
            start = ns;
            end = ne;
            newStops[0] = 0;
            newStops[count - 1] = 1;
            if (count > 2)
            {
                float m = 1.f / (lastStop - firstStop);
                float a = -firstStop * m;
                for (size_t i = 1; i < count - 1; ++i)
                    newStops[i] = stops[i] * m + a;
                for (size_t i = 1; i < count - 1; ++i)
                    newStops[i] = fmaxf(newStops[i - 1], newStops[i]);
                for (size_t i = count - 2; i != 0; --i)
                    newStops[i] = fminf(newStops[i], newStops[i + 1]);
            }
        }
        V2 v = end - start;
        v = v * (1.f / (v.x * v.x + v.y * v.y));
        g->coeffs[0] = v.x;
        g->coeffs[1] = v.y;
        g->coeffs[2] = -(v.x * start.x + v.y * start.y);
    }
    else
    {
        g->type = PT_RADIAL;
        float radius = sp.g[2];
        float lastStop = stops[count - 1];
        if (lastStop != 1 && lastStop > kEPSILON)
        {
            newStops[count - 1] = 1;
            radius *= lastStop;
            float inverseLastStop = 1.f / lastStop;
            for (size_t i = 0; i < count - 1; ++i)
                newStops[i] = stops[i] * inverseLastStop;
            if (count > 1)
            {
                newStops[0] = fmaxf(0, newStops[0]);
                for (size_t i = 1; i < count - 1; ++i)
                    newStops[i] = fmaxf(newStops[i - 1], newStops[i]);
                for (size_t i = count - 2; i != (size_t)-1; --i)
                    newStops[i] = fminf(newStops[i], newStops[i + 1]);
            }
        }
        g->coeffs[0] = sp.g[0];
        g->coeffs[1] = sp.g[1];
        g->coeffs[2] = radius;
    }
    g->stops = newStops;
    return g;
}

struct Paint
{
    bool stroked = false;
    uint32_t color = 0xff000000;
    float thickness = 1;
    uint32_t join = J_MITER, cap = C_BUTT;
    uint32_t blendMode = 3; // rive::BlendMode::srcOver
    PaintType type = PT_SOLID;
    std::shared_ptr<Gradient> gradient;
    uint32_t outerClipID = 0; // clip updates
    bool isOpaque() const
    {
        if (blendMode != 3)
            return false;
        switch (type)
        {
            case PT_SOLID:
                return (color >> 24) == 0xff;
            case PT_LINEAR:
            case PT_RADIAL:
                return gradient->isOpaque();
            default:
                return false;
        }
    }
};

uint32_t pls_blend_mode(uint32_t riveMode)
{
    // ConvertBlendModeToPLSBlendMode (gpu.cpp:717-755)
    switch (riveMode)
    {
        case 3: return 0;   // srcOver
        case 14: return 1;  // screen
        case 15: return 2;  // overlay
        case 16: return 3;  // darken
        case 17: return 4;  // lighten
        case 18: return 5;  // colorDodge
        case 19: return 6;  // colorBurn
        case 20: return 7;  // hardLight
        case 21: return 8;  // softLight
        case 22: return 9;  // difference
        case 23: return 10; // exclusion
        case 24: return 11; // multiply
        case 25: return 12; // hue
        case 26: return 13; // saturation
        case 27: return 14; // color
        case 28: return 15; // luminosity
    }
    throw PlanError("unknown blend mode");
}

// ---------------------------------------------------------------------------
// Draws.
struct ResourceCounts
{
    size_t midpointFanTessVertexCount = 0;
    size_t pathCount = 0;
    size_t contourCount = 0;
    size_t maxTessellatedSegmentCount = 0;
};

struct ContourInfo
{
    size_t endVerb;  // index of the verb that ends this contour
    size_t endPt;    // index of the point that ends this contour
    size_t startVerb, startPt;
    size_t endLineIdx;
    size_t firstCurveIdx, endCurveIdx;
    size_t firstRotationIdx, endRotationIdx;
    V2 midpoint;
    bool closed;
    size_t strokeJoinCount;
    uint32_t strokeCapSegmentCount;
    uint32_t paddingVertexCount;
};

struct LogicalFlush;

struct PathDraw
{
    IBox pixelBounds{};
    IBox clippedPixelBounds{};
    M2 matrix;
    std::shared_ptr<Path> path;
    uint32_t fillRule = 0;
    PaintType paintType = PT_SOLID;
    uint32_t color = 0xff000000;          // SimplePaintValue.color
    uint16_t rampRow = 0, rampCol = 0;    // SimplePaintValue.colorRampLocation
    uint32_t outerClipID = 0;             // SimplePaintValue.outerClipID
    std::shared_ptr<Gradient> gradient;
    uint32_t blendMode = 3;
    uint32_t drawContents = 0;
    float strokeRadius = 0;
    bool isStroke() const { return strokeRadius != 0; }
    ContourDirections contourDirections = CD_FORWARD;
    uint32_t contourFlags = 0;
    uint32_t clipID = 0;
    uint32_t pathID = 0;
    // Draw::setClipRect: the render state's clip rect, if any.
    bool hasClipRect = false;
    M2 clipRectInverse; // ClipRectInverseMatrix::inverseMatrix()

    // initForMidpointFan
    float strokeMatrixMaxScale = 0;
    float polarSegmentsPerRadian = 0;
    uint32_t strokeJoin = J_MITER, strokeCap = C_BUTT;
    std::vector<ContourInfo> contours;
    std::vector<uint32_t> parametricSegmentCounts;
    std::vector<uint32_t> polarSegmentCounts;
    std::vector<std::pair<V2, V2>> tangentPairs;
    std::vector<uint8_t> numChops; // queue
    size_t numChopsHead = 0;
    std::vector<V2> chopVertices; // queue
    size_t chopVerticesHead = 0;
    ResourceCounts counts;

    void setClipID(uint32_t id)
    {
        clipID = id;
        if (!(drawContents & DC_CLIP_UPDATE))
        {
            if (clipID != 0)
                drawContents |= DC_ACTIVE_CLIP;
            else
                drawContents &= ~DC_ACTIVE_CLIP;
        }
    }

    void initForMidpointFan();
};

constexpr int STROKE_FLAG = 8, ROUND_JOIN_FLAG = 16;

// draw.cpp:253-276
uint32_t empty_stroke_cap(bool closed, uint32_t join, uint32_t cap)
{
    if (closed)
    {
        switch (join)
        {
            case J_ROUND: return C_ROUND;
            case J_MITER: return C_SQUARE;
            case J_BEVEL: return C_BUTT;
        }
    }
    return cap;
}

uint32_t join_type_flags(uint32_t join)
{
    switch (join)
    {
        case J_MITER: return MITER_REVERT_JOIN_CONTOUR_FLAG;
        case J_ROUND: return ROUND_JOIN_CONTOUR_FLAG;
        default: return BEVEL_JOIN_CONTOUR_FLAG;
    }
}

inline size_t round_up4(size_t x) { return (x + 3) & ~(size_t)3; }
template <size_t N> inline size_t padding_to_align_up(size_t x) { return (N - x % N) % N; }

// PathDraw::initForMidpointFan (draw.cpp:768-1392), rasterOrdering without
// feathers.
void PathDraw::initForMidpointFan()
{
    if (isStroke())
    {
        strokeMatrixMaxScale = matrix.findMaxScale();
        float r_ = strokeRadius * strokeMatrixMaxScale;
        polarSegmentsPerRadian = calc_polar_segments_per_radian(r_);
    }
    const std::vector<uint8_t>& verbs = path->verbs;
    const std::vector<V2>& pts = path->pts;
    size_t contourCount = path->countMoves();
    contours.reserve(contourCount);

    size_t lineCount = 0, unpaddedCurveCount = 0, emptyStrokeCountForCaps = 0;
    size_t curveIdx = 0, rotationIdx = 0;
    bool roundJoinStroked = isStroke() && strokeJoin == J_ROUND;
    int preChopVerbCount = 0;
    V2 endpointsSum{};
    bool closed = !isStroke();
    V2 lastTangent{0, 1}, firstTangent{0, 1};
    size_t contourFirstCurveIdx = 0, contourFirstRotationIdx = 0;
    size_t startVerb = 0, startPt = 0;

    auto growCurves = [&](size_t n) {
        if (parametricSegmentCounts.size() < n)
            parametricSegmentCounts.resize(n + 64, 0);
    };
    auto growRotations = [&](size_t n) {
        if (tangentPairs.size() < n)
        {
            tangentPairs.resize(n + 64);
            polarSegmentCounts.resize(n + 64, 0);
        }
    };
    auto finishContour = [&](size_t verbIdx, size_t ptIdx) {
        if (closed)
        {
            V2 finalPt = pts[ptIdx - 1];
            V2 movePt = pts[startPt];
            if (!bits_equal(movePt, finalPt))
            {
                if (roundJoinStroked)
                {
                    V2 tangent = movePt - finalPt;
                    growRotations(rotationIdx + 1);
                    tangentPairs[rotationIdx++] = {lastTangent, tangent};
                    lastTangent = tangent;
                }
                ++lineCount;
                ++preChopVerbCount;
                endpointsSum = endpointsSum + movePt;
            }
            if (roundJoinStroked && preChopVerbCount != 0)
            {
                growRotations(rotationIdx + 1);
                tangentPairs[rotationIdx++] = {lastTangent, firstTangent};
            }
        }
        size_t strokeJoinCount = (size_t)preChopVerbCount;
        if (!closed)
            strokeJoinCount = std::max<size_t>(strokeJoinCount, 1) - 1;
        ContourInfo ci{};
        ci.endVerb = verbIdx;
        ci.endPt = ptIdx;
        ci.startVerb = startVerb;
        ci.startPt = startPt;
        ci.endLineIdx = lineCount;
        ci.firstCurveIdx = contourFirstCurveIdx;
        ci.endCurveIdx = curveIdx;
        ci.firstRotationIdx = contourFirstRotationIdx;
        ci.endRotationIdx = rotationIdx;
        ci.midpoint = isStroke() ? V2{} : endpointsSum * (1.f / (float)preChopVerbCount);
        ci.closed = closed;
        ci.strokeJoinCount = strokeJoinCount;
        contours.push_back(ci);
        unpaddedCurveCount += curveIdx - contourFirstCurveIdx;
        contourFirstCurveIdx = curveIdx = round_up4(curveIdx);
        contourFirstRotationIdx = rotationIdx = round_up4(rotationIdx);
        growCurves(curveIdx + 4);
        if (isStroke())
            growRotations(rotationIdx + 4);
    };

    growCurves(8);
    if (isStroke())
        growRotations(8);
    size_t ptIdx = 0;
    for (size_t vi = 0; vi < verbs.size(); ++vi)
    {
        const uint8_t verb = verbs[vi];
        const size_t verbPt = ptIdx; // first new point of this verb
        switch (verb)
        {
            case V_MOVE:
                if (vi != 0)
                {
                    finishContour(vi, verbPt);
                    startVerb = vi;
                    startPt = verbPt;
                }
                preChopVerbCount = 0;
                endpointsSum = {0, 0};
                closed = !isStroke();
                lastTangent = {0, 1};
                firstTangent = {0, 1};
                ptIdx += 1;
                break;
            case V_CLOSE:
                closed = true;
                break;
            case V_LINE:
            {
                const V2* p = &pts[verbPt - 1];
                if (roundJoinStroked)
                {
                    V2 tangent = p[1] - p[0];
                    if (preChopVerbCount == 0)
                        firstTangent = tangent;
                    else
                    {
                        growRotations(rotationIdx + 1);
                        tangentPairs[rotationIdx++] = {lastTangent, tangent};
                    }
                    lastTangent = tangent;
                }
                ++preChopVerbCount;
                endpointsSum = endpointsSum + p[1];
                ++lineCount;
                ptIdx += 1;
                break;
            }
            case V_QUAD:
                throw PlanError("quadratic verbs are not supported");
            case V_CUBIC:
            {
                const V2* p = &pts[verbPt - 1];
                ++preChopVerbCount;
                if (isStroke())
                {
                    if (roundJoinStroked)
                    {
                        V2 t0 = find_cubic_tan0(p), t1 = find_cubic_tan1(p);
                        if (preChopVerbCount == 1)
                            firstTangent = t0;
                        else
                        {
                            growRotations(rotationIdx + 1);
                            tangentPairs[rotationIdx++] = {lastTangent, t0};
                        }
                        lastTangent = t1;
                    }
                    endpointsSum = endpointsSum + p[3];
                    float t[2];
                    bool areCusps = false;
                    int n = find_cubic_convex_180_chops(p, t, &areCusps);
                    uint8_t chopKey = (uint8_t)((n << 1) | (areCusps ? 1 : 0));
                    numChops.push_back(chopKey);
                    V2 local[16];
                    const V2* q = p;
                    int numChopsLocal = n;
                    if (areCusps && n > 0)
                    {
                        chopVertices.push_back({t[0], t[1]});
                        chop_cubic_around_cusps(p, local, t, n, strokeMatrixMaxScale);
                        q = local;
                        numChopsLocal = n * 2;
                    }
                    else if (n == 2)
                    {
                        chopVertices.push_back({t[0], t[1]});
                        chop_cubic_at(p, local, t[0], t[1]);
                        q = local;
                    }
                    else if (n == 1)
                    {
                        chop_cubic_at(p, local, t[0]);
                        q = local;
                        for (int k = 1; k <= 5; ++k)
                            chopVertices.push_back(local[k]);
                    }
                    for (int k = 0; k <= numChopsLocal; ++k, q += 3)
                    {
                        growCurves(curveIdx + 1);
                        growRotations(rotationIdx + 1);
                        float n4 = cubic_pow4(q, matrix);
                        memcpy(&parametricSegmentCounts[curveIdx], &n4, 4);
                        tangentPairs[rotationIdx] = {find_cubic_tan0(q), find_cubic_tan1(q)};
                        ++curveIdx;
                        ++rotationIdx;
                    }
                }
                else
                {
                    endpointsSum = endpointsSum + p[3];
                    growCurves(curveIdx + 1);
                    float n4 = cubic_pow4(p, matrix);
                    memcpy(&parametricSegmentCounts[curveIdx++], &n4, 4);
                }
                ptIdx += 3;
                break;
            }
            default:
                throw PlanError("bad verb");
        }
    }
    if (!verbs.empty())
        finishContour(verbs.size(), pts.size());
    growCurves(curveIdx + 4);
    if (isStroke())
        growRotations(rotationIdx + 4);

    // Pass 2 (draw.cpp:1185-1370).
    size_t contourFirstLineIdx = 0;
    size_t tessVertexCount = 0;
    for (ContourInfo& contour : contours)
    {
        size_t contourLineCount = contour.endLineIdx - contourFirstLineIdx;
        uint32_t contourVertexCount = (uint32_t)(contourLineCount * 2);
        uint32_t mergedSum = 0;
        size_t j;
        for (j = contour.firstCurveIdx; j < contour.endCurveIdx; j += 4)
        {
            for (size_t k = j; k < j + 4; ++k)
            {
                float n;
                memcpy(&n, &parametricSegmentCounts[k], 4);
                n = ceilf(sqrtf(sqrtf(n)));
                n = simd_clamp(n, 1.f, (float)kMaxParametricSegments);
                uint32_t u = (uint32_t)n;
                parametricSegmentCounts[k] = u;
                mergedSum += u;
            }
        }
        while (j-- > contour.endCurveIdx)
            contourVertexCount -= parametricSegmentCounts[j];

        if (isStroke())
        {
            for (j = contour.firstRotationIdx; j < contour.endRotationIdx; j += 4)
            {
                for (size_t k = j; k < j + 4; ++k)
                {
                    V2 a = tangentPairs[k].first, b = tangentPairs[k].second;
                    float numer = a.x * b.x + a.y * b.y;
                    float denom_pow2 = (a.x * a.x + a.y * a.y) * (b.x * b.x + b.y * b.y);
                    float cosTheta = numer / sqrtf(denom_pow2);
                    cosTheta = simd_clamp(cosTheta, -1.f, 1.f);
                    float theta = fast_acos(cosTheta);
                    float n = ceilf(theta * polarSegmentsPerRadian);
                    n = simd_clamp(n, 1.f, (float)kMaxPolarSegments);
                    uint32_t u = (uint32_t)n;
                    polarSegmentCounts[k] = u;
                    mergedSum += u;
                }
            }
            while (j-- > contour.endRotationIdx)
                contourVertexCount -= polarSegmentCounts[j];
            if (strokeJoin == J_ROUND)
                contourVertexCount -= (uint32_t)contour.strokeJoinCount;
            else
                contourVertexCount += (uint32_t)(contour.strokeJoinCount *
                                                 (NUM_SEGMENTS_IN_MITER_OR_BEVEL_JOIN - 1));
            bool empty = contour.endLineIdx == contourFirstLineIdx &&
                         contour.endCurveIdx == contour.firstCurveIdx;
            uint32_t cap = C_BUTT;
            bool needsCaps = false;
            if (!empty)
            {
                cap = strokeCap;
                needsCaps = !contour.closed;
            }
            else
            {
                cap = empty_stroke_cap(contour.closed, strokeJoin, strokeCap);
                needsCaps = cap != C_BUTT;
            }
            if (needsCaps)
            {
                if (cap == C_ROUND)
                {
                    float s = ceilf(polarSegmentsPerRadian * kPI);
                    s += 2;
                    s = fminf(s, (float)kMaxPolarSegments);
                    contour.strokeCapSegmentCount = (uint32_t)s;
                }
                else
                {
                    contour.strokeCapSegmentCount = NUM_SEGMENTS_IN_MITER_OR_BEVEL_JOIN;
                }
                emptyStrokeCountForCaps += empty ? 2 : 1;
                contourVertexCount += (contour.strokeCapSegmentCount - 1) * 2;
            }
        }
        else
        {
            contourVertexCount += (uint32_t)(contour.endCurveIdx - contour.firstCurveIdx);
        }
        contourVertexCount += mergedSum;
        contour.paddingVertexCount =
            (uint32_t)padding_to_align_up<kMidpointFanPatchSegmentSpan>(contourVertexCount);
        contourVertexCount += contour.paddingVertexCount;
        tessVertexCount += contourVertexCount;
        contourFirstLineIdx = contour.endLineIdx;
    }
    if (tessVertexCount > 0)
    {
        counts.pathCount = 1;
        counts.contourCount = contourCount;
        counts.maxTessellatedSegmentCount = lineCount + unpaddedCurveCount + emptyStrokeCountForCaps;
        counts.midpointFanTessVertexCount =
            contourDirections != CD_FORWARD ? tessVertexCount * 2 : tessVertexCount;
    }
}

// ---------------------------------------------------------------------------
// Frame output buffers (the mapped buffers of the frame).
template <typename T> struct Buf
{
    std::vector<T> v;
    T& push() { return v.emplace_back(); }
    void skip(size_t n) { v.resize(v.size() + n); }
    size_t size() const { return v.size(); }
};

#pragma pack(push, 1)
struct TessVertexSpan
{
    float pts[8];
    float joinTangent[2];
    float y, reflectionY;
    int32_t x0x1, reflectionX0X1;
    uint32_t segmentCounts, contourIDWithFlags;
};
struct PathRec
{
    float m[6];
    float strokeRadius, featherRadius;
    uint32_t zIndex;
    float atlas[3];
    uint32_t cov[4];
};
struct PaintRec
{
    uint32_t params;
    uint32_t value;
};
struct PaintAuxRec
{
    float paintMatrix[6];
    float gradSpan[2];
    float clipRectInverse[6];
    float inverseFwidth[2];
    float image[7];
    float pad[9];
};
struct ContourRec
{
    float midpoint[2];
    uint32_t pathID;
    uint32_t vertexIndex0;
};
struct GradSpanRec
{
    uint32_t horizontalSpan, yWithFlags, color0, color1;
};
struct UniformRec
{
    float inverseViewports[4];
    uint32_t renderTargetWidth, renderTargetHeight;
    uint32_t colorClearValue, coverageClearValue;
    int32_t updateBounds[4];
    float featherAtlasTextureInverseSize[2];
    float featherAtlasContentInverseViewport[2];
    uint32_t coverageBufferPrefix;
    float epsilonForPseudoMemoryBarrier;
    uint32_t pathIDGranularity;
    float vertexDiscardValue;
    float mipMapLODBias;
    uint32_t maxPathId;
    float ditherScale, ditherBias, ditherConversionToRGB10;
    uint32_t wireframeEnabled;
    uint8_t pad[256 - 104];
};
#pragma pack(pop)
static_assert(sizeof(TessVertexSpan) == 64, "span");
static_assert(sizeof(PathRec) == 64, "path");
static_assert(sizeof(PaintAuxRec) == 128, "aux");
static_assert(sizeof(UniformRec) == 256, "uniforms");

struct Frame
{
    Buf<UniformRec> uniforms;
    Buf<PathRec> paths;
    Buf<PaintRec> paints;
    Buf<PaintAuxRec> paintAux;
    Buf<ContourRec> contours;
    Buf<GradSpanRec> gradSpans;
    Buf<TessVertexSpan> tessSpans;
};

uint32_t swizzle_rgba(uint32_t c) // SwizzleRiveColorToRGBA
{
    uint32_t rot = (c << 16) | (c >> 16);
    return (c & 0xff00ff00u) | (rot & 0x00ff00ffu);
}
uint32_t swizzle_rgba_premul(uint32_t c) // SwizzleRiveColorToRGBAPremul
{
    uint32_t r = (c >> 16) & 0xff, g = (c >> 8) & 0xff, b = c & 0xff, a = c >> 24;
    uint32_t pr = r * a / 255, pg = g * a / 255, pb = b * a / 255, pa = 255 * a / 255;
    return pr | (pg << 8) | (pb << 16) | (pa << 24);
}

void set_span(TessVertexSpan& s, const V2 p[4], V2 joinTangent, float y, int32_t x0, int32_t x1,
              float reflectionY, int32_t rx0, int32_t rx1, uint32_t parametric, uint32_t polar,
              uint32_t join, uint32_t contourIDWithFlags)
{
    for (int k = 0; k < 4; ++k)
    {
        s.pts[2 * k] = p[k].x;
        s.pts[2 * k + 1] = p[k].y;
    }
    s.joinTangent[0] = joinTangent.x;
    s.joinTangent[1] = joinTangent.y;
    s.y = y;
    s.reflectionY = reflectionY;
    s.x0x1 = (int32_t)(((uint32_t)x1 << 16) | ((uint32_t)x0 & 0xffff));
    s.reflectionX0X1 = (int32_t)(((uint32_t)rx1 << 16) | ((uint32_t)rx0 & 0xffff));
    s.segmentCounts = (join << 20) | (polar << 10) | parametric;
    s.contourIDWithFlags = contourIDWithFlags;
}

struct ClipInfo
{
    IBox contentBounds;
    uint32_t parentClipID;
};

struct Context;

// RenderContext::TessellationWriter (render_context.cpp:3079-3402).
struct TessWriter
{
    LogicalFlush* flush;
    Frame* frame;
    uint32_t pathID;
    ContourDirections dirs;
    uint32_t pathTessLocation;
    uint32_t pathMirroredTessLocation;
    uint32_t nextCubicPaddingVertexCount = 0;

    uint32_t pushContour(V2 midpoint, bool isStroke, bool closed, uint32_t paddingVertexCount);
    void pushCubic(const V2 pts[4], V2 joinTangent, uint32_t parametric, uint32_t polar,
                   uint32_t join, uint32_t contourIDWithFlags)
    {
        uint32_t total = nextCubicPaddingVertexCount + parametric + polar + join - 1;
        nextCubicPaddingVertexCount = 0;
        if (dirs == CD_FORWARD)
            pushSpans(pts, joinTangent, total, parametric, polar, join, contourIDWithFlags);
        else
            pushDoubleSided(pts, joinTangent, total, parametric, polar, join, contourIDWithFlags);
    }
    void pushSpans(const V2 pts[4], V2 joinTangent, uint32_t total, uint32_t parametric,
                   uint32_t polar, uint32_t join, uint32_t flags)
    {
        uint32_t y = pathTessLocation / kTessTextureWidth;
        int32_t x0 = (int32_t)(pathTessLocation % kTessTextureWidth);
        int32_t x1 = x0 + (int32_t)total;
        for (;;)
        {
            set_span(frame->tessSpans.push(), pts, joinTangent, (float)y, x0, x1,
                     std::numeric_limits<float>::quiet_NaN(), -1, -1, parametric, polar, join,
                     flags);
            if (x1 > (int32_t)kTessTextureWidth)
            {
                ++y;
                x0 -= kTessTextureWidth;
                x1 -= kTessTextureWidth;
                continue;
            }
            break;
        }
        pathTessLocation += total;
    }
    void pushDoubleSided(const V2 pts[4], V2 joinTangent, uint32_t total, uint32_t parametric,
                         uint32_t polar, uint32_t join, uint32_t flags)
    {
        int32_t y = (int32_t)(pathTessLocation / kTessTextureWidth);
        int32_t x0 = (int32_t)(pathTessLocation % kTessTextureWidth);
        int32_t x1 = x0 + (int32_t)total;
        uint32_t reflectionY = (pathMirroredTessLocation - 1) / kTessTextureWidth;
        int32_t rx0 = (int32_t)((pathMirroredTessLocation - 1) % kTessTextureWidth + 1);
        int32_t rx1 = rx0 - (int32_t)total;
        for (;;)
        {
            set_span(frame->tessSpans.push(), pts, joinTangent, (float)y, x0, x1,
                     (float)reflectionY, rx0, rx1, parametric, polar, join, flags);
            if (x1 > (int32_t)kTessTextureWidth || rx1 < 0)
            {
                ++y;
                x0 -= kTessTextureWidth;
                x1 -= kTessTextureWidth;
                --reflectionY;
                rx0 += kTessTextureWidth;
                rx1 += kTessTextureWidth;
                continue;
            }
            break;
        }
        pathTessLocation += total;
        pathMirroredTessLocation -= total;
    }
};

struct Batch
{
    rive_cuda_draw_batch b;
};

struct LogicalFlush
{
    Context* ctx;
    Frame* frame;
    std::vector<std::unique_ptr<PathDraw>> draws;
    ResourceCounts counts;
    // Gradients.
    std::map<uint64_t, uint32_t> simpleGradients;
    std::vector<std::pair<uint32_t, uint32_t>> pendingSimpleGradDraws;
    std::vector<std::shared_ptr<Gradient>> complexGradients; // row order
    size_t pendingGradSpanCount = 0;
    std::vector<ClipInfo> clips;
    IBox combinedDrawBounds = IBox::maximallyNegative();
    uint32_t combinedDrawContents = 0;
    // Layout.
    size_t pathPaddingCount = 0, paintPaddingCount = 0, paintAuxPaddingCount = 0;
    size_t contourPaddingCount = 0, gradSpanPaddingCount = 0;
    uint32_t midpointFanTessVertexIdx = 0, midpointFanTessEndLocation = 0;
    uint32_t outerCubicTessVertexIdx = 0, outerCubicTessEndLocation = 0;
    uint32_t complexOffsetY = 0;
    float gradInverseHeight = 0;
    rive_cuda_flush_desc desc{};
    std::vector<rive_cuda_draw_batch> batches;
    uint32_t combinedShaderFeatures = 0;
    uint32_t currentPathID = 0, currentContourID = 0;

    explicit LogicalFlush(Context* c, Frame* f) : ctx(c), frame(f) {}

    bool allocateGradient(const std::shared_ptr<Gradient>& g, uint16_t* row, uint16_t* col);
    bool pushDraws(std::vector<std::unique_ptr<PathDraw>>& batch);
    uint32_t generateClipID(IBox contentBounds, uint32_t parentClipID)
    {
        if (clips.size() < kMaxPathID)
        {
            clips.push_back({contentBounds, parentClipID});
            return (uint32_t)clips.size();
        }
        return 0;
    }
    uint32_t pushContour(uint32_t pathID, V2 midpoint, bool isStroke, bool closed,
                         uint32_t vertexIndex0)
    {
        if (isStroke)
            midpoint.x = closed ? 1.f : 0.f;
        ContourRec& c = frame->contours.push();
        c.midpoint[0] = midpoint.x;
        c.midpoint[1] = midpoint.y;
        c.pathID = pathID;
        c.vertexIndex0 = vertexIndex0;
        return ++currentContourID;
    }
    void layout(size_t flushIdx, ResourceCounts* running, struct LayoutCounts* layoutCounts);
    void write();
    uint32_t pushPath(PathDraw* d);
    void pushPaddingVertices(uint32_t count, uint32_t location)
    {
        TessWriter w{this, frame, 0, CD_FORWARD, location, 0};
        static const V2 empty[4] = {};
        w.pushSpans(empty, {0, 0}, count, 0, 0, 1, 0);
    }
    void pushMidpointFanData(PathDraw* d, TessWriter* w);
    void pushDrawBatch(PathDraw* d, uint32_t tessVertexCount, uint32_t tessLocation);
};

uint32_t TessWriter::pushContour(V2 midpoint, bool isStroke, bool closed, uint32_t paddingVertexCount)
{
    nextCubicPaddingVertexCount = paddingVertexCount;
    uint32_t vertexIndex0 = pathTessLocation; // nextVertexIndex() for non-reverse directions
    return flush->pushContour(pathID, midpoint, isStroke, closed, vertexIndex0);
}

struct LayoutCounts
{
    size_t pathPaddingCount = 0, paintPaddingCount = 0, paintAuxPaddingCount = 0;
    size_t contourPaddingCount = 0, gradSpanCount = 0, gradSpanPaddingCount = 0;
    uint32_t maxGradTextureHeight = 0, maxTessTextureHeight = 0;
};

struct Context
{
    uint32_t width = 0, height = 0;
    uint32_t clearColor = 0xffffffff;
    uint32_t ditherMode = 1;
    uint32_t clipContentID = 0;
    std::vector<std::unique_ptr<LogicalFlush>> flushes;
    Frame frame;
    uint32_t gradTextureHeightAlloc = 0;

    bool isOutsideCurrentFrame(IBox b) const
    {
        return b.l >= (int32_t)width || b.t >= (int32_t)height || b.r <= 0 || b.b <= 0 ||
               b.l >= b.r || b.t >= b.b;
    }
    void logicalFlush()
    {
        clipContentID = 0;
        flushes.emplace_back(new LogicalFlush(this, &frame));
    }
};

bool LogicalFlush::allocateGradient(const std::shared_ptr<Gradient>& g, uint16_t* row, uint16_t* col)
{
    const std::vector<float>& stops = g->stops;
    size_t stopCount = stops.size();
    auto gradientDataHeight = [](size_t simple, size_t complex) {
        return (simple + kGradTextureWidthInSimpleRamps - 1) / kGradTextureWidthInSimpleRamps +
               complex;
    };
    if (stopCount == 1 || (stopCount == 2 && stops[0] == 0 && stops[1] == 1))
    {
        uint32_t c0 = g->colors[0], c1 = g->colors[std::min<size_t>(1, stopCount - 1)];
        uint64_t key = (uint64_t)c0 | ((uint64_t)c1 << 32);
        uint32_t idx;
        auto it = simpleGradients.find(key);
        if (it != simpleGradients.end())
        {
            idx = it->second;
        }
        else
        {
            if (gradientDataHeight(simpleGradients.size() + 1, complexGradients.size()) >
                kMaxTextureHeight)
                return false;
            idx = (uint32_t)(simpleGradients.size() * 2);
            simpleGradients[key] = idx;
            pendingSimpleGradDraws.push_back({c0, c1});
            ++pendingGradSpanCount;
        }
        *row = (uint16_t)(idx / kGradTextureWidth);
        *col = (uint16_t)(idx % kGradTextureWidth);
    }
    else
    {
        // GradientContentKey: same stops and colors share a row.
        uint32_t r = (uint32_t)-1;
        for (size_t i = 0; i < complexGradients.size(); ++i)
        {
            const Gradient& o = *complexGradients[i];
            if (o.colors == g->colors && o.stops == g->stops)
            {
                r = (uint32_t)i;
                break;
            }
        }
        if (r == (uint32_t)-1)
        {
            if (gradientDataHeight(simpleGradients.size(), complexGradients.size() + 1) >
                kMaxTextureHeight)
                return false;
            r = (uint32_t)complexGradients.size();
            complexGradients.push_back(g);
            pendingGradSpanCount += stopCount - 1;
        }
        *row = (uint16_t)r;
        *col = 0xffff;
    }
    return true;
}

// LogicalFlush::pushDraws (render_context.cpp:509-586).
bool LogicalFlush::pushDraws(std::vector<std::unique_ptr<PathDraw>>& batch)
{
    ResourceCounts c = counts;
    for (auto& d : batch)
    {
        c.midpointFanTessVertexCount += d->counts.midpointFanTessVertexCount;
        c.pathCount += d->counts.pathCount;
        c.contourCount += d->counts.contourCount;
        c.maxTessellatedSegmentCount += d->counts.maxTessellatedSegmentCount;
    }
    if (c.pathCount > kMaxPathID || c.contourCount > kMaxContourID ||
        c.midpointFanTessVertexCount > kMaxTessellationVertexCountBeforePadding)
        return false;
    for (auto& d : batch)
    {
        if (d->gradient)
        {
            if (!allocateGradient(d->gradient, &d->rampRow, &d->rampCol))
                return false;
        }
    }
    for (auto& d : batch)
    {
        combinedDrawContents |= d->drawContents;
        draws.push_back(std::move(d));
    }
    counts = c;
    return true;
}

// LogicalFlush::layoutResources (render_context.cpp:1116-1392).
void LogicalFlush::layout(size_t flushIdx, ResourceCounts* running, LayoutCounts* lc)
{
    ++counts.pathCount; // path 0: the clear color
    pathPaddingCount = padding_to_align_up<4>(counts.pathCount);
    paintPaddingCount = padding_to_align_up<32>(counts.pathCount);
    paintAuxPaddingCount = padding_to_align_up<2>(counts.pathCount);
    contourPaddingCount = padding_to_align_up<16>(counts.contourCount);
    gradSpanPaddingCount = padding_to_align_up<16>(pendingGradSpanCount);

    size_t totalTessVertexCountWithPadding = 0;
    if (counts.midpointFanTessVertexCount != 0)
    {
        midpointFanTessVertexIdx = kMidpointFanPatchSegmentSpan;
        midpointFanTessEndLocation =
            midpointFanTessVertexIdx + (uint32_t)counts.midpointFanTessVertexCount;
        uint32_t interiorPadding = (uint32_t)padding_to_align_up<kOuterCubicPatchSegmentSpanPlusJoin>(
            midpointFanTessEndLocation);
        outerCubicTessVertexIdx = midpointFanTessEndLocation + interiorPadding;
        outerCubicTessEndLocation = outerCubicTessVertexIdx;
        totalTessVertexCountWithPadding = outerCubicTessEndLocation + 1;
    }
    uint32_t tessDataHeight =
        (uint32_t)((totalTessVertexCountWithPadding + kTessTextureWidth - 1) / kTessTextureWidth);
    complexOffsetY = (uint32_t)((simpleGradients.size() + kGradTextureWidthInSimpleRamps - 1) /
                                kGradTextureWidthInSimpleRamps);

    desc.render_target_width = ctx->width;
    desc.render_target_height = ctx->height;
    desc.interlock_mode = 0;
    desc.color_load_action = flushIdx != 0 ? RIVE_CUDA_LOAD_PRESERVE : RIVE_CUDA_LOAD_CLEAR;
    desc.color_clear_value = ctx->clearColor;
    // tightenClipBounds: without clip scissor the combined bounds are the
    // join of every draw's pixel bounds.
    for (size_t i = draws.size(); i-- > 0;)
        combinedDrawBounds = combinedDrawBounds.join(draws[i]->pixelBounds);
    IBox target{0, 0, (int32_t)ctx->width, (int32_t)ctx->height};
    IBox ub = desc.color_load_action == RIVE_CUDA_LOAD_CLEAR ? target
                                                             : target.intersect(combinedDrawBounds);
    if (ub.empty())
        ub = {0, 0, 0, 0};
    desc.update_bounds[0] = ub.l;
    desc.update_bounds[1] = ub.t;
    desc.update_bounds[2] = ub.r;
    desc.update_bounds[3] = ub.b;
    desc.flush_uniform_offset_bytes = (uint32_t)(flushIdx * sizeof(UniformRec));
    desc.path_count = (uint32_t)counts.pathCount;
    desc.first_path = (uint32_t)(running->pathCount + lc->pathPaddingCount);
    desc.first_paint = (uint32_t)(running->pathCount + lc->paintPaddingCount);
    desc.first_paint_aux = (uint32_t)(running->pathCount + lc->paintAuxPaddingCount);
    desc.contour_count = (uint32_t)counts.contourCount;
    desc.first_contour = (uint32_t)(running->contourCount + lc->contourPaddingCount);
    desc.grad_span_count = (uint32_t)pendingGradSpanCount;
    desc.first_grad_span = (uint32_t)(lc->gradSpanCount + lc->gradSpanPaddingCount);
    desc.grad_data_height = complexOffsetY + (uint32_t)complexGradients.size();
    desc.tess_data_height = tessDataHeight;
    desc.dither_mode = ctx->ditherMode;

    running->pathCount += counts.pathCount;
    running->contourCount += counts.contourCount;
    lc->pathPaddingCount += pathPaddingCount;
    lc->paintPaddingCount += paintPaddingCount;
    lc->paintAuxPaddingCount += paintAuxPaddingCount;
    lc->contourPaddingCount += contourPaddingCount;
    lc->gradSpanCount += pendingGradSpanCount;
    lc->gradSpanPaddingCount += gradSpanPaddingCount;
    lc->maxGradTextureHeight = std::max(desc.grad_data_height, lc->maxGradTextureHeight);
    lc->maxTessTextureHeight = std::max(desc.tess_data_height, lc->maxTessTextureHeight);
}

// LogicalFlush::pushPath + PathData/PaintData/PaintAuxData::set
// (render_context.cpp:3037-3077, gpu.cpp:859-1063).
uint32_t LogicalFlush::pushPath(PathDraw* d)
{
    ++currentPathID;
    PathRec& pr = frame->paths.push();
    memcpy(pr.m, d->matrix.v, sizeof(pr.m));
    pr.strokeRadius = d->strokeRadius;
    pr.featherRadius = 0;
    pr.zIndex = 0;

    PaintRec& pd = frame->paints.push();
    uint32_t shiftedClipID = d->clipID << 16;
    uint32_t local = (uint32_t)d->paintType;
    switch (d->paintType)
    {
        case PT_SOLID:
            pd.value = swizzle_rgba(d->color);
            local |= shiftedClipID | (pls_blend_mode(d->blendMode) << 4);
            break;
        case PT_LINEAR:
        case PT_RADIAL:
        {
            uint32_t row = d->rampRow;
            if (d->rampCol == 0xffff)
                row += complexOffsetY;
            float y = ((float)row + .5f) * gradInverseHeight;
            memcpy(&pd.value, &y, 4);
            local |= shiftedClipID | (pls_blend_mode(d->blendMode) << 4);
            break;
        }
        case PT_CLIP_UPDATE:
            pd.value = shiftedClipID;
            local |= d->outerClipID << 16;
            break;
    }
    if (d->drawContents & DC_NONZERO)
        local |= PAINT_FLAG_NON_ZERO_FILL;
    else if (d->drawContents & DC_EVENODD)
        local |= PAINT_FLAG_EVEN_ODD_FILL;
    if (d->hasClipRect)
        local |= PAINT_FLAG_HAS_CLIP_RECT;
    pd.params = local;

    PaintAuxRec& ax = frame->paintAux.push();
    if (d->paintType == PT_LINEAR || d->paintType == PT_RADIAL)
    {
        const float* gc = d->gradient->coeffs;
        M2 pm;
        d->matrix.invert(&pm);
        if (d->paintType == PT_LINEAR)
        {
            M2 g;
            g.v[0] = gc[0];
            g.v[1] = 0;
            g.v[2] = gc[1];
            g.v[3] = 0;
            g.v[4] = gc[2];
            g.v[5] = 0;
            pm = g * pm;
        }
        else
        {
            float w = 1 / gc[2];
            M2 g;
            g.v[0] = w;
            g.v[1] = 0;
            g.v[2] = 0;
            g.v[3] = w;
            g.v[4] = -gc[0] * w;
            g.v[5] = -gc[1] * w;
            pm = g * pm;
        }
        float left, right;
        if (d->rampCol == 0xffff)
        {
            left = 0;
            right = (float)kGradTextureWidth;
        }
        else
        {
            left = (float)d->rampCol;
            right = left + 2;
        }
        ax.gradSpan[0] = (right - left - 1) * (1.f / kGradTextureWidth);
        ax.gradSpan[1] = (left + .5f) * (1.f / kGradTextureWidth);
        memcpy(ax.paintMatrix, pm.v, sizeof(pm.v));
    }
    if (d->hasClipRect)
    {
        const M2& m = d->clipRectInverse;
        memcpy(ax.clipRectInverse, m.v, sizeof(m.v));
        ax.inverseFwidth[0] = -1.f / (fabsf(m.v[0]) + fabsf(m.v[1]));
        ax.inverseFwidth[1] = -1.f / (fabsf(m.v[2]) + fabsf(m.v[3]));
    }
    else
    {
        // No clip rect: ClipRectInverseMatrix::WideOpen() = {0, 0, 0, 0, 1, 1}.
        ax.clipRectInverse[0] = ax.clipRectInverse[1] = ax.clipRectInverse[2] = 0;
        ax.clipRectInverse[3] = 0;
        ax.clipRectInverse[4] = ax.clipRectInverse[5] = 1;
        ax.inverseFwidth[0] = ax.inverseFwidth[1] = 0;
    }
    return currentPathID;
}

// PathDraw::pushMidpointFanTessellationData (draw.cpp:1992-2375).
void LogicalFlush::pushMidpointFanData(PathDraw* d, TessWriter* w)
{
    const std::vector<uint8_t>& verbs = d->path->verbs;
    const std::vector<V2>& pts = d->path->pts;
    const bool stroke = d->isStroke();
    for (const ContourInfo& contour : d->contours)
    {
        const V2* contourPts = &pts[contour.startPt];
        const V2* endPts = pts.data() + contour.endPt; // end.rawPtsPtr()
        size_t curveIdx = contour.firstCurveIdx;
        size_t rotationIdx = contour.firstRotationIdx;
        uint32_t joinTypeFlags = 0;
        bool roundJoinStroked = false;
        bool needsFirstCap = false;
        uint32_t capFlags = 0;
        if (stroke)
        {
            joinTypeFlags = join_type_flags(d->strokeJoin);
            roundJoinStroked = joinTypeFlags == ROUND_JOIN_CONTOUR_FLAG;
            if (contour.strokeCapSegmentCount != 0)
            {
                uint32_t cap = !contour.closed ? d->strokeCap
                                               : empty_stroke_cap(true, d->strokeJoin, d->strokeCap);
                capFlags = cap == C_BUTT     ? BEVEL_JOIN_CONTOUR_FLAG
                           : cap == C_SQUARE ? MITER_CLIP_JOIN_CONTOUR_FLAG
                                             : ROUND_JOIN_CONTOUR_FLAG;
                capFlags |= EMULATED_STROKE_CAP_CONTOUR_FLAG;
                needsFirstCap = true;
            }
        }
        uint32_t contourIDWithFlags =
            d->contourFlags |
            w->pushContour(contour.midpoint, stroke, contour.closed, contour.paddingVertexCount);
        const uint32_t notRoundJoinSegments = NUM_SEGMENTS_IN_MITER_OR_BEVEL_JOIN;

        auto findJoinTangent = [&](const V2* joinPoint) -> V2 {
            // find_join_tangent (draw.cpp:210-251)
            const V2* next = joinPoint + 1;
            next = next != endPts ? next : contourPts;
            V2 tangent = *next - *joinPoint;
            if (tangent != V2{0, 0})
                return tangent;
            for (const V2* p = joinPoint + 1; p != endPts; ++p)
                if (*p != *joinPoint)
                    return *p - *joinPoint;
            if (contour.closed)
                for (const V2* p = contourPts; p != joinPoint; ++p)
                    if (*p != *joinPoint)
                        return *p - *joinPoint;
            throw PlanError("no join tangent");
        };
        auto findEndingTangent = [&]() -> V2 {
            const V2* end = endPts;
            const V2 endpoint = end[-1];
            while (--end > contourPts)
            {
                V2 p = end[-1];
                if (p != endpoint)
                    return endpoint - p;
            }
            return {-1, 0};
        };
        auto findStartingTangent = [&]() -> V2 {
            const V2 p0 = contourPts[0];
            for (const V2* p = contourPts + 1; p < endPts; ++p)
                if (*p != p0)
                    return *p - p0;
            return {1, 0};
        };
        auto pushCapBeforeCubic = [&](const V2 cubic[4]) {
            // pushEmulatedStrokeCapAsJoinBeforeCubic (draw.cpp:2377-2398)
            V2 rev[4] = {cubic[3], cubic[2], cubic[1], cubic[0]};
            w->pushCubic(rev, find_cubic_tan0(cubic), 0, 0, contour.strokeCapSegmentCount,
                         contourIDWithFlags | capFlags);
        };

        V2 joinTangent{0, 1};
        uint32_t joinSegmentCount = 1;
        V2 implicitClose[2];
        size_t ptIdx = contour.startPt;
        for (size_t vi = contour.startVerb; vi < contour.endVerb; ++vi)
        {
            const uint8_t verb = verbs[vi];
            const bool isFinalVerb = vi + 1 == contour.endVerb;
            switch (verb)
            {
                case V_MOVE:
                    implicitClose[1] = pts[ptIdx];
                    ptIdx += 1;
                    break;
                case V_CLOSE:
                    break;
                case V_LINE:
                {
                    const V2* lp = &pts[ptIdx - 1];
                    if (stroke)
                    {
                        if (contour.closed || !isFinalVerb)
                        {
                            if (roundJoinStroked)
                            {
                                joinTangent = d->tangentPairs[rotationIdx].second;
                                joinSegmentCount = d->polarSegmentCounts[rotationIdx];
                                ++rotationIdx;
                            }
                            else
                            {
                                joinTangent = findJoinTangent(lp + 1);
                                joinSegmentCount = notRoundJoinSegments;
                            }
                        }
                        else
                        {
                            joinTangent = -findEndingTangent();
                            joinTypeFlags = capFlags;
                            joinSegmentCount = contour.strokeCapSegmentCount;
                        }
                    }
                    V2 cubic[4];
                    line_to_cubic(lp[0], lp[1], cubic);
                    if (needsFirstCap)
                    {
                        pushCapBeforeCubic(cubic);
                        needsFirstCap = false;
                    }
                    w->pushCubic(cubic, joinTangent, 1, 1, joinSegmentCount,
                                 contourIDWithFlags | joinTypeFlags);
                    ptIdx += 1;
                    break;
                }
                case V_CUBIC:
                {
                    const V2* cp = &pts[ptIdx - 1];
                    if (stroke)
                    {
                        const V2* p = cp;
                        uint8_t chopKey = d->numChops[d->numChopsHead++];
                        int numChops = 0;
                        V2 local[16];
                        if (chopKey == 3 || chopKey == 5) // cusps
                        {
                            V2 tt = d->chopVertices[d->chopVerticesHead++];
                            float cuspT[2] = {tt.x, tt.y};
                            chop_cubic_around_cusps(p, local, cuspT, chopKey >> 1,
                                                    d->strokeMatrixMaxScale);
                            p = local;
                            numChops = chopKey ^ 1;
                        }
                        else if (chopKey == 4) // 2 simple chops
                        {
                            V2 tt = d->chopVertices[d->chopVerticesHead++];
                            chop_cubic_at(p, local, tt.x, tt.y);
                            p = local;
                            numChops = 2;
                        }
                        else if (chopKey == 2) // 1 simple chop
                        {
                            local[0] = p[0];
                            for (int k = 0; k < 5; ++k)
                                local[1 + k] = d->chopVertices[d->chopVerticesHead++];
                            local[6] = p[3];
                            p = local;
                            numChops = 1;
                        }
                        if (needsFirstCap)
                        {
                            pushCapBeforeCubic(p);
                            needsFirstCap = false;
                        }
                        for (int k = 0; k < numChops; ++k, ++curveIdx, ++rotationIdx, p += 3)
                        {
                            w->pushCubic(p, joinTangent, d->parametricSegmentCounts[curveIdx],
                                         d->polarSegmentCounts[rotationIdx], 1,
                                         contourIDWithFlags | joinTypeFlags);
                        }
                        uint32_t parametric = d->parametricSegmentCounts[curveIdx++];
                        uint32_t polar = d->polarSegmentCounts[rotationIdx++];
                        if (contour.closed || !isFinalVerb)
                        {
                            if (roundJoinStroked)
                            {
                                joinTangent = d->tangentPairs[rotationIdx].second;
                                joinSegmentCount = d->polarSegmentCounts[rotationIdx];
                                ++rotationIdx;
                            }
                            else
                            {
                                joinTangent = findJoinTangent(cp + 3);
                                joinSegmentCount = notRoundJoinSegments;
                            }
                        }
                        else
                        {
                            joinTangent = -findEndingTangent();
                            joinTypeFlags = capFlags;
                            joinSegmentCount = contour.strokeCapSegmentCount;
                        }
                        w->pushCubic(p, joinTangent, parametric, polar, joinSegmentCount,
                                     contourIDWithFlags | joinTypeFlags);
                    }
                    else
                    {
                        uint32_t parametric = d->parametricSegmentCounts[curveIdx++];
                        w->pushCubic(cp, V2{}, parametric, 1, 1, contourIDWithFlags);
                    }
                    ptIdx += 3;
                    break;
                }
                default:
                    throw PlanError("bad verb");
            }
        }
        if (needsFirstCap)
        {
            V2 p0 = contourPts[0], left{p0.x - 1, p0.y}, right{p0.x + 1, p0.y};
            V2 a[4] = {p0, right, right, right};
            V2 b[4] = {p0, left, left, left};
            pushCapBeforeCubic(a);
            pushCapBeforeCubic(b);
        }
        else if (contour.closed)
        {
            implicitClose[0] = endPts[-1];
            if (!bits_equal(implicitClose[0], implicitClose[1]))
            {
                V2 cubic[4];
                line_to_cubic(implicitClose[0], implicitClose[1], cubic);
                if (roundJoinStroked)
                {
                    joinTangent = d->tangentPairs[rotationIdx].second;
                    joinSegmentCount = d->polarSegmentCounts[rotationIdx];
                    ++rotationIdx;
                }
                else if (stroke)
                {
                    joinTangent = findStartingTangent();
                    joinSegmentCount = notRoundJoinSegments;
                }
                w->pushCubic(cubic, joinTangent, 1, 1, joinSegmentCount,
                             contourIDWithFlags | joinTypeFlags);
            }
        }
    }
}

// pushMidpointFanDraw -> pushPathDraw -> pushDraw (render_context.cpp).
void LogicalFlush::pushDrawBatch(PathDraw* d, uint32_t tessVertexCount, uint32_t tessLocation)
{
    uint32_t baseInstance = tessLocation / kMidpointFanPatchSegmentSpan;
    uint32_t instanceCount = tessVertexCount / kMidpointFanPatchSegmentSpan;
    // pushPathDraw (render_context.cpp:3630-3639): clockwise fills get their
    // own shader variant in rasterOrdering.
    const uint32_t misc = (d->drawContents & DC_CLOCKWISE) ? MISC_CLOCKWISE_FILL : 0u;
    rive_cuda_draw_batch* batch;
    bool merge = !batches.empty() &&
                 batches.back().base_element + batches.back().element_count == baseInstance;
    if (merge)
    {
        // can_combine_shader_misc_flags (render_context.cpp:3680-3700):
        // strokes draw the same in either shader, so the flag only separates
        // batches when both hold fills.
        const rive_cuda_draw_batch& tail = batches.back();
        if ((tail.draw_contents & DC_ANY_FILL) && (d->drawContents & DC_ANY_FILL) &&
            (tail.shader_misc_flags & MISC_CLOCKWISE_FILL) != misc)
            merge = false;
    }
    if (merge)
    {
        batch = &batches.back();
        batch->element_count += instanceCount;
        batch->draw_contents |= d->drawContents;
        batch->shader_misc_flags |= misc;
    }
    else
    {
        batches.push_back(rive_cuda_draw_batch{});
        batch = &batches.back();
        batch->draw_type = 0;
        batch->element_count = instanceCount;
        batch->base_element = baseInstance;
        batch->draw_contents = d->drawContents;
        batch->shader_misc_flags = misc;
        batch->first_blend_mode = d->blendMode;
    }
    uint32_t features = 0;
    if (d->clipID != 0)
        features |= SF_CLIPPING;
    if (d->hasClipRect && d->paintType != PT_CLIP_UPDATE)
        features |= SF_CLIP_RECT;
    if (ctx->ditherMode == 1)
        features |= SF_DITHER;
    if (d->paintType != PT_CLIP_UPDATE)
    {
        switch (d->blendMode)
        {
            case 25: case 26: case 27: case 28:
                features |= SF_HSL;
                features |= SF_ADVANCED_BLEND;
                break;
            case 3:
                break;
            default:
                features |= SF_ADVANCED_BLEND;
                break;
        }
    }
    batch->shader_features |= features;
    uint32_t pathFeatures = 0;
    if (d->drawContents & DC_EVENODD)
        pathFeatures |= SF_EVEN_ODD;
    if ((d->drawContents & (DC_CLIP_UPDATE | DC_ACTIVE_CLIP)) == (DC_CLIP_UPDATE | DC_ACTIVE_CLIP))
        pathFeatures |= SF_NESTED_CLIPPING;
    batch->shader_features |= pathFeatures;
    combinedShaderFeatures |= batch->shader_features;
}

// LogicalFlush::writeResources (render_context.cpp:1424-2408).
void LogicalFlush::write()
{
    gradInverseHeight = 1.f / (float)ctx->gradTextureHeightAlloc;
    size_t firstTessSpan = frame->tessSpans.size();
    size_t tessAlignmentPadding = padding_to_align_up<4>(firstTessSpan);
    frame->tessSpans.skip(tessAlignmentPadding);
    desc.first_tess_span = (uint32_t)(firstTessSpan + tessAlignmentPadding);

    // Simple gradients: one empty span with 1px borders each.
    constexpr uint32_t ONE_TEXEL_FIXED = 65536 / kGradTextureWidth;
    for (size_t i = 0; i < pendingSimpleGradDraws.size(); ++i)
    {
        uint32_t y = (uint32_t)(i / kGradTextureWidthInSimpleRamps);
        uint32_t centerX = (uint32_t)((i % kGradTextureWidthInSimpleRamps) * 2 + 1);
        uint32_t cx = centerX * ONE_TEXEL_FIXED;
        GradSpanRec& s = frame->gradSpans.push();
        s.horizontalSpan = (cx << 16) | cx;
        s.yWithFlags = GRAD_SPAN_FLAG_LEFT_BORDER | GRAD_SPAN_FLAG_RIGHT_BORDER | y;
        s.color0 = pendingSimpleGradDraws[i].first;
        s.color1 = pendingSimpleGradDraws[i].second;
    }
    // Complex gradients: one span per stop interval, on a full row each.
    for (uint32_t i = 0; i < complexGradients.size(); ++i)
    {
        const Gradient& g = *complexGradients[i];
        uint32_t y = i + complexOffsetY;
        float m = (kGradTextureWidth - 1.f) * ONE_TEXEL_FIXED;
        float a = .5f * ONE_TEXEL_FIXED;
        uint32_t lastXFixed = (uint32_t)(g.stops[0] * m + a);
        uint32_t lastColor = g.colors[0];
        for (size_t k = 1; k < g.stops.size(); ++k)
        {
            uint32_t xFixed = (uint32_t)(g.stops[k] * m + a);
            uint32_t flags = GRAD_SPAN_FLAG_COMPLEX_BORDER;
            if (k == 1)
                flags |= GRAD_SPAN_FLAG_LEFT_BORDER;
            if (k == g.stops.size() - 1)
                flags |= GRAD_SPAN_FLAG_RIGHT_BORDER;
            GradSpanRec& s = frame->gradSpans.push();
            s.horizontalSpan = (xFixed << 16) | lastXFixed;
            s.yWithFlags = flags | y;
            s.color0 = lastColor;
            s.color1 = g.colors[k];
            lastColor = g.colors[k];
            lastXFixed = xFixed;
        }
    }

    // Path 0: the clear colour paint.
    frame->paths.skip(1);
    PaintRec& p0 = frame->paints.push();
    p0.params = (uint32_t)PT_SOLID;
    p0.value = swizzle_rgba(ctx->clearColor);
    frame->paintAux.skip(1);

    if (desc.tess_data_height > 0)
    {
        pushPaddingVertices(kMidpointFanPatchSegmentSpan, 0);
        if (outerCubicTessVertexIdx > midpointFanTessEndLocation)
            pushPaddingVertices(outerCubicTessVertexIdx - midpointFanTessEndLocation,
                                midpointFanTessEndLocation);
        pushPaddingVertices(1, outerCubicTessEndLocation);
    }

    // Draws in painter's order.
    for (auto& dp : draws)
    {
        PathDraw* d = dp.get();
        uint32_t tessVertexCount = (uint32_t)d->counts.midpointFanTessVertexCount;
        if (tessVertexCount == 0)
            continue;
        if (d->pathID == 0)
            d->pathID = pushPath(d);
        uint32_t tessLocation = midpointFanTessVertexIdx;
        midpointFanTessVertexIdx += tessVertexCount;
        uint32_t fwdCount, fwdLoc, mirCount, mirLoc;
        if (d->contourDirections == CD_FORWARD)
        {
            fwdCount = tessVertexCount;
            fwdLoc = tessLocation;
            mirCount = mirLoc = 0;
        }
        else if (d->contourDirections == CD_REVERSE_THEN_FORWARD)
        {
            fwdCount = mirCount = tessVertexCount / 2;
            fwdLoc = mirLoc = tessLocation + tessVertexCount / 2;
        }
        else
        {
            // forwardThenReverse (draw.cpp:1945-1965): forward from the start,
            // mirrored growing down from the end.
            fwdCount = mirCount = tessVertexCount / 2;
            fwdLoc = tessLocation;
            mirLoc = tessLocation + tessVertexCount;
        }
        (void)fwdCount;
        (void)mirCount;
        TessWriter w{this, frame, d->pathID, d->contourDirections, fwdLoc, mirLoc};
        pushMidpointFanData(d, &w);
        pushDrawBatch(d, tessVertexCount, tessLocation);
    }

    frame->paths.skip(pathPaddingCount);
    frame->paints.skip(paintPaddingCount);
    frame->paintAux.skip(paintAuxPaddingCount);
    frame->contours.skip(contourPaddingCount);
    frame->gradSpans.skip(gradSpanPaddingCount);

    desc.combined_shader_features = combinedShaderFeatures;
    desc.tess_span_count = (uint32_t)(frame->tessSpans.size() - desc.first_tess_span);
    desc.has_triangle_vertices = 0;
    desc.grad_texture_height = ctx->gradTextureHeightAlloc;
    desc.draw_batch_count = (uint32_t)batches.size();

    // FlushUniforms (gpu.cpp:767-834): Vulkan-style platform, no Y flips.
    UniformRec& u = frame->uniforms.push();
    memset(&u, 0, sizeof(u));
    u.inverseViewports[0] = 2.f / (float)desc.grad_data_height;
    u.inverseViewports[1] = 2.f / (float)desc.tess_data_height;
    u.inverseViewports[2] = 2.f / (float)ctx->width;
    u.inverseViewports[3] = 2.f / (float)ctx->height;
    u.renderTargetWidth = ctx->width;
    u.renderTargetHeight = ctx->height;
    u.colorClearValue = swizzle_rgba_premul(ctx->clearColor);
    u.coverageClearValue = 0;
    memcpy(u.updateBounds, desc.update_bounds, sizeof(u.updateBounds));
    u.featherAtlasTextureInverseSize[0] = 1.f / 0.f;
    u.featherAtlasTextureInverseSize[1] = 1.f / 0.f;
    u.featherAtlasContentInverseViewport[0] = 2.f / 0.f;
    u.featherAtlasContentInverseViewport[1] = 2.f / 0.f;
    u.coverageBufferPrefix = 0;
    u.epsilonForPseudoMemoryBarrier = 1e-9f;
    u.pathIDGranularity = 1;
    u.vertexDiscardValue = std::numeric_limits<float>::quiet_NaN();
    u.mipMapLODBias = -.5f;
    u.maxPathId = desc.path_count;
    u.ditherScale = ctx->ditherMode == 0 ? 0.0f : (1.0f / 256.0f);
    u.ditherBias = u.ditherScale * -0.5f;
    u.ditherConversionToRGB10 = ctx->ditherMode == 0 ? 0.0f : (-1.0f / 1024.0f) / u.ditherScale;
    u.wireframeEnabled = 0;
}

// ---------------------------------------------------------------------------
// RiveRenderer (renderer/src/rive_renderer.cpp).
struct ClipElement
{
    M2 matrix;
    std::shared_ptr<Path> path;
    uint32_t fillRule;
    IBox pixelBounds;
    uint32_t clipID = 0;
};

struct RenderState
{
    M2 matrix;
    size_t clipStackHeight = 0;
    IBox overallClipPixelBounds = IBox::maximal();
    float modulatedOpacity = 1.f;
    // RiveRenderer clip rect state (rive_renderer.cpp:267-323).
    bool hasClipRect = false;
    FBox clipRect{};
    M2 clipRectMatrix;
    M2 clipRectInverse; // ClipRectInverseMatrix of (clipRectMatrix, clipRect)
};

// colorModulateOpacity (src/shapes/paint/color.cpp:36-67): the alpha byte
// rescaled, rounded to nearest, clamped to [0, 255].
uint32_t color_modulate_opacity(uint32_t c, float opacity)
{
    float o = (float)(c >> 24) / 0xFF * opacity;
    uint32_t a = (uint32_t)std::lround(255.f * std::max(0.0f, std::min(1.0f, o)));
    return (c & 0x00ffffffu) | ((a & 0xffu) << 24);
}

// RiveRenderer::IsAABB (rive_renderer.cpp:16-55): a move and three lines
// forming an axis-aligned rectangle; any further points must equal p0.
bool is_aabb(const Path& path, FBox* out)
{
    const auto& v = path.verbs;
    const auto& p = path.pts;
    if (v.size() < 4 || v[0] != V_MOVE || v[1] != V_LINE || v[2] != V_LINE || v[3] != V_LINE ||
        p.size() < 4)
        return false;
    for (size_t i = 4; i < p.size(); ++i)
        if (p[i] != p[0])
            return false;
    const bool a = p[0].x == p[3].x && p[0].y == p[1].y && p[2].x == p[1].x && p[2].y == p[3].y;
    const bool b = p[0].x == p[1].x && p[0].y == p[3].y && p[2].x == p[3].x && p[2].y == p[1].y;
    if (!a && !b)
        return false;
    *out = {simd_min(p[0].x, p[2].x), simd_min(p[0].y, p[2].y), simd_max(p[0].x, p[2].x),
            simd_max(p[0].y, p[2].y)};
    return true;
}

// Mat2D::mapPoints (src/math/mat2d.cpp:59-101) for one point.
V2 map_point(const M2& m, V2 p)
{
    if (m.v[1] == 0.f && m.v[2] == 0.f)
        return {m.v[0] * p.x + m.v[4], m.v[3] * p.y + m.v[5]};
    float sx = m.v[2] * p.y + m.v[4], sy = m.v[1] * p.x + m.v[5];
    return {m.v[0] * p.x + sx, m.v[3] * p.y + sy};
}

// transform_rect_to_new_space (rive_renderer.cpp:230-265).
bool transform_rect_to_new_space(FBox* rect, const M2& currentMatrix, const M2& newMatrix)
{
    if (currentMatrix == newMatrix)
        return true;
    M2 currentToNew;
    if (!newMatrix.invert(&currentToNew))
        return false;
    currentToNew = currentToNew * currentMatrix;
    const float* c = currentToNew.v;
    float maxSkew = fmaxf(fabsf(c[1]), fabsf(c[2]));
    float maxScale = fmaxf(fabsf(c[0]), fabsf(c[3]));
    constexpr float kEpsilon = 1.f / (1 << 12); // math::EPSILON
    if (maxSkew > kEpsilon && maxScale > kEpsilon)
        return false;
    V2 a = map_point(currentToNew, {rect->l, rect->t});
    V2 b = map_point(currentToNew, {rect->r, rect->b});
    *rect = {simd_min(a.x, b.x), simd_min(a.y, b.y), simd_max(a.x, b.x), simd_max(a.y, b.y)};
    return true;
}

// ClipRectInverseMatrix::reset (gpu.cpp:689-706): pixel space to the clip
// rect's normalised [-1, +1]^2; all zeros (clip everything) when degenerate.
M2 clip_rect_inverse(const M2& clipMatrix, const FBox& r)
{
    float w = r.width(), h = r.height();
    M2 box;
    box.v[0] = w * .5f;
    box.v[1] = 0;
    box.v[2] = 0;
    box.v[3] = h * .5f;
    box.v[4] = (r.l + r.r) * 0.5f;
    box.v[5] = (r.t + r.b) * 0.5f;
    M2 m = clipMatrix * box;
    M2 inv;
    if (w <= 0 || h <= 0 || !m.invert(&inv))
    {
        for (float& x : inv.v)
            x = 0;
    }
    return inv;
}

struct Renderer
{
    Context* ctx;
    std::vector<RenderState> stack{1};
    std::vector<ClipElement> clipStack;
    std::vector<std::unique_ptr<PathDraw>> internalBatch;

    // PathDraw::Make + ctor + initForMidpointFan (draw.cpp:420-757).
    std::unique_ptr<PathDraw> makeDraw(const M2& matrix, const std::shared_ptr<Path>& path,
                                       uint32_t fillRule, const Paint& paint,
                                       const IBox* precomputed, float modulatedOpacity = 1.f)
    {
        IBox pixelBounds;
        if (precomputed)
            pixelBounds = *precomputed;
        else
        {
            FBox mapped = matrix.mapBoundingBox(path->pts.data(), path->pts.size());
            if (paint.stroked)
            {
                float outset = paint.thickness * .5f;
                if (paint.join == J_MITER)
                    outset *= kRiveMiterLimit;
                else if (paint.cap == C_SQUARE)
                    outset *= kSQRT2;
                FBox so = matrix.mapBoundingBox(FBox{0, 0, outset, outset});
                mapped = mapped.outset(so.width() + 1, so.height() + 1);
            }
            pixelBounds = mapped.roundOut();
        }
        if (ctx->isOutsideCurrentFrame(pixelBounds))
            return nullptr;
        auto d = std::make_unique<PathDraw>();
        d->pixelBounds = d->clippedPixelBounds = pixelBounds;
        d->matrix = matrix;
        d->path = path;
        d->fillRule = fillRule;
        d->paintType = paint.type;
        d->blendMode = paint.blendMode;
        // RiveRenderPaint::getGradientWithOpacity -> Gradient::getModulated
        // (gradient.cpp:191-221): every stop colour's alpha scaled.
        d->gradient = paint.gradient;
        if (paint.gradient && modulatedOpacity != 1.f)
        {
            auto g = std::make_shared<Gradient>(*paint.gradient);
            for (uint32_t& c : g->colors)
                c = color_modulate_opacity(c, modulatedOpacity);
            d->gradient = g;
        }
        if (paint.blendMode != 3)
            d->drawContents |= DC_ADVANCED_BLEND;
        // The reference tests the paint itself, before opacity modulation.
        if (paint.isOpaque())
            d->drawContents |= DC_OPAQUE;
        if (paint.stroked)
        {
            d->strokeRadius = paint.thickness * .5f;
            d->strokeRadius = fmaxf(d->strokeRadius, std::numeric_limits<float>::min());
            d->drawContents |= DC_STROKE;
            d->contourDirections = CD_FORWARD;
        }
        else if (fillRule == FILL_RULE_CLOCKWISE)
        {
            // draw.cpp:627-631, 657-680: clockwise fills keep their forward
            // triangles clockwise; a left-handed matrix reverses the
            // contours and negates the coverage.
            d->drawContents |= DC_CLOCKWISE;
            const M2& m = matrix;
            float det = m.v[0] * m.v[3] - m.v[2] * m.v[1];
            if (det < 0)
            {
                d->contourDirections = CD_FORWARD_THEN_REVERSE;
                d->contourFlags |= NEGATE_PATH_FILL_COVERAGE_FLAG;
            }
            else
            {
                d->contourDirections = CD_REVERSE_THEN_FORWARD;
            }
        }
        else
        {
            d->drawContents |= fillRule == 1 ? DC_EVENODD : DC_NONZERO;
            d->contourDirections = CD_REVERSE_THEN_FORWARD;
        }
        if (paint.type == PT_CLIP_UPDATE)
        {
            d->drawContents |= DC_CLIP_UPDATE;
            if (paint.outerClipID != 0)
                d->drawContents |= DC_ACTIVE_CLIP;
            d->outerClipID = paint.outerClipID;
        }
        if (paint.type == PT_SOLID)
            d->color = modulatedOpacity != 1.f ? color_modulate_opacity(paint.color, modulatedOpacity)
                                               : paint.color;
        d->strokeJoin = paint.join;
        d->strokeCap = paint.cap;
        d->initForMidpointFan();
        return d;
    }

    enum ApplyClipResult
    {
        CLIP_SUCCESS,
        CLIP_FAILURE,
        CLIP_FULLY_CLIPPED
    };

    // RiveRenderer::applyClip (rive_renderer.cpp:631-824), rasterOrdering.
    ApplyClipResult applyClip(PathDraw* draw)
    {
        RenderState& rs = stack.back();
        // Draw::setClipRect
        draw->hasClipRect = rs.hasClipRect;
        draw->clipRectInverse = rs.clipRectInverse;
        draw->clippedPixelBounds = draw->clippedPixelBounds.intersect(rs.overallClipPixelBounds);
        if (draw->clippedPixelBounds.empty() || ctx->isOutsideCurrentFrame(draw->clippedPixelBounds))
            return CLIP_FULLY_CLIPPED;
        size_t height = rs.clipStackHeight;
        if (height == 0)
            return CLIP_SUCCESS;
        size_t inBuffer = (size_t)-1;
        if (ctx->clipContentID != 0)
        {
            for (size_t i = height - 1; i != (size_t)-1; --i)
                if (clipStack[i].clipID == ctx->clipContentID)
                {
                    inBuffer = i;
                    break;
                }
        }
        uint32_t parentClipID = inBuffer == (size_t)-1 ? 0 : clipStack[inBuffer].clipID;
        for (size_t i = inBuffer + 1; i < height; ++i)
        {
            ClipElement& clip = clipStack[i];
            Paint clipPaint;
            clipPaint.type = PT_CLIP_UPDATE;
            clipPaint.outerClipID = parentClipID;
            auto clipDraw = makeDraw(clip.matrix, clip.path, clip.fillRule, clipPaint, &clip.pixelBounds);
            if (!clipDraw)
                throw PlanError("clip draw outside the frame");
            clip.clipID = ctx->flushes.back()->generateClipID(clipDraw->pixelBounds, parentClipID);
            if (clip.clipID == 0)
                return CLIP_FAILURE;
            clipDraw->setClipID(clip.clipID);
            if (!ctx->isOutsideCurrentFrame(clipDraw->pixelBounds))
                internalBatch.push_back(std::move(clipDraw));
            parentClipID = clip.clipID;
        }
        draw->setClipID(parentClipID);
        ctx->clipContentID = parentClipID;
        return CLIP_SUCCESS;
    }

    // RiveRenderer::clipAndPushDraw (rive_renderer.cpp:496-570).
    void clipAndPushDraw(std::unique_ptr<PathDraw> draw)
    {
        if (!draw)
            return;
        if (ctx->isOutsideCurrentFrame(draw->pixelBounds))
            return;
        for (int attempt = 0; attempt < 2; ++attempt)
        {
            internalBatch.clear();
            ApplyClipResult r = applyClip(draw.get());
            if (r == CLIP_FAILURE)
            {
                ctx->logicalFlush();
                continue;
            }
            if (r == CLIP_FULLY_CLIPPED)
                return;
            PathDraw* raw = draw.get();
            internalBatch.push_back(std::move(draw));
            if (!ctx->flushes.back()->pushDraws(internalBatch))
            {
                ctx->logicalFlush();
                // Reclaim the draw for the retry.
                for (auto& p : internalBatch)
                    if (p.get() == raw)
                        draw = std::move(p);
                internalBatch.clear();
                continue;
            }
            internalBatch.clear();
            return;
        }
        fprintf(stderr, "planner: draw dropped (clip stack or draw too complex)\n");
    }

    void drawPath(const std::shared_ptr<Path>& path, const Paint& paint)
    {
        if (path->verbs.empty())
            return;
        if (paint.stroked && !(paint.thickness > 0))
            return;
        if (stack.back().overallClipPixelBounds.empty())
            return;
        clipAndPushDraw(makeDraw(stack.back().matrix, path, path->fillRule, paint, nullptr,
                                 stack.back().modulatedOpacity));
    }

    void clipPath(const std::shared_ptr<Path>& path)
    {
        RenderState& rs = stack.back();
        if (rs.overallClipPixelBounds.empty())
            return;
        if (path->verbs.empty())
        {
            rs.overallClipPixelBounds = {0, 0, 0, 0};
            return;
        }
        // Axis-aligned rectangles become the ENABLE_CLIP_RECT clip rect.
        FBox rect;
        if (is_aabb(*path, &rect))
        {
            clipRectImpl(rect, path);
            return;
        }
        clipPathImpl(path);
    }

    // RiveRenderer::clipRectImpl (rive_renderer.cpp:267-323).
    void clipRectImpl(FBox rect, const std::shared_ptr<Path>& path)
    {
        RenderState& rs = stack.back();
        if (!(rect.width() > 0 && rect.height() > 0)) // AABB::isEmptyOrNaN
        {
            rs.overallClipPixelBounds = {0, 0, 0, 0};
            return;
        }
        if (rs.hasClipRect && !transform_rect_to_new_space(&rect, rs.matrix, rs.clipRectMatrix))
        {
            clipPathImpl(path);
            return;
        }
        if (!rs.hasClipRect)
        {
            rs.clipRect = rect;
            rs.clipRectMatrix = rs.matrix;
        }
        else
        {
            rs.clipRect = {simd_max(rs.clipRect.l, rect.l), simd_max(rs.clipRect.t, rect.t),
                           simd_min(rs.clipRect.r, rect.r), simd_min(rs.clipRect.b, rect.b)};
        }
        IBox pixelBounds = rs.clipRectMatrix.mapBoundingBox(rs.clipRect).roundOut();
        rs.overallClipPixelBounds = rs.overallClipPixelBounds.intersect(pixelBounds);
        rs.hasClipRect = true;
        rs.clipRectInverse = clip_rect_inverse(rs.clipRectMatrix, rs.clipRect);
    }

    // RiveRenderer::clipPathImpl (rive_renderer.cpp:323-382).
    void clipPathImpl(const std::shared_ptr<Path>& path)
    {
        RenderState& rs = stack.back();
        FBox pb = M2{}.mapBoundingBox(path->pts.data(), path->pts.size()); // path bounds
        if (!(pb.r - pb.l > 0 && pb.b - pb.t > 0))
        {
            rs.overallClipPixelBounds = {0, 0, 0, 0};
            return;
        }
        size_t height = rs.clipStackHeight;
        bool equivalent = clipStack.size() > height && clipStack[height].matrix == rs.matrix &&
                          clipStack[height].path->id == path->id &&
                          clipStack[height].fillRule == path->fillRule;
        if (!equivalent)
        {
            IBox pixelBounds = rs.matrix.mapBoundingBox(path->pts.data(), path->pts.size()).roundOut();
            rs.overallClipPixelBounds = rs.overallClipPixelBounds.intersect(pixelBounds);
            if (rs.overallClipPixelBounds.empty())
                return;
            clipStack.resize(height);
            clipStack.push_back({rs.matrix, path, path->fillRule, pixelBounds, 0});
        }
        else
        {
            rs.overallClipPixelBounds =
                rs.overallClipPixelBounds.intersect(clipStack[height].pixelBounds);
            if (rs.overallClipPixelBounds.empty())
                return;
        }
        rs.clipStackHeight = height + 1;
    }
};

// ---------------------------------------------------------------------------
std::vector<uint8_t> plan(const uint8_t* data, size_t size)
{
    if (size < sizeof(rive_scene_header))
        throw PlanError("scene too small");
    rive_scene_header hdr;
    memcpy(&hdr, data, sizeof(hdr));
    if (hdr.magic != RIVE_SCENE_MAGIC)
        throw PlanError("bad scene magic");
    if (hdr.width == 0 || hdr.height == 0 || hdr.width > 16384 || hdr.height > 16384)
        throw PlanError("bad canvas size");
    if (hdr.flags & RIVE_SCENE_FLAG_TRIANGULATE)
        throw PlanError("interior triangulation is not planned here (midpoint fans only)");
    size_t off = sizeof(hdr);
    auto need = [&](size_t n) {
        if (off + n > size)
            throw PlanError("truncated scene");
    };
    need(sizeof(rive_scene_path) * (size_t)hdr.path_count);
    std::vector<rive_scene_path> spaths(hdr.path_count);
    memcpy(spaths.data(), data + off, sizeof(rive_scene_path) * spaths.size());
    off += sizeof(rive_scene_path) * spaths.size();
    need(sizeof(rive_scene_paint) * (size_t)hdr.paint_count);
    std::vector<rive_scene_paint> spaints(hdr.paint_count);
    memcpy(spaints.data(), data + off, sizeof(rive_scene_paint) * spaints.size());
    off += sizeof(rive_scene_paint) * spaints.size();
    need(sizeof(rive_scene_cmd) * (size_t)hdr.cmd_count);
    std::vector<rive_scene_cmd> cmds(hdr.cmd_count);
    memcpy(cmds.data(), data + off, sizeof(rive_scene_cmd) * cmds.size());
    off += sizeof(rive_scene_cmd) * cmds.size();
    need(((size_t)hdr.verb_count + 3) & ~(size_t)3);
    const uint8_t* verbs = data + off;
    off += ((size_t)hdr.verb_count + 3) & ~(size_t)3;
    need(sizeof(float) * 2 * (size_t)hdr.point_count);
    std::vector<V2> points(hdr.point_count);
    memcpy(points.data(), data + off, sizeof(V2) * points.size());
    off += sizeof(V2) * points.size();
    need(sizeof(rive_scene_stop) * (size_t)hdr.stop_count);
    std::vector<rive_scene_stop> stops(hdr.stop_count);
    memcpy(stops.data(), data + off, sizeof(rive_scene_stop) * stops.size());

    // Factory: paths (RawPath + pruneEmptySegments) and paints.
    std::vector<std::shared_ptr<Path>> paths;
    for (uint32_t i = 0; i < hdr.path_count; ++i)
    {
        const rive_scene_path& sp = spaths[i];
        if ((size_t)sp.verb_offset + sp.verb_count > hdr.verb_count ||
            (size_t)sp.point_offset + sp.point_count > hdr.point_count)
            throw PlanError("path out of range");
        auto p = std::make_shared<Path>();
        p->fillRule = sp.fill_rule & RIVE_SCENE_FILL_RULE_MASK;
        p->id = i + 1;
        // RawPath::move/line/cubic/close with implicit moves.
        bool open = false;
        size_t lastMove = 0;
        const V2* pp = points.data() + sp.point_offset;
        const V2* pend = pp + sp.point_count;
        for (uint32_t v = 0; v < sp.verb_count; ++v)
        {
            uint8_t verb = verbs[sp.verb_offset + v];
            int adv = verb == V_CUBIC ? 3 : verb == V_QUAD ? 2 : verb == V_CLOSE ? 0 : 1;
            if (pp + adv > pend)
                throw PlanError("path points out of range");
            if (verb == V_MOVE)
            {
                open = true;
                lastMove = p->pts.size();
                p->verbs.push_back(V_MOVE);
                p->pts.push_back(*pp);
            }
            else if (verb == V_CLOSE)
            {
                if (open)
                {
                    p->verbs.push_back(V_CLOSE);
                    open = false;
                }
            }
            else
            {
                if (!open)
                {
                    V2 m = p->pts.empty() ? V2{0, 0} : p->pts[lastMove];
                    open = true;
                    lastMove = p->pts.size();
                    p->verbs.push_back(V_MOVE);
                    p->pts.push_back(m);
                }
                p->verbs.push_back(verb);
                p->pts.insert(p->pts.end(), pp, pp + adv);
            }
            pp += adv;
        }
        // Factory::makeRenderPath prunes; makeEmptyRenderPath + addRawPath
        // (rive_render_path.cpp:16-21, 115-120) keeps empty segments.
        if (!(sp.fill_rule & RIVE_SCENE_PATH_APPENDED))
            prune_empty_segments(*p);
        paths.push_back(p);
    }
    std::vector<Paint> paints;
    for (uint32_t i = 0; i < hdr.paint_count; ++i)
    {
        const rive_scene_paint& s = spaints[i];
        if (s.feather != 0)
            throw PlanError("feathered paints are not planned here (the reference front end plans them)");
        Paint q;
        q.stroked = s.style == RIVE_SCENE_STYLE_STROKE;
        q.type = PT_SOLID;
        q.color = s.color;
        q.thickness = fabsf(s.thickness);
        q.join = s.join;
        q.cap = s.cap;
        q.blendMode = s.blend_mode;
        if (s.shader != RIVE_SCENE_SHADER_NONE)
        {
            if ((size_t)s.stop_offset + s.stop_count > hdr.stop_count)
                throw PlanError("stops out of range");
            q.gradient = make_gradient(s, stops.data());
            q.type = q.gradient ? q.gradient->type : PT_SOLID;
            q.color = 0xff000000;
        }
        paints.push_back(q);
    }

    Context ctx;
    ctx.width = hdr.width;
    ctx.height = hdr.height;
    ctx.clearColor = hdr.clear_color;
    ctx.ditherMode = hdr.dither_mode;
    ctx.logicalFlush();
    {
        Renderer r{&ctx};
        for (const rive_scene_cmd& c : cmds)
        {
            switch (c.op)
            {
                case RIVE_SCENE_CMD_SAVE:
                    r.stack.push_back(r.stack.back());
                    break;
                case RIVE_SCENE_CMD_RESTORE:
                    if (r.stack.size() > 1)
                        r.stack.pop_back();
                    break;
                case RIVE_SCENE_CMD_TRANSFORM:
                {
                    M2 m;
                    memcpy(m.v, c.m, sizeof(m.v));
                    r.stack.back().matrix = r.stack.back().matrix * m;
                    break;
                }
                case RIVE_SCENE_CMD_DRAW_PATH:
                    if (c.a >= paths.size() || c.b >= paints.size())
                        throw PlanError("draw references a missing path or paint");
                    r.drawPath(paths[c.a], paints[c.b]);
                    break;
                case RIVE_SCENE_CMD_CLIP_PATH:
                    if (c.a >= paths.size())
                        throw PlanError("clip references a missing path");
                    r.clipPath(paths[c.a]);
                    break;
                case RIVE_SCENE_CMD_MODULATE_OPACITY:
                    // RiveRenderer::modulateOpacity (rive_renderer.cpp:115-119)
                    r.stack.back().modulatedOpacity =
                        std::max(0.0f, r.stack.back().modulatedOpacity * c.m[0]);
                    break;
                case RIVE_SCENE_CMD_DRAW_IMAGE:
                case RIVE_SCENE_CMD_DRAW_IMAGE_MESH:
                    throw PlanError("image draws are not planned here (the reference front end plans them)");
                default:
                    throw PlanError("bad command");
            }
        }
    }

    // RenderContext::flush: layout, allocate, write.
    ctx.clipContentID = 0;
    ResourceCounts running;
    LayoutCounts lc;
    for (size_t i = 0; i < ctx.flushes.size(); ++i)
        ctx.flushes[i]->layout(i, &running, &lc);
    // First frame of a fresh context: allocations grow to 125% of need.
    uint32_t gradRows = lc.maxGradTextureHeight;
    ctx.gradTextureHeightAlloc =
        gradRows == 0 ? 0 : std::min<uint32_t>((gradRows * 5) >> 2, kMaxTextureHeight);
    for (auto& f : ctx.flushes)
        f->write();

    // Serialise in the capture layout.
    std::vector<uint8_t> out;
    auto put = [&](const void* p, size_t n) {
        const uint8_t* b = (const uint8_t*)p;
        out.insert(out.end(), b, b + n);
    };
    uint32_t head[4] = {0x31504352u, hdr.width, hdr.height, 7};
    put(head, sizeof(head));
    auto putBuf = [&](const void* p, size_t n) {
        uint64_t nn = n;
        put(&nn, 8);
        if (n)
            put(p, n);
        static const uint8_t zeros[8] = {};
        put(zeros, (8 - (n & 7)) & 7);
    };
    Frame& fr = ctx.frame;
    putBuf(fr.uniforms.v.data(), fr.uniforms.v.size() * sizeof(UniformRec));
    putBuf(fr.paths.v.data(), fr.paths.v.size() * sizeof(PathRec));
    putBuf(fr.paints.v.data(), fr.paints.v.size() * sizeof(PaintRec));
    putBuf(fr.paintAux.v.data(), fr.paintAux.v.size() * sizeof(PaintAuxRec));
    putBuf(fr.contours.v.data(), fr.contours.v.size() * sizeof(ContourRec));
    putBuf(fr.gradSpans.v.data(), fr.gradSpans.v.size() * sizeof(GradSpanRec));
    putBuf(fr.tessSpans.v.data(), fr.tessSpans.v.size() * sizeof(TessVertexSpan));
    uint32_t nf = (uint32_t)ctx.flushes.size();
    put(&nf, 4);
    for (auto& f : ctx.flushes)
    {
        rive_cuda_flush_desc d = f->desc;
        d.draw_batches = nullptr;
        // The RCP1 flush record: the descriptor up to its draw_batches
        // pointer (this front end plans no feather atlas).
        put(&d, offsetof(rive_cuda_flush_desc, atlas_texture_width));
        if (!f->batches.empty())
            put(f->batches.data(), f->batches.size() * sizeof(rive_cuda_draw_batch));
    }
    return out;
}
} // namespace

extern "C" int rive_plan_scene(const void* scene,
                               size_t scene_bytes,
                               void** out,
                               size_t* out_bytes,
                               char* err,
                               size_t err_len)
{
    if (!scene || !out || !out_bytes)
        return 1;
    try
    {
        std::vector<uint8_t> cap = plan((const uint8_t*)scene, scene_bytes);
        void* p = malloc(cap.size());
        if (!p)
            return 3;
        memcpy(p, cap.data(), cap.size());
        *out = p;
        *out_bytes = cap.size();
        return 0;
    }
    catch (const std::exception& e)
    {
        if (err && err_len)
            snprintf(err, err_len, "%s", e.what());
        return 2;
    }
}

extern "C" void rive_plan_free(void* p) { free(p); }
