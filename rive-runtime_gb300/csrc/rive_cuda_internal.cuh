// Internal definitions shared by the sm_103a kernels of the flush backend.
//
// Record layouts are the reference's GPU records (renderer/include/rive/
// renderer/gpu.hpp): TessVertexSpan (291-376), GradientSpan (248-271),
// PathData (1593-1619), PaintData (1627-1653), PaintAuxData (1660-1691),
// ContourData (1698-1716), FlushUniforms (1466-1537). Flag values are those of
// renderer/src/shaders/constants.glsl.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rivecuda
{
constexpr int kTessTextureWidth = 2048;
constexpr int kTessTextureWidthLog2 = 11;
constexpr int kGradTextureWidth = 512;
constexpr int kPatchSegmentSpan = 8;   // kMidpointFanPatchSegmentSpan
constexpr int kPatchVertexCount = 42;  // kMidpointFanPatchVertexCount
constexpr int kPatchIndexCount = 72;   // kMidpointFanPatchIndexCount
constexpr int kPatchTriangleCount = 24;
// Outer-curve patches (interior triangulation; gpu.hpp:591-646).
constexpr int kOuterPatchSegmentSpan = 17;   // OuterCubicPatchSegmentSpanPlusJoin
constexpr int kOuterPatchVertexCount = 153;  // kOuterCurvePatchVertexCount
constexpr int kOuterPatchTriangleCount = 83; // kOuterCurvePatchIndexCount / 3
// Center-AA midpoint-fan patches (feathered fills; gpu.hpp:591-646): both AA
// ramps of an 8-segment span, the 9-vertex fan and the midpoint vertex.
constexpr int kCenterPatchVertexCount = 8 * 8 + 8 + 2;           // 74
constexpr int kCenterPatchTriangleCount = (8 * 12 + 7 * 3 + 3) / 3; // 40
// gpu::DrawType values (gpu.hpp:657-668).
constexpr uint32_t DRAW_MIDPOINT_FAN_PATCHES = 0u;
constexpr uint32_t DRAW_MIDPOINT_FAN_CENTER_AA_PATCHES = 1u;
constexpr uint32_t DRAW_OUTER_CURVE_PATCHES = 2u;
constexpr uint32_t DRAW_INTERIOR_TRIANGULATION = 3u;
constexpr uint32_t DRAW_FEATHER_ATLAS_BLIT = 4u;
constexpr uint32_t DRAW_IMAGE_MESH = 6u;

constexpr float kPi = 3.14159265359f;
constexpr float k2Pi = 6.28318530718f;
constexpr float kAARadius = .5f;

constexpr uint32_t GRAD_SPAN_FLAG_LEFT_BORDER = 0x80000000u;
constexpr uint32_t GRAD_SPAN_FLAG_RIGHT_BORDER = 0x40000000u;
constexpr uint32_t GRAD_SPAN_FLAG_COMPLEX_BORDER = 0x20000000u;
constexpr uint32_t GRAD_SPAN_FLAGS_MASK = 0xe0000000u;

constexpr uint32_t RETROFIT_TRI_STRIP_CONTOUR_FLAG = 1u << 31;
constexpr uint32_t CULL_EXCESS_TESSELLATION_SEGMENTS_CONTOUR_FLAG = 1u << 29;
constexpr uint32_t JOIN_TYPE_MASK = 7u << 26;
constexpr uint32_t MITER_CLIP_JOIN_CONTOUR_FLAG = 5u << 26;
constexpr uint32_t MITER_REVERT_JOIN_CONTOUR_FLAG = 4u << 26;
constexpr uint32_t ROUND_JOIN_CONTOUR_FLAG = 2u << 26;
constexpr uint32_t FEATHER_JOIN_CONTOUR_FLAG = 1u << 26;
constexpr uint32_t EMULATED_STROKE_CAP_CONTOUR_FLAG = 1u << 25;
constexpr uint32_t NEGATE_PATH_FILL_COVERAGE_FLAG = 1u << 24;
constexpr uint32_t MIRRORED_CONTOUR_CONTOUR_FLAG = 1u << 23;
constexpr uint32_t JOIN_TANGENT_0_CONTOUR_FLAG = 1u << 22;
constexpr uint32_t JOIN_TANGENT_INNER_CONTOUR_FLAG = 1u << 21;
constexpr uint32_t LEFT_JOIN_CONTOUR_FLAG = 1u << 20;
constexpr uint32_t RIGHT_JOIN_CONTOUR_FLAG = 1u << 19;
constexpr uint32_t CONTOUR_ID_MASK = 0xffffu;

constexpr int STROKE_VERTEX = 0;
constexpr int FAN_VERTEX = 1;
constexpr int FAN_MIDPOINT_VERTEX = 2;

constexpr uint32_t CLIP_UPDATE_PAINT_TYPE = 0u;
constexpr uint32_t SOLID_COLOR_PAINT_TYPE = 1u;
constexpr uint32_t LINEAR_GRADIENT_PAINT_TYPE = 2u;
constexpr uint32_t RADIAL_GRADIENT_PAINT_TYPE = 3u;
constexpr uint32_t PAINT_FLAG_EVEN_ODD_FILL = 0x200u;

constexpr uint32_t MAX_DENORM_F16 = 1023u;
constexpr float EPSILON_FP16_NON_DENORM = 6.2e-5f;

// gpu::ShaderFeatures (gpu.hpp:840-856).
constexpr uint32_t SF_CLIPPING = 1u << 0;
constexpr uint32_t SF_CLIP_RECT = 1u << 1;
constexpr uint32_t SF_ADVANCED_BLEND = 1u << 2;
constexpr uint32_t SF_FEATHER = 1u << 3;
constexpr uint32_t SF_EVEN_ODD = 1u << 4;
constexpr uint32_t SF_NESTED_CLIPPING = 1u << 5;
constexpr uint32_t SF_HSL_BLEND_MODES = 1u << 6;
constexpr uint32_t SF_DITHER = 1u << 7;
constexpr uint32_t SF_MODULATED_IMAGE = 1u << 8;
// gpu::ShaderMiscFlags::clockwiseFill (gpu.hpp:917), the one misc flag a
// rasterOrdering draw batch carries. It travels with each triangle's shader
// features in bit 15, which ShaderFeatures leaves free.
constexpr uint32_t MISC_CLOCKWISE_FILL = 1u << 1;
// Feathering (constants.glsl:19-43, draw_path_common.glsl:7-13).
constexpr int kGaussianTableSize = 512;
constexpr float kGaussianStddevs = 3.f;
constexpr float kFeatherCoverageBias = -2.f;
constexpr float kFeatherCoverageThreshold = -1.5f;
constexpr float kFeatherXCoordBias = .25f;
constexpr float kHorizontalCotangentThreshold = 1e3f;
constexpr float kHorizontalCotangentValue = 1e6f;
constexpr float kFeatherJoinHelperVertexCount = 3.f;
// The inverse feather table for tessellation softening (kernels_tess.cu).
cudaError_t upload_inverse_feather_lut(const float table[kGaussianTableSize]);
void build_inverse_feather_table(float out[kGaussianTableSize]);
// The tessellation pass's device functions on n host items (kernels_tess.cu;
// rive_cuda_eval_tessellation_math).
cudaError_t run_tess_math(int fn, const float* in, float* out, size_t n);
// Uploads the feather table to a device once (kernels_raster.cu).
cudaError_t ensure_feather_lut(int device);
void feather_table_f16(uint16_t out[kGaussianTableSize]);
constexpr uint32_t FEATURE_CLOCKWISE_FILL = 1u << 15;
// A featherAtlasBlit triangle (main scenes): its coverage is the feather
// atlas sampled at the pixel, its coverage planes carry atlas coordinates.
constexpr uint32_t FEATURE_ATLAS_BLIT = 1u << 12;
// An atlas fill triangle that faced away (the atlas fill pipeline culls
// nothing): turned clockwise, its coverage is subtracted.
constexpr uint32_t FEATURE_ATLAS_NEGATE = 1u << 11;
// An image-mesh triangle: its colour is the batch's image at the texture
// coordinates of the pixel (planes in the feather-plane slots), blended at
// once, triangle by triangle.
constexpr uint32_t FEATURE_IMAGE_MESH = 1u << 10;
// Two more bits of a triangle record's feature half-word, set only when the
// batch draws interior tiles as winding records: a fan triangle whose tiles
// are counted after its path's winding grid is complete, and the record of a
// patch's winding slot (one per midpoint-fan patch, after its 24 triangles).
constexpr uint32_t FEATURE_FAN_DEFERRED = 1u << 14;
constexpr uint32_t FEATURE_WINDING_SLOT = 1u << 13;
// A bin entry's value with this bit set names a winding slot, not a triangle.
constexpr uint32_t BIN_WINDING_ENTRY = 1u << 31;
// tileCounts value of a deferred fan triangle until its tiles are counted.
constexpr uint32_t kDeferredCount = 0xffffffffu;

// Per path of a batch, for drawing interior tiles as winding records: the
// path's tile box (clipped to the canvas), its place in the grid pool (one
// int32 winding and one edge byte per tile of the box), and the slot that
// carries its winding entries.
struct PathGrid
{
    int tx0, ty0, tx1, ty1; // tiles [tx0, tx1) x [ty0, ty1)
    uint32_t offset;        // first cell in the pool
    uint32_t flags;         // PATH_GRID_* bits
    uint32_t anchor;        // winding slot of the path's first patch
    uint32_t entries;       // winding entries (interior tiles with a nonzero winding)
    float length;           // pixels of control polygon (bounds the contour's length)
};
constexpr uint32_t PATH_GRID_ELIGIBLE = 1u; // a fill whose interior tiles may be winding records
constexpr uint32_t PATH_GRID_UNSAFE = 2u;   // a patch was discarded or non-finite: no winding records
constexpr uint32_t PATH_GRID_PLACED = 4u;   // the grid fits the pool (offset valid)
// Pixels of margin around a tile's pixel centres within which a contour edge
// or midpoint makes the tile an edge tile: an AA ramp lies within 1 px
// (max norm) of its contour edge, plus snapping and float rounding.
constexpr float kWindingEdgeMargin = 2.f;
// A path gets a winding grid only when its contour cannot mark more than
// this share of its box's tiles as edge tiles (a contour of length L crosses
// at most about 1.5 L / T tiles of size T, margins included): scribbles whose
// contour passes through nearly every tile keep their plain fans.
constexpr float kWindingMaxEdgeShare = .75f;

// Raster tiles: 16x16 by default; 8x8 and 32x32 are the autotuner's other
// choices (rive_cuda_set_raster_config).
constexpr int kTileSize = 16;
constexpr int kTileLog2 = 4;
constexpr int kRaster32SmemBytes = 1024 * 80 + 1024 * 4; // staged records + block masks

// Device error word bits (read by rive_cuda_sync).
constexpr uint32_t ERR_BAD_TESS_INDEX = 1u << 0;
constexpr uint32_t ERR_BAD_CONTOUR = 1u << 1;
constexpr uint32_t ERR_BAD_PATH = 1u << 2;
constexpr uint32_t ERR_RESERVED_8 = 1u << 3; // no longer raised (feathers are drawn)
constexpr uint32_t ERR_COORD_RANGE = 1u << 4;
constexpr uint32_t ERR_BIN_OVERFLOW = 1u << 5;
constexpr uint32_t ERR_BAD_MESH_INDEX = 1u << 6;

// One set-up triangle, ready for the tile raster (96 bytes). Edge k is
// E_k(p) = A_k * (p.x - ax_k) + B_k * (p.y - ay_k), positive inside. Each edge
// is anchored at its canonical endpoint (the same vertex for the two triangles
// that share the edge), so shared edges evaluate to bitwise-negated values and
// the fill is watertight. Coverage components are planes anchored at edge 0's
// anchor: cov(p) = c + gx * (p.x - ax_0) + gy * (p.y - ay_0). The record also
// carries the path's PaintData words, so the raster never reads them from
// global memory, and the pixel bounding box for sub-tile rejection.
struct __align__(16) TriRecord
{
    float4 e0;   // ax, ay, A, B
    float4 e1;
    float4 e2;
    float4 cov0; // covx: c, gx, gy; covy: c
    float4 cov1; // covy: gx, gy; paint.x, paint.y (as float bits)
    uint4 meta;  // pathAndFeatures, x0 | x1 << 16, y0 | y1 << 16, key | scene << 16
};
static_assert(sizeof(TriRecord) == 96, "TriRecord layout");

// An image texture in device memory: RGBA8 premultiplied texels of every mip
// level, level l at texel offset off[l] with size max(w >> l, 1) x
// max(h >> l, 1); `sampler` is the ImageSampler key it is drawn with
// (include/rive/shapes/paint/image_sampler.hpp: wrapX + 3 wrapY + 9 filter).
constexpr int kMaxMipLevels = 16;
struct ImageTex
{
    const uchar4* texels;
    uint32_t width, height, levels, sampler;
    uint32_t off[kMaxMipLevels];
};
constexpr uint32_t PAINT_FLAG_HAS_IMAGE = 0x800u;
constexpr uint32_t kNoImage = 0xffffffffu;

// The mesh of an imageMesh draw batch: its render buffers (float2 positions,
// float2 texture coordinates, uint16 triangle list), the vertices both
// vertex buffers hold, its ImageDrawInstance and its image slot.
struct MeshDesc
{
    const float2* positions;
    const float2* uvs;
    const uint16_t* indices;
    uint32_t vertexCount, indexCount;
    uint32_t imageDraw, image;
    uint32_t pad;
};
constexpr uint32_t kNoMesh = 0xffffffffu;

struct FlushParams
{
    // Record buffers at the frame's element 0.
    const uint4* paths;      // PathData as 4 x uint4
    const uint2* paints;     // PaintData
    const float4* paintAux;  // PaintAuxData as 8 x float4
    const uint4* contours;   // ContourData
    const uint4* gradSpans;  // GradientSpan
    const uint4* tessSpans;  // TessVertexSpan as 4 x uint4
    uint32_t firstPath, firstPaint, firstPaintAux, firstContour;
    uint32_t firstGradSpan, gradSpanCount;
    uint32_t firstTessSpan, tessSpanCount;
    uint32_t pathCount, contourCount;
    uint32_t gradDataHeight, tessDataHeight;
    uint32_t gradTextureHeight; // rows the normalised gradient coordinate spans
    uint32_t width, height;
    uint32_t pathIDGranularity;
    float ditherScale, ditherBias;
    uint32_t wireframe;
    uint32_t loadClear;
    uint32_t clearColorPremulRGBA; // packed RGBA8, R in the low byte
    // Intermediate textures.
    uint4* tess;    // 2048 x tessDataHeight
    uchar4* grad;   // 512 x gradDataHeight
    uint32_t* error;
    uint32_t* fb;   // render target, RGBA8, width x height
    uint32_t tilesX;
    const uint32_t* triangleVertices; // TriangleVertex records (3 words each)
    uint32_t triangleVertexCount;
    // This flush's FlushUniforms record (device); scene_uniforms_kernel copies
    // pathIDGranularity and the dither terms from it before any other pass.
    const uint8_t* uniforms;
    // The flush's feather atlas: atlasW x atlasH fp16 texels, row-major. A
    // main scene samples it for its featherAtlasBlit draws; the flush's atlas
    // scene (atlasMode = 1: width x height = the atlas content, no target)
    // renders it.
    uint16_t* atlas;
    uint32_t atlasW, atlasH;
    uint32_t atlasMode;
    // Images: the batch's image table, and per path of this flush the slot of
    // the image its paint modulates (kNoImage: none), written by the set-up.
    const ImageTex* images;
    uint32_t* pathImage;
    // Image meshes: the flush's ImageDrawInstance records (4 x float4 each:
    // view matrix, clip-rect inverse matrix, translates, then opacity, clip
    // ID, blend mode, z index as words), and FlushUniforms::mipMapLODBias
    // (copied by scene_uniforms_kernel).
    const float4* imageDraws;
    uint32_t imageDrawCount;
    float mipLodBias;
};

// One DrawBatch of one flush in a set-up work list: its first element (patch
// instance, or triangle vertex for interior triangulation), its shader
// features and where its triangle slots start.
struct PatchSegment
{
    uint32_t scene, baseElement, features, slotBase;
    // Pixel rectangle the segment's triangles are clipped to, as
    // left | top << 16 and right | bottom << 16: an atlas batch's scissor, or
    // everything (0, 0xffffffff) for the draw batches of a main scene.
    uint32_t scissorLT, scissorRB;
    // The draw batch's image: a slot of the batch's image table, or kNoImage.
    uint32_t image;
    // An imageMesh batch's entry in the batch's mesh table, or kNoMesh.
    uint32_t mesh;
};

// Set-up work lists: midpoint-fan patches, outer-curve patches, interior
// triangles, center-AA midpoint-fan patches (items: instances, instances,
// triangles, instances).
constexpr int kSetupLists = 4;

// The work of a batch of independent logical flushes ("scenes"); a single
// flush is a batch of one. Every kernel maps its global work index to a scene
// through the prefix arrays (base[0] = 0, base[count] = total).
struct BatchTables
{
    const FlushParams* scenes;       // [sceneCount]
    const uint32_t* gradSpanBase;    // [sceneCount + 1]
    const uint32_t* tessSpanBase;    // [sceneCount + 1]
    const uint32_t* tileBase;        // [sceneCount + 1]
    const uint2* sceneTiles;         // [sceneCount]: (tileBase, tilesX)
    // Per set-up list: segments [segCount] and the prefix of their items
    // [segCount + 1].
    const PatchSegment* segments[kSetupLists];
    const uint32_t* segBase[kSetupLists];
    uint32_t segCount[kSetupLists];
    uint32_t totalItems[kSetupLists];
    uint32_t sceneCount;
    uint32_t totalGradSpans, totalTessSpans, totalTiles;
    // Tiles [0, mainTiles) belong to the flushes' targets, the rest to their
    // feather atlases (scenes after the main ones).
    uint32_t mainTiles;
    int tileLog2; // raster tile size of this batch (3, 4 or 5)
    // Per triangle slot, when the batch holds feathered fills or image
    // meshes: the planes of the feather coverage's third and fourth
    // components (cotTheta, y0), or of a mesh triangle's texture coordinates
    // (u, v), as (z0, dz/dx, dz/dy, w0), (dw/dx, dw/dy, anchor x, anchor y).
    float4* featherPlanes;
    // Image meshes of the batch (PatchSegment::mesh indexes it).
    const MeshDesc* meshes;
    // Interior tiles as winding records (null grids: off). Midpoint-fan
    // patches then take fanSlotStride = 25 slots (24 triangles and the
    // winding slot), otherwise 24.
    uint32_t fanSlotStride;
    const uint32_t* pathBase;  // [sceneCount + 1]: first path of each scene
    PathGrid* grids;           // [pathBase[sceneCount]]
    int32_t* gridWinding;      // pool: per cell, deltas, then the winding
    uint8_t* gridEdge;         // pool: per cell, nonzero for an edge tile
    uint32_t gridCapacity;     // cells in the pool
    uint32_t* gridCounters;    // [0] cells asked for, [1] winding entries
};

// Index j with base[j] <= i < base[j + 1] (empty ranges skipped), n >= 1.
__device__ __forceinline__ uint32_t find_range(const uint32_t* __restrict__ base, uint32_t n,
                                               uint32_t i)
{
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(base + mid) <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}
} // namespace rivecuda
