// rive_cuda_flush_device_noalloc (include/rive_cuda.h): one logical flush of a
// small frame whose every intermediate (tessellation and gradient textures,
// triangle records, tile bins, scan/sort temporaries, status words) lives in
// one fixed, file-scope device pool. The call allocates nothing: no
// cudaMalloc/cudaFree, no allocating library routine. It launches the same
// kernels, in the same order, as rive_cuda_flush_device.
//
// The pool is one per device and per process, so calls that overlap in time
// (two host threads, or two streams of one device) race on it.
#include "rive_cuda.h"
#include "rive_cuda_internal.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace rivecuda
{
__global__ void color_ramp_kernel(BatchTables B);
__global__ void tessellate_kernel(BatchTables B);
__global__ void tessellate_feather_kernel(BatchTables B);
__global__ void patch_setup_kernel(BatchTables B,
                                   TriRecord* tris,
                                   uint32_t* tileCounts,
                                   uint8_t* tileMasks);
__global__ void patch_setup_feather_kernel(BatchTables B,
                                           TriRecord* tris,
                                           uint32_t* tileCounts,
                                           uint8_t* tileMasks);
__global__ void outer_setup_kernel(BatchTables B,
                                   TriRecord* tris,
                                   uint32_t* tileCounts,
                                   uint8_t* tileMasks);
__global__ void scene_uniforms_kernel(FlushParams* scenes, uint32_t sceneCount);
__global__ void bin_scatter_kernel(uint32_t slotCount,
                                   int tileLog2,
                                   const uint2* sceneTiles,
                                   const TriRecord* tris,
                                   const uint32_t* tileCounts,
                                   const uint8_t* tileMasks,
                                   const uint32_t* offsets,
                                   uint32_t capacity,
                                   uint32_t* error,
                                   uint32_t* keys,
                                   uint32_t* vals);
__global__ void tile_ranges_kernel(uint32_t pairCount,
                                   uint32_t tileCount,
                                   const uint32_t* keys,
                                   uint2* ranges);
__global__ void raster_tile_kernel(BatchTables B,
                                   const TriRecord* tris,
                                   const uint32_t* sortedSlots,
                                   const uint2* ranges);
__global__ void raster_tile_feather_kernel(BatchTables B,
                                   const TriRecord* tris,
                                   const uint32_t* sortedSlots,
                                   const uint2* ranges);
} // namespace rivecuda

using namespace rivecuda;

namespace
{
constexpr size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// Pool layout: each region starts on a 256-byte boundary.
constexpr size_t kMaxTiles = (RIVE_CUDA_NOALLOC_MAX_WIDTH / kTileSize) *
                             (RIVE_CUDA_NOALLOC_MAX_HEIGHT / kTileSize);
constexpr size_t kMaxSlots = (size_t)RIVE_CUDA_NOALLOC_MAX_PATCHES * kPatchTriangleCount;
constexpr size_t kStatusOff = 0;                                     // error word, pair total
constexpr size_t kTessOff = 256;
constexpr size_t kTessBytes = (size_t)kTessTextureWidth * RIVE_CUDA_NOALLOC_MAX_TESS_ROWS * 16;
constexpr size_t kGradOff = kTessOff + align256(kTessBytes);
constexpr size_t kGradBytes = (size_t)kGradTextureWidth * RIVE_CUDA_NOALLOC_MAX_GRAD_ROWS * 4;
constexpr size_t kTrisOff = kGradOff + align256(kGradBytes);
constexpr size_t kTrisBytes = kMaxSlots * sizeof(TriRecord);
constexpr size_t kCountsOff = kTrisOff + align256(kTrisBytes);
constexpr size_t kMasksOff = kCountsOff + align256(kMaxSlots * 4);
constexpr size_t kOffsetsOff = kMasksOff + align256(kMaxSlots);
constexpr size_t kKeysOff = kOffsetsOff + align256(kMaxSlots * 4 + 4);
constexpr size_t kPairBytes = (size_t)RIVE_CUDA_NOALLOC_MAX_BIN_ENTRIES * 4;
constexpr size_t kValsOff = kKeysOff + align256(kPairBytes);
constexpr size_t kKeysAltOff = kValsOff + align256(kPairBytes);
constexpr size_t kValsAltOff = kKeysAltOff + align256(kPairBytes);
constexpr size_t kRangesOff = kValsAltOff + align256(kPairBytes);
constexpr size_t kScanTempOff = kRangesOff + align256(kMaxTiles * sizeof(uint2));
constexpr size_t kScanTempBytes = 64u << 10;
constexpr size_t kSortTempOff = kScanTempOff + kScanTempBytes;
constexpr size_t kSortTempBytes = 4u << 20;
// Launch tables of the flush (a batch of one): FlushParams, prefix arrays and
// one PatchSegment per draw batch.
constexpr uint32_t kMaxSegments = 256;
constexpr size_t kTabScenes = 0;
constexpr size_t kTabPrefix = align256(sizeof(FlushParams));        // 3 x 2 u32
constexpr size_t kTabSceneTiles = kTabPrefix + 32;                  // 1 uint2
constexpr size_t kTabSegments = kTabSceneTiles + 16;
constexpr size_t kTabSegBase = kTabSegments + kMaxSegments * sizeof(PatchSegment);
constexpr size_t kTablesBytes = align256(kTabSegBase + 4 * (kMaxSegments + 1));
constexpr size_t kTablesOff = kSortTempOff + kSortTempBytes;
constexpr size_t kPoolBytes = kTablesOff + kTablesBytes;
static_assert(kPoolBytes == RIVE_CUDA_NOALLOC_POOL_BYTES,
              "RIVE_CUDA_NOALLOC_POOL_BYTES must match the pool layout");

constexpr int kMaxDevices = 64;
std::mutex gPoolMutex;
bool gTablesUp[kMaxDevices] = {};

int fail(char* err, size_t len, int code, const char* fmt, ...)
{
    if (err && len)
    {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, len, fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CKN(call)                                                                                  \
    do                                                                                             \
    {                                                                                              \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return fail(err, err_len, RIVE_CUDA_ERR_CUDA, "%s: %s", #call,                         \
                        cudaGetErrorString(_e));                                                   \
    } while (0)

uint32_t premul_clear(uint32_t argb)
{
    float a = (float)(argb >> 24) / 255.f;
    float r = (float)((argb >> 16) & 0xffu) / 255.f * a;
    float g = (float)((argb >> 8) & 0xffu) / 255.f * a;
    float b = (float)(argb & 0xffu) / 255.f * a;
    auto q = [](float x) {
        x = x < 0.f ? 0.f : (x > 1.f ? 1.f : x);
        return (uint32_t)(x * 255.f + .5f);
    };
    return q(r) | (q(g) << 8) | (q(b) << 16) | (q(a) << 24);
}
} // namespace

// The pool itself: zero-initialised at module load, never resized or freed.
static __device__ __align__(256) uint8_t gNoAllocScratch[RIVE_CUDA_NOALLOC_POOL_BYTES];

extern "C" int rive_cuda_flush_device_noalloc(const rive_cuda_flush_desc* d,
                                              const rive_cuda_device_buffers* buffers,
                                              void* target_pixels_device,
                                              void* cuda_stream,
                                              char* err,
                                              size_t err_len)
{
    if (err && err_len)
        err[0] = 0;
    if (!d || !buffers || !target_pixels_device)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!buffers->flush_uniforms)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush_uniforms is NULL");
    if (d->interlock_mode != 0)
        return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED,
                    "interlock mode %u not supported (rasterOrdering only)", d->interlock_mode);
    if (d->atlas_fill_batch_count || d->atlas_stroke_batch_count)
        return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED,
                    "the feather atlas needs the allocating path (rive_cuda_flush_device)");
    if (d->batch_images)
        for (uint32_t i = 0; i < d->draw_batch_count; ++i)
            if (d->batch_images[i].texture)
                return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED,
                            "images need the allocating path (rive_cuda_flush_device)");
    if (d->batch_meshes)
        for (uint32_t i = 0; i < d->draw_batch_count; ++i)
            if (d->batch_meshes[i].vertices)
                return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED,
                            "image meshes need the allocating path (rive_cuda_flush_device)");
    if (d->has_triangle_vertices)
        return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED,
                    "interior triangulation draws are not supported");
    if (d->draw_batch_count && !d->draw_batches)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT, "draw_batches is NULL");
    // Size limits of the fixed pool: refused before anything is launched.
    if (d->render_target_width == 0 || d->render_target_height == 0)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT, "empty render target");
    if (d->render_target_width > RIVE_CUDA_NOALLOC_MAX_WIDTH ||
        d->render_target_height > RIVE_CUDA_NOALLOC_MAX_HEIGHT)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                    "render target %ux%u exceeds the no-allocation limit %ux%u",
                    d->render_target_width, d->render_target_height, RIVE_CUDA_NOALLOC_MAX_WIDTH,
                    RIVE_CUDA_NOALLOC_MAX_HEIGHT);
    if (d->tess_data_height > RIVE_CUDA_NOALLOC_MAX_TESS_ROWS)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                    "tessellation texture height %u exceeds the no-allocation limit %u rows",
                    d->tess_data_height, RIVE_CUDA_NOALLOC_MAX_TESS_ROWS);
    if (d->grad_data_height > RIVE_CUDA_NOALLOC_MAX_GRAD_ROWS)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                    "gradient texture height %u exceeds the no-allocation limit %u rows",
                    d->grad_data_height, RIVE_CUDA_NOALLOC_MAX_GRAD_ROWS);
    uint64_t instances = 0;
    bool feather = false; // some batch draws with ENABLE_FEATHER
    for (uint32_t i = 0; i < d->draw_batch_count; ++i)
    {
        const rive_cuda_draw_batch& b = d->draw_batches[i];
        feather = feather || (b.shader_features & SF_FEATHER) != 0;
        if (b.draw_type != RIVE_CUDA_DRAW_MIDPOINT_FAN_PATCHES)
            return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED, "draw type %u not supported",
                        b.draw_type);
        // Only midpoint-fan batches reach here, feathered strokes included
        // (feathered fills draw in center-AA batches, which need the
        // allocating path's per-slot coverage planes).
        if (b.shader_misc_flags & ~MISC_CLOCKWISE_FILL)
            return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED,
                        "shader misc flags 0x%x not supported", b.shader_misc_flags);
        if (((uint64_t)b.base_element + b.element_count) * kPatchSegmentSpan >
            (uint64_t)d->tess_data_height * kTessTextureWidth)
            return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                        "batch %u reads past the tessellation texture", i);
        instances += b.element_count;
    }
    if (d->draw_batch_count > kMaxSegments)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                    "%u draw batches exceed the no-allocation limit %u", d->draw_batch_count,
                    kMaxSegments);
    if (instances > RIVE_CUDA_NOALLOC_MAX_PATCHES)
        return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                    "%llu patches exceed the no-allocation limit %u",
                    (unsigned long long)instances, RIVE_CUDA_NOALLOC_MAX_PATCHES);

    int dev = 0;
    CKN(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(err, err_len, RIVE_CUDA_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    uint8_t* pool = nullptr;
    {
        // The pool's address in the current CUDA context, looked up on every
        // call (cheap), so no address from an earlier context is reused. The
        // feather tables (copies into file-scope symbols, no allocation) go up
        // on the first call on each device.
        std::lock_guard<std::mutex> lock(gPoolMutex);
        void* p = nullptr;
        CKN(cudaGetSymbolAddress(&p, gNoAllocScratch));
        if (!gTablesUp[dev])
        {
            CKN(ensure_feather_lut(dev));
            gTablesUp[dev] = true;
        }
        pool = (uint8_t*)p;
    }
    cudaStream_t stream = (cudaStream_t)cuda_stream;
    uint32_t* dError = (uint32_t*)(pool + kStatusOff);

    FlushParams P = {};
    P.paths = (const uint4*)buffers->paths;
    P.paints = (const uint2*)buffers->paints;
    P.paintAux = (const float4*)buffers->paint_aux;
    P.contours = (const uint4*)buffers->contours;
    P.gradSpans = (const uint4*)buffers->grad_spans;
    P.tessSpans = (const uint4*)buffers->tess_spans;
    P.firstPath = d->first_path;
    P.firstPaint = d->first_paint;
    P.firstPaintAux = d->first_paint_aux;
    P.firstContour = d->first_contour;
    P.firstGradSpan = d->first_grad_span;
    P.gradSpanCount = d->grad_span_count;
    P.firstTessSpan = d->first_tess_span;
    P.tessSpanCount = d->tess_span_count;
    P.pathCount = d->path_count;
    P.contourCount = d->contour_count;
    P.gradDataHeight = d->grad_data_height;
    P.gradTextureHeight = d->grad_texture_height ? d->grad_texture_height : d->grad_data_height;
    P.tessDataHeight = d->tess_data_height;
    P.width = d->render_target_width;
    P.height = d->render_target_height;
    P.wireframe = d->wireframe;
    P.loadClear = d->color_load_action == RIVE_CUDA_LOAD_CLEAR;
    P.clearColorPremulRGBA = premul_clear(d->color_clear_value);
    P.error = dError;
    P.tess = (uint4*)(pool + kTessOff);
    P.grad = (uchar4*)(pool + kGradOff);
    P.fb = (uint32_t*)target_pixels_device;
    P.tilesX = (d->render_target_width + kTileSize - 1) / kTileSize;

    // FlushUniforms (renderer/include/rive/renderer/gpu.hpp:1466-1537) stay on
    // the device; scene_uniforms_kernel copies the fields the passes use.
    P.uniforms = (const uint8_t*)buffers->flush_uniforms + d->flush_uniform_offset_bytes;
    P.pathIDGranularity = 1;

    const uint32_t tilesX = P.tilesX;
    const uint32_t tilesY = (d->render_target_height + kTileSize - 1) / kTileSize;
    const uint32_t tiles = tilesX * tilesY;

    // Launch tables, built on the stack and copied into the pool.
    alignas(16) uint8_t tab[kTablesBytes];
    memset(tab, 0, sizeof(tab));
    memcpy(tab + kTabScenes, &P, sizeof(P));
    uint32_t* prefix = (uint32_t*)(tab + kTabPrefix); // grad, tess, tile bases: {0, total}
    prefix[1] = d->grad_span_count;
    prefix[3] = d->tess_span_count;
    prefix[5] = tiles;
    *(uint2*)(tab + kTabSceneTiles) = make_uint2(0u, tilesX);
    PatchSegment* segs = (PatchSegment*)(tab + kTabSegments);
    uint32_t* segBase = (uint32_t*)(tab + kTabSegBase);
    uint32_t segCount = 0, instAcc = 0;
    for (uint32_t i = 0; i < d->draw_batch_count; ++i)
    {
        const rive_cuda_draw_batch& b = d->draw_batches[i];
        if (!b.element_count)
            continue;
        segs[segCount] = PatchSegment{0u, b.base_element,
                                      b.shader_features | ((b.shader_misc_flags & MISC_CLOCKWISE_FILL)
                                                               ? FEATURE_CLOCKWISE_FILL
                                                               : 0u),
                                      instAcc * kPatchTriangleCount, 0u, 0xffffffffu, kNoImage,
                                      kNoMesh};
        segBase[segCount] = instAcc;
        ++segCount;
        instAcc += b.element_count;
    }
    segBase[segCount] = instAcc;
    uint8_t* dTab = pool + kTablesOff;
    CKN(cudaMemcpyAsync(dTab, tab, sizeof(tab), cudaMemcpyHostToDevice, stream));
    scene_uniforms_kernel<<<1, 32, 0, stream>>>((FlushParams*)(dTab + kTabScenes), 1u);
    BatchTables B = {};
    B.scenes = (const FlushParams*)(dTab + kTabScenes);
    B.gradSpanBase = (const uint32_t*)(dTab + kTabPrefix);
    B.tessSpanBase = (const uint32_t*)(dTab + kTabPrefix) + 2;
    B.tileBase = (const uint32_t*)(dTab + kTabPrefix) + 4;
    B.sceneTiles = (const uint2*)(dTab + kTabSceneTiles);
    // Midpoint-fan patches only (the other set-up lists stay empty).
    for (int l = 0; l < kSetupLists; ++l)
    {
        B.segments[l] = (const PatchSegment*)(dTab + kTabSegments);
        B.segBase[l] = (const uint32_t*)(dTab + kTabSegBase);
    }
    B.segCount[0] = segCount;
    B.totalItems[0] = instAcc;
    B.sceneCount = 1;
    B.mainTiles = tiles;
    B.tileLog2 = kTileLog2;
    B.totalGradSpans = d->grad_span_count;
    B.totalTessSpans = d->tess_span_count;
    B.totalTiles = tiles;

    // What must start at zero on every call: the error word, the tile
    // ranges, the gradient rows in use and the scan's leading offset.
    uint2* ranges = (uint2*)(pool + kRangesOff);
    CKN(cudaMemsetAsync(dError, 0, 4, stream));
    CKN(cudaMemsetAsync(ranges, 0, (size_t)tiles * sizeof(uint2), stream));
    if (d->grad_data_height)
        CKN(cudaMemsetAsync(P.grad, 0, (size_t)kGradTextureWidth * d->grad_data_height * 4, stream));

    if (d->grad_span_count)
        color_ramp_kernel<<<d->grad_span_count, 128, 0, stream>>>(B);
    if (d->tess_span_count)
        (feather ? tessellate_feather_kernel : tessellate_kernel)<<<
            (d->tess_span_count * 32u + 255u) / 256u, 256, 0, stream>>>(B);

    TriRecord* tris = (TriRecord*)(pool + kTrisOff);
    uint8_t* masks = (uint8_t*)(pool + kMasksOff);
    uint32_t* counts = (uint32_t*)(pool + kCountsOff);
    uint32_t* offs = (uint32_t*)(pool + kOffsetsOff);
    const uint32_t slots = (uint32_t)(instances * kPatchTriangleCount);
    uint32_t pairs = 0;
    if (slots)
    {
        (feather ? patch_setup_feather_kernel : patch_setup_kernel)<<<(instAcc + 3) / 4, 128, 0,
                                                                     stream>>>(B, tris, counts,
                                                                               masks);
        size_t tempBytes = 0;
        CKN(cub::DeviceScan::InclusiveSum(nullptr, tempBytes, counts, offs + 1, slots, stream));
        if (tempBytes > kScanTempBytes)
            return fail(err, err_len, RIVE_CUDA_ERR_OUT_OF_MEMORY,
                        "scan needs %zu temporary bytes, pool holds %zu", tempBytes,
                        kScanTempBytes);
        CKN(cudaMemsetAsync(offs, 0, 4, stream));
        CKN(cub::DeviceScan::InclusiveSum(pool + kScanTempOff, tempBytes, counts, offs + 1, slots,
                                          stream));
        CKN(cudaMemcpyAsync(&pairs, offs + slots, 4, cudaMemcpyDeviceToHost, stream));
        CKN(cudaStreamSynchronize(stream));
        if (pairs > RIVE_CUDA_NOALLOC_MAX_BIN_ENTRIES)
            return fail(err, err_len, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                        "%u tile bin entries exceed the no-allocation limit %u (target not "
                        "written)",
                        pairs, RIVE_CUDA_NOALLOC_MAX_BIN_ENTRIES);
    }
    uint32_t* keys = (uint32_t*)(pool + kKeysOff);
    uint32_t* vals = (uint32_t*)(pool + kValsOff);
    const uint32_t* sortedSlots = nullptr;
    if (pairs)
    {
        bin_scatter_kernel<<<(slots + 255) / 256, 256, 0, stream>>>(
            slots, kTileLog2, B.sceneTiles, tris, counts, masks, offs, pairs, dError, keys, vals);
        int endBit = 1;
        while ((1u << endBit) <= tiles)
            ++endBit;
        cub::DoubleBuffer<uint32_t> k(keys, (uint32_t*)(pool + kKeysAltOff));
        cub::DoubleBuffer<uint32_t> v(vals, (uint32_t*)(pool + kValsAltOff));
        size_t tempBytes = 0;
        CKN(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, k, v, (int)pairs, 0, endBit, stream));
        if (tempBytes > kSortTempBytes)
            return fail(err, err_len, RIVE_CUDA_ERR_OUT_OF_MEMORY,
                        "sort needs %zu temporary bytes, pool holds %zu", tempBytes,
                        kSortTempBytes);
        CKN(cub::DeviceRadixSort::SortPairs(pool + kSortTempOff, tempBytes, k, v, (int)pairs, 0,
                                            endBit, stream));
        tile_ranges_kernel<<<(pairs + 255) / 256, 256, 0, stream>>>(pairs, tiles, k.Current(),
                                                                  ranges);
        sortedSlots = v.Current();
    }
    (feather ? raster_tile_feather_kernel : raster_tile_kernel)<<<tiles, 256, 0, stream>>>(
        B, tris, sortedSlots, ranges);
    CKN(cudaGetLastError());

    // Device status of this flush (overflow and range flags of the kernels).
    uint32_t status = 0;
    CKN(cudaMemcpyAsync(&status, dError, 4, cudaMemcpyDeviceToHost, stream));
    CKN(cudaStreamSynchronize(stream));
    if (status)
        return fail(err, err_len, RIVE_CUDA_ERR_DEVICE_STATUS,
                    "device status 0x%x (1 tess index, 2 contour, 4 path, "
                    "16 coordinate range, 32 bin overflow, 64 mesh index)",
                    status);
    return RIVE_CUDA_OK;
}
