// C-ABI of the flush backend (include/rive_cuda.h): context, buffer rings,
// render targets and the per-flush kernel sequence.
//
// The ABI mirrors rive::gpu::RenderContextImpl
// (renderer/include/rive/renderer/render_context_impl.hpp:26-243) as
// implemented by RenderContextHelperImpl + BufferRing
// (render_context_helper_impl.hpp, buffer_ring.hpp): each record buffer is a
// 3-deep ring (gpu::kBufferRingSize, gpu.hpp:77) of pinned, write-combined
// host staging buffers, and unmap enqueues one host->device copy into a
// device-resident copy of the buffer. flush() then runs, in stream order:
//   color_ramp_kernel -> tessellate_kernel -> patch_setup_kernel (midpoint fans,
//   outer curves) + interior_setup_kernel ->
//   (scan) -> bin_scatter_kernel -> (radix sort by tile) ->
//   tile_ranges_kernel -> raster_tile_kernel.
#include "rive_cuda.h"
#include "rive_cuda_internal.cuh"

#include <cuda_fp16.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace rivecuda
{
__global__ void color_ramp_kernel(BatchTables B);
__global__ void tessellate_kernel(BatchTables B);
__global__ void tessellate_feather_kernel(BatchTables B);
__global__ void patch_setup_kernel(BatchTables B,
                                   TriRecord* tris,
                                   uint32_t* tileCounts,
                                   uint8_t* tileMasks);
__global__ void outer_setup_kernel(BatchTables B,
                                   TriRecord* tris,
                                   uint32_t* tileCounts,
                                   uint8_t* tileMasks);
__global__ void interior_setup_kernel(BatchTables B,
                                      TriRecord* tris,
                                      uint32_t* tileCounts,
                                      uint8_t* tileMasks);
__global__ void patch_setup_feather_kernel(BatchTables B,
                                           TriRecord* tris,
                                           uint32_t* tileCounts,
                                           uint8_t* tileMasks);
__global__ void patch_setup_winding_kernel(BatchTables B,
                                           TriRecord* tris,
                                           uint32_t* tileCounts,
                                           uint8_t* tileMasks);
__global__ void center_setup_kernel(BatchTables B,
                                    TriRecord* tris,
                                    uint32_t* tileCounts,
                                    uint8_t* tileMasks);
__global__ void scene_uniforms_kernel(FlushParams* scenes, uint32_t sceneCount);
__global__ void bin_fill_kernel(const uint32_t* pairTotal,
                                uint32_t capacity,
                                uint32_t sentinel,
                                uint32_t* keys);
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
// The same three with 16-bit tile keys (batches of at most 65,535 tiles).
__global__ void bin_fill16_kernel(const uint32_t* pairTotal,
                                  uint32_t capacity,
                                  uint32_t sentinel,
                                  uint16_t* keys);
__global__ void bin_scatter16_kernel(uint32_t slotCount,
                                     int tileLog2,
                                     const uint2* sceneTiles,
                                     const TriRecord* tris,
                                     const uint32_t* tileCounts,
                                     const uint8_t* tileMasks,
                                     const uint32_t* offsets,
                                     uint32_t capacity,
                                     uint32_t* error,
                                     uint16_t* keys,
                                     uint32_t* vals);
__global__ void tile_ranges16_kernel(uint32_t pairCount,
                                     uint32_t tileCount,
                                     const uint16_t* keys,
                                     uint2* ranges);
__global__ void ranges_guard_kernel(const uint32_t* pairTotal,
                                    uint32_t capacity,
                                    uint2* ranges,
                                    uint32_t tiles);
// The work-queue raster (kernels_raster.cu).
__global__ void raster_queue_kernel(BatchTables B,
                                    const TriRecord* tris,
                                    const uint32_t* sortedSlots,
                                    const uint2* ranges,
                                    const uint32_t* order,
                                    uint32_t* cursor,
                                    uint32_t tiles);
__global__ void raster_queue_feather_kernel(BatchTables B,
                                            const TriRecord* tris,
                                            const uint32_t* sortedSlots,
                                            const uint2* ranges,
                                            const uint32_t* order,
                                            uint32_t* cursor,
                                            uint32_t tiles);
// One mip level of an image from the level above (kernels_raster.cu).
__global__ void mip_level_kernel(const uchar4* src, uint32_t sw, uint32_t sh, uchar4* dst,
                                 uint32_t dw, uint32_t dh);
// The feather atlas pass at 8, 16 and 32 pixel tiles (kernels_raster.cu).
__global__ void raster_atlas8_kernel(BatchTables B, const TriRecord* tris,
                                     const uint32_t* sortedSlots, const uint2* ranges,
                                     uint32_t firstTile);
__global__ void raster_atlas_kernel(BatchTables B, const TriRecord* tris,
                                    const uint32_t* sortedSlots, const uint2* ranges,
                                    uint32_t firstTile);
__global__ void raster_atlas32_kernel(BatchTables B, const TriRecord* tris,
                                      const uint32_t* sortedSlots, const uint2* ranges,
                                      uint32_t firstTile);
__global__ void tile_order_keys_kernel(uint32_t tiles,
                                       const uint2* ranges,
                                       uint32_t* keys,
                                       uint32_t* vals);
// Interior tiles as winding records (kernels_raster.cu).
__global__ void path_init_kernel(BatchTables B);
__global__ void path_bounds_kernel(BatchTables B);
__global__ void path_alloc_kernel(BatchTables B);
__global__ void path_winding_kernel(BatchTables B, uint32_t* tileCounts);
__global__ void fan_filter_kernel(BatchTables B,
                                  const TriRecord* tris,
                                  uint32_t* tileCounts,
                                  uint8_t* tileMasks);
__global__ void bin_scatter_winding_kernel(BatchTables B,
                                           const TriRecord* tris,
                                           const uint32_t* tileCounts,
                                           const uint8_t* tileMasks,
                                           const uint32_t* offsets,
                                           uint32_t slotCount,
                                           uint32_t capacity,
                                           uint32_t* error,
                                           uint32_t* keys,
                                           uint32_t* vals);
// The raster kernels without and with the feather paths.
#define RIVE_DECLARE_RASTER(NAME)                                                                  \
    __global__ void NAME(BatchTables B, const TriRecord* tris, const uint32_t* sortedSlots,        \
                         const uint2* ranges);
RIVE_DECLARE_RASTER(raster_tile_kernel)
RIVE_DECLARE_RASTER(raster_tile_feather_kernel)
RIVE_DECLARE_RASTER(raster_tile8_kernel)
RIVE_DECLARE_RASTER(raster_tile8_feather_kernel)
RIVE_DECLARE_RASTER(raster_tile32_kernel)
RIVE_DECLARE_RASTER(raster_tile32_feather_kernel)
#undef RIVE_DECLARE_RASTER
} // namespace rivecuda

using namespace rivecuda;

namespace
{
constexpr int kRingSize = 3;

struct DeviceBuffer
{
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t need)
    {
        if (need <= bytes)
            return cudaSuccess;
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t n = std::max(need, (size_t)256);
        n = n + n / 4; // grow by 1.25x, like RenderContext's resource growth
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess)
            bytes = n;
        return e;
    }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

struct HostBuffer
{
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t need)
    {
        if (need <= bytes)
            return cudaSuccess;
        if (ptr)
            cudaFreeHost(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t n = std::max(need, (size_t)4096);
        n = n + n / 4;
        cudaError_t e = cudaMallocHost(&ptr, n);
        if (e == cudaSuccess)
            bytes = n;
        return e;
    }
    void release()
    {
        if (ptr)
            cudaFreeHost(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

struct RecordRing
{
    void* host[kRingSize] = {};
    cudaEvent_t done[kRingSize] = {};
    size_t capacity = 0;
    int current = 0;
    bool mapped = false;
    // Two device copies in turn: an upload goes to the copy the flushes in
    // flight do not read, on the context's copy stream, so frame k+1's
    // records cross while frame k renders. `slot` is the copy the next flush
    // reads; `used` says a flush has read it since its upload (the next
    // upload then takes the other copy, once the flushes that read that one
    // are done: `readDone`). `copied` orders a flush after its slot's upload.
    DeviceBuffer device[2];
    size_t deviceValidBytes[2] = {};
    int slot = 0;
    bool used = false;
    cudaEvent_t readDone[2] = {};
    cudaEvent_t copied[2] = {};
};
} // namespace

// An image texture (rive_cuda_texture_create): one device allocation with
// every mip level, and its descriptor for the kernels.
namespace
{
struct PendingFlush;
} // namespace

struct rive_cuda_texture
{
    void* mem = nullptr;
    rivecuda::ImageTex desc = {};
    uint32_t texels = 0;
};

// A RenderBuffer of image-mesh data (rive_cuda_render_buffer_create).
struct rive_cuda_render_buffer
{
    void* mem = nullptr;
    size_t bytes = 0;
    uint32_t type = 0;
};

struct rive_cuda_render_target
{
    uint32_t width = 0, height = 0;
    uint32_t* pixels = nullptr;
    // An asynchronous read-back on the context's read stream that the next
    // raster into this target waits for (readPending until a flush took it).
    cudaEvent_t readDone = nullptr;
    bool readPending = false;
};

struct rive_cuda_context
{
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copyStream = nullptr; // record uploads (rive_cuda_unmap_buffer)
    cudaStream_t readStream = nullptr; // asynchronous read-backs of targets
    bool readsInFlight = false;        // read-backs queued since the last sync
    // Set by rive_cuda_flush for one flush: the raster waits for it (a
    // read-back of the target still in flight), the front half does not.
    cudaEvent_t rasterWait = nullptr;
    // The stream of the last batch and an event after its work (the next
    // batch on another stream waits for it).
    cudaStream_t lastStream = nullptr;
    cudaEvent_t lastDone = nullptr;
    std::string lastError;
    RecordRing rings[RIVE_CUDA_BUFFER_KIND_COUNT];
    DeviceBuffer tess, grad;
    uint32_t tessWidth = 0, tessHeight = 0, gradWidth = 0, gradHeight = 0;
    DeviceBuffer tris, tileCounts, tileMasks, offsets, featherPlanes;
    DeviceBuffer keys, vals, keysAlt, valsAlt, sortTemp, scanTemp, ranges;
    DeviceBuffer dTables;  // batch tables (device)
    // Pinned staging of the tables, a ring of three, so the host writes the
    // next flush's tables while earlier copies are still queued.
    static constexpr int kTableRing = 3;
    HostBuffer hTables[kTableRing];
    cudaEvent_t tablesCopied[kTableRing] = {};
    int tableSlot = 0;
    // Speculative bins (flushes on the context's own stream): the back half
    // of a flush is enqueued with bins sized from the largest bin-entry total
    // seen (plus a quarter) instead of waiting for the scan's total; the
    // total is read back without a wait and checked at the next call
    // (settle_pending), which re-runs the back half with exact bins in the
    // rare case it did not fit. binHighWater = 0: no total seen yet.
    bool speculate = true;
    uint32_t binHighWater = 0;
    PendingFlush* pending = nullptr;
    uint32_t* hSpecTotal = nullptr;    // pinned: the pending flush's scanned total
    uint32_t* dSpecOverflow = nullptr; // bin overflow status of speculative passes
    uint32_t* dError = nullptr;
    uint32_t* hError = nullptr;  // pinned
    uint32_t* hPairs = nullptr;  // pinned: scanned pair total
    // Interior tiles as winding records (rive_cuda_set_winding_tiles): per-path
    // grids and the cell pool, grown when a flush asked for more cells.
    bool windingTiles = false;
    // Raster as a persistent work queue over heaviest-first tiles
    // (rive_cuda_set_raster_queue; 16-pixel tiles).
    bool rasterQueue = false;
    int queueCtas[2] = {0, 0}; // resident queue CTAs per SM [feather variant]
    int smCount = 0;
    DeviceBuffer queueKeys, queueVals, queueKeysAlt, queueValsAlt, queueTemp, queueCursor;
    DeviceBuffer pathGrids, gridWinding, gridEdge, gridCounters;
    DeviceBuffer atlas; // the batch's feather atlases (fp16 texels)
    DeviceBuffer pathImage; // per path of the batch: the slot of its image
    uint32_t gridCapacity = 0;
    uint32_t* hGridCounters = nullptr; // pinned: cells asked, winding entries
    rive_cuda_flush_stats stats = {};
    // Raster configuration (rive_cuda_set_raster_config).
    int tileLog2 = kTileLog2;
    int rasterCtasPerSm = 0; // 0: as many as fit
    bool raster32Ready = false;
    size_t rasterPad[2][2] = {};      // [feather variant][8 or 16 pixel kernel]: padding
    int rasterPadFor[2] = {-1, -1};   // the CTAs-per-SM limit it was found for
    size_t queuePad[2] = {};          // [feather variant]: the work-queue kernel's padding
    int queuePadFor = -1;             // the CTAs-per-SM limit it was found for
    // Stage timing (rive_cuda_set_profiling).
    bool profiling = false;
    std::vector<cudaEvent_t> eventPool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> stageEvents[RIVE_CUDA_STAGE_COUNT];
    cudaEvent_t openEvent = nullptr;
    int openStage = -1;
    // Last flush's texture extents (for debug read-backs).
    size_t lastTessBytes = 0, lastGradBytes = 0, lastAtlasBytes = 0;
};

// A batch captured as a CUDA graph (rive_cuda_graph_*): it owns every
// intermediate, so replays never allocate and never wait for the host.
struct rive_cuda_graph
{
    rive_cuda_context* ctx = nullptr;
    DeviceBuffer tables, tess, grad, tris, counts, masks, offsets, keys, vals, keysAlt, valsAlt,
        scanTemp, sortTemp, ranges, error, featherPlanes, pathGrids, gridWinding, gridEdge,
        gridCounters, queueKeys, queueVals, queueKeysAlt, queueValsAlt, queueTemp, queueCursor,
        atlas, pathImage;
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t* hError = nullptr; // pinned, 2 words
    uint32_t capacity = 0, measured = 0;
    rive_cuda_flush_stats stats = {};
};

namespace
{
int set_error(rive_cuda_context* ctx, int code, const char* fmt, ...)
{
    if (ctx)
    {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->lastError = buf;
    }
    return code;
}

int cuda_fail(rive_cuda_context* ctx, cudaError_t e, const char* what)
{
    return set_error(ctx, RIVE_CUDA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call)                                                                                   \
    do                                                                                             \
    {                                                                                              \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return cuda_fail(ctx, _e, #call);                                                      \
    } while (0)

uint32_t premul_rgba8(uint32_t argb)
{
    // UnpackColorToRGBA32FPremul followed by UNORM8 store.
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

cudaEvent_t pool_event(rive_cuda_context* ctx)
{
    if (!ctx->eventPool.empty())
    {
        cudaEvent_t e = ctx->eventPool.back();
        ctx->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void stage_begin(rive_cuda_context* ctx, int stage, cudaStream_t s)
{
    if (!ctx->profiling)
        return;
    ctx->openEvent = pool_event(ctx);
    ctx->openStage = stage;
    cudaEventRecord(ctx->openEvent, s);
}

void stage_end(rive_cuda_context* ctx, cudaStream_t s)
{
    if (!ctx->profiling || ctx->openStage < 0)
        return;
    cudaEvent_t e = pool_event(ctx);
    cudaEventRecord(e, s);
    ctx->stageEvents[ctx->openStage].push_back({ctx->openEvent, e});
    ctx->openStage = -1;
    ctx->openEvent = nullptr;
}

// The record buffers a flush reads, in buffer-kind order (flush uniforms ..
// triangle vertices, image draw instances).
constexpr int kResolvedKinds = 9;
struct ResolvedBuffers
{
    const void* ptr[kResolvedKinds];
    size_t bytes[kResolvedKinds];
};

// Caller-owned device buffers: sizes are the caller's; ranges come from desc.
ResolvedBuffers resolve_device_buffers(const rive_cuda_device_buffers& b)
{
    const void* p[kResolvedKinds] = {b.flush_uniforms, b.paths,      b.paints,
                                     b.paint_aux,      b.contours,   b.grad_spans,
                                     b.tess_spans,     b.triangle_vertices, b.image_draws};
    ResolvedBuffers rb;
    for (int k = 0; k < kResolvedKinds; ++k)
    {
        rb.ptr[k] = p[k];
        rb.bytes[k] = p[k] ? (size_t)-1 / 2 : 0;
    }
    return rb;
}

// One logical flush of a batch.
struct FlushInput
{
    const rive_cuda_flush_desc* d;
    ResolvedBuffers rb;
    uint32_t* fb;
};

// Set-up list of a draw type and the triangles one of its items makes.
int setup_list(uint32_t drawType)
{
    return drawType == DRAW_MIDPOINT_FAN_PATCHES  ? 0
           : drawType == DRAW_OUTER_CURVE_PATCHES ? 1
           : drawType == DRAW_INTERIOR_TRIANGULATION ? 2
           : drawType == DRAW_MIDPOINT_FAN_CENTER_AA_PATCHES ? 3
           : drawType == DRAW_FEATHER_ATLAS_BLIT ? 2 // a rectangle of triangle vertices
           : drawType == DRAW_IMAGE_MESH ? 2 // the mesh's triangles
                                                             : -1;
}
constexpr uint32_t kTrianglesPerItem[kSetupLists] = {
    kPatchTriangleCount, kOuterPatchTriangleCount, 1, kCenterPatchTriangleCount};

// The mesh of draw batch i of a flush, or null.
const rive_cuda_batch_mesh* batch_mesh(const rive_cuda_flush_desc* d, uint32_t i)
{
    return d->batch_meshes && d->batch_meshes[i].vertices ? &d->batch_meshes[i] : nullptr;
}

// Items (patch instances or triangles) of draw batch i of a flush.
uint32_t batch_items(const rive_cuda_flush_desc* d, uint32_t i)
{
    const rive_cuda_draw_batch& b = d->draw_batches[i];
    if (b.draw_type == DRAW_IMAGE_MESH)
    {
        const rive_cuda_batch_mesh* m = batch_mesh(d, i);
        return m ? m->index_count / 3 : 0u;
    }
    return b.draw_type == DRAW_INTERIOR_TRIANGULATION || b.draw_type == DRAW_FEATHER_ATLAS_BLIT
               ? b.element_count / 3
               : b.element_count;
}

// Atlas batch i of a flush: fill batches come first.
bool atlas_is_fill(const rive_cuda_flush_desc* d, uint32_t i) { return i < d->atlas_fill_batch_count; }
uint32_t atlas_batch_count(const rive_cuda_flush_desc* d)
{
    return d->atlas_fill_batch_count + d->atlas_stroke_batch_count;
}
// Whether the flush renders a feather atlas (content and batches).
bool has_atlas(const rive_cuda_flush_desc* d)
{
    return atlas_batch_count(d) != 0 && d->atlas_content_width != 0 &&
           d->atlas_content_height != 0;
}

// Host-side checks of one flush; counts its triangle slots.
int validate_flush(rive_cuda_context* ctx, const rive_cuda_flush_desc* d, const ResolvedBuffers& rb,
                   uint64_t& slots)
{
    if (d->interlock_mode != 0)
        return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED,
                         "interlock mode %u not supported (rasterOrdering only)", d->interlock_mode);
    if (d->render_target_width == 0 || d->render_target_height == 0)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "empty render target");
    if (d->render_target_width > 16384 || d->render_target_height > 16384)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "render target too large");
    if (d->draw_batch_count && !d->draw_batches)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "draw_batches is NULL");
    // Bounds of every record range this flush reads.
    struct
    {
        int kind;
        uint64_t first, count, elem;
    } checks[] = {
        {RIVE_CUDA_BUFFER_PATH, d->first_path, d->path_count, 64},
        {RIVE_CUDA_BUFFER_PAINT, d->first_paint, d->path_count, 8},
        {RIVE_CUDA_BUFFER_PAINT_AUX, d->first_paint_aux, d->path_count, 128},
        {RIVE_CUDA_BUFFER_CONTOUR, d->first_contour, d->contour_count, 16},
        {RIVE_CUDA_BUFFER_GRAD_SPAN, d->first_grad_span, d->grad_span_count, 16},
        {RIVE_CUDA_BUFFER_TESS_SPAN, d->first_tess_span, d->tess_span_count, 64},
    };
    for (auto& c : checks)
        if (c.count && (c.first + c.count) * c.elem > rb.bytes[c.kind])
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                             "buffer kind %d too small: need %llu bytes, have %zu", c.kind,
                             (unsigned long long)((c.first + c.count) * c.elem), rb.bytes[c.kind]);
    if ((uint64_t)d->flush_uniform_offset_bytes + 256 > rb.bytes[RIVE_CUDA_BUFFER_FLUSH_UNIFORM])
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush uniforms out of range");
    if (d->grad_data_height > 65536 || d->tess_data_height > 65536)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "texture height out of range");
    slots = 0;
    for (uint32_t i = 0; i < d->draw_batch_count; ++i)
    {
        const rive_cuda_draw_batch& b = d->draw_batches[i];
        const int list = setup_list(b.draw_type);
        if (list < 0)
            return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED, "draw type %u not supported",
                             b.draw_type);
        // ENABLE_FEATHER: feathered strokes draw in midpoint-fan batches,
        // feathered fills in center-AA midpoint-fan batches.
        if ((b.shader_features & SF_FEATHER) && b.draw_type != DRAW_MIDPOINT_FAN_PATCHES &&
            b.draw_type != DRAW_MIDPOINT_FAN_CENTER_AA_PATCHES &&
            b.draw_type != DRAW_FEATHER_ATLAS_BLIT)
            return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED,
                             "feathered draws of draw type %u not supported", b.draw_type);
        if (b.shader_misc_flags & ~MISC_CLOCKWISE_FILL)
            return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED,
                             "shader misc flags 0x%x not supported (rasterOrdering: clockwiseFill only)",
                             b.shader_misc_flags);
        if (b.draw_type == DRAW_IMAGE_MESH)
        {
            // An image mesh: its buffers, its ImageDrawInstance and its
            // texture (RiveRenderer::drawImageMesh draws nothing without one).
            const rive_cuda_batch_mesh* m = batch_mesh(d, i);
            if (!m || !m->uvs || !m->indices)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "image mesh batch %u has no vertex, uv or index buffer", i);
            if (m->index_count % 3 || (uint64_t)m->index_count * 2 > m->indices->bytes)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "image mesh batch %u: %u indices in a %zu-byte index buffer", i,
                                 m->index_count, m->indices->bytes);
            if (!d->batch_images || !d->batch_images[i].texture)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "image mesh batch %u has no texture", i);
            if (b.element_count != 1 || !rb.ptr[RIVE_CUDA_BUFFER_IMAGE_DRAW] ||
                ((uint64_t)b.base_element + 1) * 64 > rb.bytes[RIVE_CUDA_BUFFER_IMAGE_DRAW])
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "image mesh batch %u reads past the image draw instances", i);
            if (d->path_count == 0)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "a flush with image meshes has path 0 (the clear path)");
        }
        else if (list == 2)
        {
            if (b.element_count % 3 || !rb.ptr[RIVE_CUDA_BUFFER_TRIANGLE] ||
                ((uint64_t)b.base_element + b.element_count) * 12 >
                    rb.bytes[RIVE_CUDA_BUFFER_TRIANGLE])
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "batch %u reads past the triangle vertices", i);
        }
        else
        {
            const uint64_t span = list == 1 ? kOuterPatchSegmentSpan : kPatchSegmentSpan;
            if (((uint64_t)b.base_element + b.element_count) * span >
                (uint64_t)d->tess_data_height * kTessTextureWidth)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "batch %u reads past the tessellation texture", i);
        }
        slots += (uint64_t)batch_items(d, i) * kTrianglesPerItem[list];
    }
    // Images: a known sampler for every batch that samples a texture.
    if (d->batch_images)
        for (uint32_t i = 0; i < d->draw_batch_count; ++i)
            if (d->batch_images[i].texture && d->batch_images[i].sampler_key >= 18)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "batch %u has an unknown image sampler key %u", i,
                                 d->batch_images[i].sampler_key);
    // The feather atlas: its size, and every batch within the tessellation
    // texture and the atlas.
    const uint32_t na = atlas_batch_count(d);
    if (na)
    {
        if (!d->atlas_batches)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "atlas_batches is NULL");
        if (d->atlas_content_width > 16384 || d->atlas_content_height > 16384)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "feather atlas too large");
        for (uint32_t i = 0; i < na; ++i)
        {
            const rive_cuda_atlas_batch& a = d->atlas_batches[i];
            if (((uint64_t)a.base_patch + a.patch_count) * kPatchSegmentSpan >
                (uint64_t)d->tess_data_height * kTessTextureWidth)
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "atlas batch %u reads past the tessellation texture", i);
            if (a.scissor[0] > a.scissor[2] || a.scissor[1] > a.scissor[3])
                return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                                 "atlas batch %u has an inverted scissor", i);
            slots += (uint64_t)a.patch_count *
                     (atlas_is_fill(d, i) ? kCenterPatchTriangleCount : kPatchTriangleCount);
        }
    }
    return RIVE_CUDA_OK;
}

size_t align16(size_t n) { return (n + 15) & ~(size_t)15; }

// Host-side layout of a batch of independent logical flushes.
struct BatchLayout
{
    uint32_t n = 0;
    int tileLog2 = kTileLog2;
    uint32_t segCount[kSetupLists] = {}, items[kSetupLists] = {};
    uint32_t gradSpans = 0, tessSpans = 0, tiles = 0, slots = 0, paths = 0;
    // Feather atlases: one more scene per flush that renders one (after the
    // n main scenes), with its tiles after all the main ones.
    uint32_t atlasScenes = 0, mainTiles = 0;
    uint64_t atlasTexels = 0;
    std::vector<uint32_t> atlasScene; // per flush: its atlas scene, or ~0u
    std::vector<uint64_t> atlasTexel0; // per flush: its first atlas texel
    uint32_t scenes() const { return n + atlasScenes; }
    // Images: draw batches that sample a texture (slots of the batch's image
    // table), and the per-path image slots of every main scene.
    uint32_t imageSlots = 0;
    size_t oImages = 0;
    // Image meshes: the batch's mesh table.
    uint32_t meshes = 0;
    size_t oMeshes = 0;
    // Per-slot planes: feathered fills' third and fourth coverage
    // components, image meshes' texture coordinates.
    bool planes() const { return items[3] != 0 || meshes != 0; }
    // The extended kernel variants: some batch feathers, blits the feather
    // atlas or samples an image.
    bool feather = false;
    // Interior tiles as winding records for this batch: midpoint-fan patches
    // then take fanStride slots (their 24 triangles and a winding slot).
    bool winding = false;
    uint32_t fanStride = kPatchTriangleCount;
    uint64_t tessRows = 0, gradRows = 0;
    std::vector<uint64_t> tessRow0, gradRow0;
    // Table blob offsets.
    size_t oScenes = 0, oGradBase = 0, oTessBase = 0, oTileBase = 0, oSceneTiles = 0,
           oPathBase = 0, oSegments[kSetupLists] = {}, oSegBase[kSetupLists] = {}, tableBytes = 0;
    size_t tessBytes() const { return (size_t)kTessTextureWidth * tessRows * 16; }
    size_t gradBytes() const { return (size_t)kGradTextureWidth * gradRows * 4; }
    // Bin keys fit 16 bits (the sentinel key `tiles` included) without
    // winding entries, whose binner writes 32-bit keys.
    bool keys16() const { return tiles <= 0xffffu && !winding; }
    int endBit() const
    {
        int b = 1;
        while ((1ull << b) <= tiles) // room for the sentinel key `tiles`
            ++b;
        return b;
    }
};

// Validates the flushes and lays out their work.
int plan_batch(rive_cuda_context* ctx, const FlushInput* in, uint32_t n, BatchLayout& L)
{
    if (n == 0 || n > 65535)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "a batch holds 1 to 65535 flushes");
    L = BatchLayout();
    L.n = n;
    L.tileLog2 = ctx->tileLog2;
    const uint32_t ts = 1u << L.tileLog2;
    L.tessRow0.resize(n);
    L.gradRow0.resize(n);
    L.atlasScene.assign(n, ~0u);
    L.atlasTexel0.assign(n, 0);
    uint64_t slots = 0, tiles = 0, gradSpans = 0, tessSpans = 0, paths = 0;
    uint64_t segs[kSetupLists] = {}, items[kSetupLists] = {};
    for (uint32_t i = 0; i < n; ++i)
    {
        uint64_t fs = 0;
        int rc = validate_flush(ctx, in[i].d, in[i].rb, fs);
        if (rc)
            return rc;
        if (!in[i].fb)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush %u has no target", i);
        if (!in[i].rb.ptr[RIVE_CUDA_BUFFER_FLUSH_UNIFORM])
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush %u has no uniforms", i);
        const rive_cuda_flush_desc* d = in[i].d;
        slots += fs;
        for (uint32_t b = 0; b < d->draw_batch_count; ++b)
        {
            const rive_cuda_draw_batch& db = d->draw_batches[b];
            const uint32_t k = batch_items(d, b);
            if (!k)
                continue;
            const int list = setup_list(db.draw_type);
            segs[list] += 1;
            items[list] += k;
            if ((db.shader_features & SF_FEATHER) || db.draw_type == DRAW_FEATHER_ATLAS_BLIT)
                L.feather = true;
            if (db.draw_type == DRAW_IMAGE_MESH)
                ++L.meshes;
            if (d->batch_images && d->batch_images[b].texture)
            {
                ++L.imageSlots;
                L.feather = true; // the raster's extended variant samples images
            }
        }
        L.tessRow0[i] = L.tessRows;
        L.gradRow0[i] = L.gradRows;
        L.tessRows += std::max(d->tess_data_height, 1u);
        L.gradRows += std::max(d->grad_data_height, 1u);
        tiles += (uint64_t)((d->render_target_width + ts - 1) / ts) *
                 ((d->render_target_height + ts - 1) / ts);
        gradSpans += d->grad_span_count;
        tessSpans += d->tess_span_count;
        paths += d->path_count;
    }
    L.mainTiles = (uint32_t)std::min<uint64_t>(tiles, 0xffffffffu);
    for (uint32_t i = 0; i < n; ++i)
    {
        const rive_cuda_flush_desc* d = in[i].d;
        if (!has_atlas(d))
            continue;
        L.atlasScene[i] = n + L.atlasScenes++;
        L.atlasTexel0[i] = L.atlasTexels;
        L.atlasTexels += (uint64_t)d->atlas_content_width * d->atlas_content_height;
        tiles += (uint64_t)((d->atlas_content_width + ts - 1) / ts) *
                 ((d->atlas_content_height + ts - 1) / ts);
        L.feather = true;
        for (uint32_t b = 0; b < atlas_batch_count(d); ++b)
        {
            const uint32_t k = d->atlas_batches[b].patch_count;
            if (!k)
                continue;
            const int list = atlas_is_fill(d, b) ? 3 : 0;
            segs[list] += 1;
            items[list] += k;
        }
    }
    if (L.scenes() > 65535)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                         "a batch holds at most 65535 flushes and feather atlases");
    // Winding records for the interior tiles of fills: on unless turned off
    // or the batch feathers (feathered batches keep their fans).
    L.winding = ctx->windingTiles && !L.feather && items[0] > 0;
    if (L.winding)
    {
        L.fanStride = kPatchTriangleCount + 1;
        slots += items[0]; // one winding slot per midpoint-fan patch
    }
    if (slots > 0xffffffffull || tiles >= 0x7fffffffull || gradSpans > 0x7fffffffull ||
        tessSpans * 32 > 0xffffffffull || paths > 0x7fffffffull)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "batch too large");
    L.paths = (uint32_t)paths;
    if (n > 1)
    {
        // The flushes of one batch run concurrently: each needs its own target.
        std::vector<const uint32_t*> fbs(n);
        for (uint32_t i = 0; i < n; ++i)
            fbs[i] = in[i].fb;
        std::sort(fbs.begin(), fbs.end());
        if (std::adjacent_find(fbs.begin(), fbs.end()) != fbs.end())
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                             "two flushes of one batch share a render target");
    }
    for (int l = 0; l < kSetupLists; ++l)
    {
        L.segCount[l] = (uint32_t)segs[l];
        L.items[l] = (uint32_t)items[l];
    }
    L.gradSpans = (uint32_t)gradSpans;
    L.tessSpans = (uint32_t)tessSpans;
    L.tiles = (uint32_t)tiles;
    L.slots = (uint32_t)slots;
    const uint32_t ns = L.scenes();
    L.oScenes = 0;
    L.oGradBase = align16(L.oScenes + sizeof(FlushParams) * ns);
    L.oTessBase = align16(L.oGradBase + 4 * (ns + 1));
    L.oTileBase = align16(L.oTessBase + 4 * (ns + 1));
    L.oSceneTiles = align16(L.oTileBase + 4 * (ns + 1));
    L.oPathBase = align16(L.oSceneTiles + 8 * ns);
    L.oImages = align16(L.oPathBase + 4 * (ns + 1));
    L.oMeshes = align16(L.oImages + sizeof(ImageTex) * std::max(L.imageSlots, 1u));
    size_t o = align16(L.oMeshes + sizeof(MeshDesc) * std::max(L.meshes, 1u));
    for (int l = 0; l < kSetupLists; ++l)
    {
        L.oSegments[l] = o;
        L.oSegBase[l] = align16(o + sizeof(PatchSegment) * std::max<uint64_t>(segs[l], 1));
        o = align16(L.oSegBase[l] + 4 * (segs[l] + 1));
    }
    L.tableBytes = o;
    return RIVE_CUDA_OK;
}

// Device pointers of a batch's intermediates.
struct Scratch
{
    uint8_t* tables = nullptr; // device copy of the table blob
    uint4* tess = nullptr;
    uchar4* grad = nullptr;
    TriRecord* tris = nullptr;
    uint32_t* counts = nullptr;
    uint8_t* masks = nullptr;    // per slot: tiles overlapped, for boxes of <= 8 tiles
    uint32_t* offsets = nullptr; // slots + 1 entries
    // Bin keys: tile indices, 16-bit when keys16 (set by reserve_bins).
    void *keys = nullptr, *keysAlt = nullptr;
    uint32_t *vals = nullptr, *valsAlt = nullptr;
    bool keys16 = false;
    void* scanTemp = nullptr;
    size_t scanTempBytes = 0;
    void* sortTemp = nullptr;
    size_t sortTempBytes = 0;
    uint2* ranges = nullptr;
    uint32_t* error = nullptr;
    // Where the binner reports entries past the bins' capacity (error when
    // null; a scratch word for speculative passes, whose overflow is
    // handled by re-running the back half).
    uint32_t* binError = nullptr;
    float4* featherPlanes = nullptr; // 2 per slot, only with center-AA patches
    uint16_t* atlas = nullptr;       // the batch's feather atlases, fp16 texels
    uint32_t* pathImage = nullptr;   // per path of the batch: its image slot
    // Winding grids (only when the batch draws interior tiles as winding
    // records).
    PathGrid* pathGrids = nullptr;
    int32_t* gridWinding = nullptr;
    uint8_t* gridEdge = nullptr;
    uint32_t* gridCounters = nullptr;
    uint32_t gridCapacity = 0;
    // Work-queue raster: the tile order (sorted keys/values and their
    // alternates), the sort's temporaries and the cursor.
    uint32_t *qKeys = nullptr, *qVals = nullptr, *qKeysAlt = nullptr, *qValsAlt = nullptr;
    uint32_t* qCursor = nullptr;
    void* qTemp = nullptr;
    size_t qTempBytes = 0;
};

// Fills the table blob (host memory) and returns the device view of it.
BatchTables write_tables(rive_cuda_context* ctx,
                         const FlushInput* in,
                         const BatchLayout& L,
                         const Scratch& S,
                         uint8_t* h)
{
    auto* scenes = (FlushParams*)(h + L.oScenes);
    auto* gradBase = (uint32_t*)(h + L.oGradBase);
    auto* tessBase = (uint32_t*)(h + L.oTessBase);
    auto* tileBase = (uint32_t*)(h + L.oTileBase);
    auto* sceneTiles = (uint2*)(h + L.oSceneTiles);
    auto* pathBase = (uint32_t*)(h + L.oPathBase);
    auto* images = (ImageTex*)(h + L.oImages);
    auto* meshes = (MeshDesc*)(h + L.oMeshes);
    uint32_t imageAcc = 0, meshAcc = 0;
    PatchSegment* segs[kSetupLists];
    uint32_t* segBase[kSetupLists];
    for (int l = 0; l < kSetupLists; ++l)
    {
        segs[l] = (PatchSegment*)(h + L.oSegments[l]);
        segBase[l] = (uint32_t*)(h + L.oSegBase[l]);
    }
    uint32_t gAcc = 0, tAcc = 0, tileAcc = 0, slotAcc = 0, pathAcc = 0;
    uint32_t segAcc[kSetupLists] = {}, itemAcc[kSetupLists] = {};
    for (uint32_t i = 0; i < L.n; ++i)
    {
        const rive_cuda_flush_desc* d = in[i].d;
        const ResolvedBuffers& rb = in[i].rb;
        FlushParams& P = scenes[i];
        memset(&P, 0, sizeof(P));
        P.paths = (const uint4*)rb.ptr[RIVE_CUDA_BUFFER_PATH];
        P.paints = (const uint2*)rb.ptr[RIVE_CUDA_BUFFER_PAINT];
        P.paintAux = (const float4*)rb.ptr[RIVE_CUDA_BUFFER_PAINT_AUX];
        P.contours = (const uint4*)rb.ptr[RIVE_CUDA_BUFFER_CONTOUR];
        P.gradSpans = (const uint4*)rb.ptr[RIVE_CUDA_BUFFER_GRAD_SPAN];
        P.tessSpans = (const uint4*)rb.ptr[RIVE_CUDA_BUFFER_TESS_SPAN];
        P.uniforms = (const uint8_t*)rb.ptr[RIVE_CUDA_BUFFER_FLUSH_UNIFORM] +
                     d->flush_uniform_offset_bytes;
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
        P.gradTextureHeight = d->grad_texture_height                ? d->grad_texture_height
                              : (L.n == 1 && ctx->gradHeight != 0u) ? ctx->gradHeight
                                                                    : d->grad_data_height;
        P.tessDataHeight = d->tess_data_height;
        P.width = d->render_target_width;
        P.height = d->render_target_height;
        P.wireframe = d->wireframe;
        P.loadClear = d->color_load_action == RIVE_CUDA_LOAD_CLEAR;
        P.clearColorPremulRGBA = premul_rgba8(d->color_clear_value);
        P.pathIDGranularity = 1; // replaced on the device by scene_uniforms_kernel
        P.error = S.error;
        P.fb = in[i].fb;
        const uint32_t ts = 1u << L.tileLog2;
        P.tilesX = (d->render_target_width + ts - 1) / ts;
        P.tess = S.tess + (size_t)L.tessRow0[i] * kTessTextureWidth;
        P.grad = S.grad + (size_t)L.gradRow0[i] * kGradTextureWidth;
        P.triangleVertices = (const uint32_t*)rb.ptr[RIVE_CUDA_BUFFER_TRIANGLE];
        P.triangleVertexCount = (uint32_t)std::min<size_t>(rb.bytes[RIVE_CUDA_BUFFER_TRIANGLE] / 12,
                                                           0xffffffffu);
        if (L.atlasScene[i] != ~0u)
        {
            P.atlas = S.atlas + L.atlasTexel0[i];
            P.atlasW = d->atlas_content_width;
            P.atlasH = d->atlas_content_height;
        }
        if (L.imageSlots)
        {
            P.images = (const ImageTex*)(S.tables + L.oImages);
            P.pathImage = S.pathImage + pathAcc;
        }
        P.imageDraws = (const float4*)rb.ptr[RIVE_CUDA_BUFFER_IMAGE_DRAW];
        P.imageDrawCount = (uint32_t)std::min<size_t>(rb.bytes[RIVE_CUDA_BUFFER_IMAGE_DRAW] / 64,
                                                      0xffffffffu);

        gradBase[i] = gAcc;
        tessBase[i] = tAcc;
        tileBase[i] = tileAcc;
        pathBase[i] = pathAcc;
        pathAcc += d->path_count;
        sceneTiles[i] = make_uint2(tileAcc, P.tilesX);
        gAcc += d->grad_span_count;
        tAcc += d->tess_span_count;
        tileAcc += P.tilesX * ((d->render_target_height + ts - 1) / ts);
        // Slots follow the draw list order across all the set-up lists.
        for (uint32_t b = 0; b < d->draw_batch_count; ++b)
        {
            const rive_cuda_draw_batch& db = d->draw_batches[b];
            const uint32_t k = batch_items(d, b);
            if (!k)
                continue;
            const int l = setup_list(db.draw_type);
            uint32_t image = kNoImage;
            if (d->batch_images && d->batch_images[b].texture)
            {
                image = imageAcc++;
                images[image] = d->batch_images[b].texture->desc;
                images[image].sampler = d->batch_images[b].sampler_key;
            }
            uint32_t mesh = kNoMesh;
            if (db.draw_type == DRAW_IMAGE_MESH)
            {
                const rive_cuda_batch_mesh& m = *batch_mesh(d, b);
                mesh = meshAcc++;
                MeshDesc& M = meshes[mesh];
                M.positions = (const float2*)m.vertices->mem;
                M.uvs = (const float2*)m.uvs->mem;
                M.indices = (const uint16_t*)m.indices->mem;
                M.vertexCount = (uint32_t)std::min<size_t>(
                    std::min(m.vertices->bytes, m.uvs->bytes) / 8, 0xffffffffu);
                M.indexCount = m.index_count;
                M.imageDraw = db.base_element;
                M.image = image;
                M.pad = 0;
            }
            segs[l][segAcc[l]] = PatchSegment{
                i, db.base_element,
                db.shader_features |
                    ((db.shader_misc_flags & MISC_CLOCKWISE_FILL) ? FEATURE_CLOCKWISE_FILL : 0u) |
                    (db.draw_type == DRAW_FEATHER_ATLAS_BLIT ? FEATURE_ATLAS_BLIT : 0u) |
                    (db.draw_type == DRAW_IMAGE_MESH ? FEATURE_IMAGE_MESH : 0u),
                slotAcc, 0u, 0xffffffffu, image, mesh};
            segBase[l][segAcc[l]] = itemAcc[l];
            ++segAcc[l];
            itemAcc[l] += k;
            slotAcc += k * (l == 0 ? L.fanStride : kTrianglesPerItem[l]);
        }
    }
    // The feather atlases: per flush that renders one, a scene whose canvas
    // is the atlas content and whose set-up segments are the atlas batches
    // (center-AA fans for fills, midpoint fans for strokes; fills first),
    // each clipped to its scissor. Its slots follow all the main ones.
    for (uint32_t i = 0; i < L.n; ++i)
    {
        const uint32_t j = L.atlasScene[i];
        if (j == ~0u)
            continue;
        const rive_cuda_flush_desc* d = in[i].d;
        FlushParams& A = scenes[j];
        A = scenes[i];
        A.width = d->atlas_content_width;
        A.height = d->atlas_content_height;
        A.fb = nullptr;
        A.loadClear = 0;
        A.gradSpanCount = 0;
        A.tessSpanCount = 0;
        A.atlasMode = 1;
        A.images = nullptr;
        A.pathImage = nullptr;
        const uint32_t ts = 1u << L.tileLog2;
        A.tilesX = (A.width + ts - 1) / ts;
        gradBase[j] = gAcc;
        tessBase[j] = tAcc;
        tileBase[j] = tileAcc;
        pathBase[j] = pathAcc;
        sceneTiles[j] = make_uint2(tileAcc, A.tilesX);
        tileAcc += A.tilesX * ((A.height + ts - 1) / ts);
        for (uint32_t b = 0; b < atlas_batch_count(d); ++b)
        {
            const rive_cuda_atlas_batch& ab = d->atlas_batches[b];
            if (!ab.patch_count)
                continue;
            const int l = atlas_is_fill(d, b) ? 3 : 0;
            segs[l][segAcc[l]] = PatchSegment{
                j, ab.base_patch, SF_FEATHER, slotAcc,
                (uint32_t)ab.scissor[0] | ((uint32_t)ab.scissor[1] << 16),
                (uint32_t)ab.scissor[2] | ((uint32_t)ab.scissor[3] << 16), kNoImage, kNoMesh};
            segBase[l][segAcc[l]] = itemAcc[l];
            ++segAcc[l];
            itemAcc[l] += ab.patch_count;
            slotAcc += ab.patch_count * (l == 0 ? L.fanStride : kTrianglesPerItem[l]);
        }
    }
    const uint32_t ns = L.scenes();
    gradBase[ns] = gAcc;
    tessBase[ns] = tAcc;
    tileBase[ns] = tileAcc;
    pathBase[ns] = pathAcc;
    for (int l = 0; l < kSetupLists; ++l)
        segBase[l][segAcc[l]] = itemAcc[l];

    BatchTables B = {};
    const uint8_t* dT = S.tables;
    B.scenes = (const FlushParams*)(dT + L.oScenes);
    B.gradSpanBase = (const uint32_t*)(dT + L.oGradBase);
    B.tessSpanBase = (const uint32_t*)(dT + L.oTessBase);
    B.tileBase = (const uint32_t*)(dT + L.oTileBase);
    B.sceneTiles = (const uint2*)(dT + L.oSceneTiles);
    for (int l = 0; l < kSetupLists; ++l)
    {
        B.segments[l] = (const PatchSegment*)(dT + L.oSegments[l]);
        B.segBase[l] = (const uint32_t*)(dT + L.oSegBase[l]);
        B.segCount[l] = segAcc[l];
        B.totalItems[l] = itemAcc[l];
    }
    B.sceneCount = ns;
    B.mainTiles = L.mainTiles;
    B.tileLog2 = L.tileLog2;
    B.featherPlanes = S.featherPlanes;
    B.meshes = L.meshes ? (const MeshDesc*)(dT + L.oMeshes) : nullptr;
    B.fanSlotStride = L.fanStride;
    B.pathBase = (const uint32_t*)(dT + L.oPathBase);
    if (L.winding)
    {
        B.grids = S.pathGrids;
        B.gridWinding = S.gridWinding;
        B.gridEdge = S.gridEdge;
        B.gridCapacity = S.gridCapacity;
        B.gridCounters = S.gridCounters;
    }
    B.totalGradSpans = gAcc;
    B.totalTessSpans = tAcc;
    B.totalTiles = tileAcc;
    return B;
}

// Enqueues the passes up to and including the scan of tile counts (so
// S.offsets[L.slots] holds the batch's bin-entry total on the device).
int enqueue_front(rive_cuda_context* ctx,
                  const BatchLayout& L,
                  const BatchTables& B,
                  const Scratch& S,
                  cudaStream_t stream)
{
    scene_uniforms_kernel<<<(L.scenes() + 127) / 128, 128, 0, stream>>>(
        const_cast<FlushParams*>(B.scenes), L.scenes());
    // Texels no span covers are never sampled; zero them so the gradient
    // texture is deterministic.
    CK(cudaMemsetAsync(S.grad, 0, L.gradBytes(), stream));
    CK(cudaMemsetAsync(S.ranges, 0, (size_t)L.tiles * sizeof(uint2), stream));
    if (L.imageSlots)
        CK(cudaMemsetAsync(S.pathImage, 0xff, (size_t)std::max(L.paths, 1u) * 4, stream));
    if (L.winding)
    {
        // Winding grids: every path's box and eligibility, its box from the
        // spans' control points, then its place in the (zeroed) cell pool.
        CK(cudaMemsetAsync(S.gridWinding, 0, (size_t)S.gridCapacity * 4, stream));
        CK(cudaMemsetAsync(S.gridEdge, 0, S.gridCapacity, stream));
        CK(cudaMemsetAsync(S.gridCounters, 0, 8, stream));
        path_init_kernel<<<(L.paths + 255) / 256, 256, 0, stream>>>(B);
        if (L.tessSpans)
            path_bounds_kernel<<<(L.tessSpans + 255) / 256, 256, 0, stream>>>(B);
        path_alloc_kernel<<<(L.paths + 255) / 256, 256, 0, stream>>>(B);
    }
    if (L.gradSpans)
    {
        stage_begin(ctx, RIVE_CUDA_STAGE_COLOR_RAMP, stream);
        color_ramp_kernel<<<L.gradSpans, 128, 0, stream>>>(B);
        stage_end(ctx, stream);
    }
    if (L.tessSpans)
    {
        stage_begin(ctx, RIVE_CUDA_STAGE_TESSELLATE, stream);
        (L.feather ? tessellate_feather_kernel : tessellate_kernel)<<<(L.tessSpans * 32u + 255u) / 256u,
                                                                     256, 0, stream>>>(B);
        stage_end(ctx, stream);
    }
    if (L.slots)
    {
        stage_begin(ctx, RIVE_CUDA_STAGE_PATCH_SETUP, stream);
        if (L.items[0])
            (L.feather   ? patch_setup_feather_kernel
             : L.winding ? patch_setup_winding_kernel
                         : patch_setup_kernel)<<<(L.items[0] + 3) / 4, 128, 0, stream>>>(
                B, S.tris, S.counts, S.masks);
        if (L.items[1])
            outer_setup_kernel<<<(L.items[1] + 3) / 4, 128, 0, stream>>>(B, S.tris, S.counts,
                                                                         S.masks);
        if (L.items[2])
            interior_setup_kernel<<<(L.items[2] + 255) / 256, 256, 0, stream>>>(B, S.tris, S.counts,
                                                                                S.masks);
        if (L.items[3])
            center_setup_kernel<<<(L.items[3] + 3) / 4, 128, 0, stream>>>(B, S.tris, S.counts,
                                                                          S.masks);
        if (L.winding)
        {
            // The deferred fan triangles' winding deltas and edge tiles, then
            // the windings of every path's grid.
            fan_filter_kernel<<<(L.items[0] * 8u + 255u) / 256u, 256, 0, stream>>>(B, S.tris,
                                                                                   S.counts, S.masks);
            path_winding_kernel<<<(L.paths + 7) / 8, 256, 0, stream>>>(B, S.counts);
        }
        stage_end(ctx, stream);
        stage_begin(ctx, RIVE_CUDA_STAGE_BIN, stream);
        size_t tempBytes = S.scanTempBytes;
        CK(cudaMemsetAsync(S.offsets, 0, 4, stream));
        CK(cub::DeviceScan::InclusiveSum(S.scanTemp, tempBytes, S.counts, S.offsets + 1, L.slots,
                                         stream));
        stage_end(ctx, stream);
    }
    return RIVE_CUDA_OK;
}

// Dynamic shared memory (unused) that holds a raster kernel to at most
// `ctas` resident CTAs per SM, found with the occupancy calculator.
size_t occupancy_pad(const void* fn, int threads, int ctas)
{
    constexpr size_t kMaxPad = 160u << 10;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxPad) !=
        cudaSuccess)
        return 0;
    for (size_t dyn = 0; dyn <= kMaxPad; dyn += 256)
    {
        int occ = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, dyn) != cudaSuccess)
            return 0;
        if (occ <= ctas)
            return dyn;
    }
    return 0;
}

// Sets the kernel attributes and finds the padding the context's raster
// configuration needs. Called before any stream capture, never inside one.
int prepare_raster(rive_cuda_context* ctx)
{
    if (ctx->tileLog2 == 5 && !ctx->raster32Ready)
    {
        CK(cudaFuncSetAttribute(raster_tile32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                kRaster32SmemBytes));
        CK(cudaFuncSetAttribute(raster_tile32_feather_kernel,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, kRaster32SmemBytes));
        ctx->raster32Ready = true;
    }
    if (ctx->rasterQueue && ctx->smCount == 0)
    {
        CK(cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, ctx->device));
        const void* q[2] = {(const void*)raster_queue_kernel,
                            (const void*)raster_queue_feather_kernel};
        for (int f = 0; f < 2; ++f)
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctx->queueCtas[f], q[f], 256, 0));
    }
    const int slot = ctx->tileLog2 == 3 ? 0 : ctx->tileLog2 == 4 ? 1 : -1;
    if (slot >= 0 && ctx->rasterCtasPerSm > 0 && ctx->rasterPadFor[slot] != ctx->rasterCtasPerSm)
    {
        const void* fns[2][2] = {
            {(const void*)raster_tile8_kernel, (const void*)raster_tile_kernel},
            {(const void*)raster_tile8_feather_kernel, (const void*)raster_tile_feather_kernel}};
        for (int f = 0; f < 2; ++f)
            ctx->rasterPad[f][slot] =
                occupancy_pad(fns[f][slot], slot == 0 ? 64 : 256, ctx->rasterCtasPerSm);
        cudaGetLastError(); // a failed query only leaves the launch unpadded
        ctx->rasterPadFor[slot] = ctx->rasterCtasPerSm;
    }
    if (ctx->rasterQueue && ctx->rasterCtasPerSm > 0 && ctx->queuePadFor != ctx->rasterCtasPerSm)
    {
        // The queue kernels have their own static shared memory, so their own
        // padding (and their own dynamic shared memory limit, set there).
        const void* q[2] = {(const void*)raster_queue_kernel,
                            (const void*)raster_queue_feather_kernel};
        for (int f = 0; f < 2; ++f)
            ctx->queuePad[f] = occupancy_pad(q[f], 256, ctx->rasterCtasPerSm);
        cudaGetLastError();
        ctx->queuePadFor = ctx->rasterCtasPerSm;
    }
    return RIVE_CUDA_OK;
}

// Launches the raster for the batch's tile size (prepare_raster has run). A
// CTAs-per-SM limit is applied by asking each CTA for more (unused) dynamic
// shared memory.
int launch_raster(rive_cuda_context* ctx,
                  const BatchLayout& L,
                  const BatchTables& B,
                  const Scratch& S,
                  const TriRecord* tris,
                  const uint32_t* sortedSlots,
                  const uint2* ranges,
                  cudaStream_t stream)
{
    if (L.tileLog2 == 4 && S.qCursor)
    {
        // The work queue: tiles sorted by bin entries, heaviest first, taken
        // in turn by a persistent grid of resident CTAs.
        tile_order_keys_kernel<<<(L.mainTiles + 255) / 256, 256, 0, stream>>>(L.mainTiles, ranges,
                                                                            S.qKeys, S.qVals);
        cub::DoubleBuffer<uint32_t> k(S.qKeys, S.qKeysAlt), v(S.qVals, S.qValsAlt);
        size_t tb = S.qTempBytes;
        CK(cub::DeviceRadixSort::SortPairs(S.qTemp, tb, k, v, (int)L.mainTiles, 0, 32, stream));
        CK(cudaMemsetAsync(S.qCursor, 0, 4, stream));
        const size_t dyn = ctx->rasterCtasPerSm > 0 ? ctx->queuePad[L.feather] : 0;
        const int per = ctx->rasterCtasPerSm > 0 ? ctx->rasterCtasPerSm : ctx->queueCtas[L.feather];
        const uint32_t grid =
            std::min<uint32_t>(L.mainTiles, (uint32_t)std::max(per * ctx->smCount, 1));
        (L.feather ? raster_queue_feather_kernel : raster_queue_kernel)<<<grid, 256, dyn, stream>>>(
            B, tris, sortedSlots, ranges, v.Current(), S.qCursor, L.mainTiles);
        return RIVE_CUDA_OK;
    }
    if (L.tileLog2 == 3)
    {
        const size_t dyn = ctx->rasterCtasPerSm > 0 ? ctx->rasterPad[L.feather][0] : 0;
        (L.feather ? raster_tile8_feather_kernel : raster_tile8_kernel)<<<L.mainTiles, 64, dyn,
                                                                           stream>>>(
            B, tris, sortedSlots, ranges);
    }
    else if (L.tileLog2 == 5)
    {
        (L.feather ? raster_tile32_feather_kernel : raster_tile32_kernel)<<<
            L.mainTiles, 1024, kRaster32SmemBytes, stream>>>(B, tris, sortedSlots, ranges);
    }
    else
    {
        const size_t dyn = ctx->rasterCtasPerSm > 0 ? ctx->rasterPad[L.feather][1] : 0;
        (L.feather ? raster_tile_feather_kernel : raster_tile_kernel)<<<L.mainTiles, 256, dyn,
                                                                         stream>>>(
            B, tris, sortedSlots, ranges);
    }
    return RIVE_CUDA_OK;
}

// Enqueues binning, sort, ranges and raster over `entries` bin slots. With
// `padded`, entries is a fixed capacity: the tail past the device's total is
// filled with the sentinel key and overflow is flagged on the device.
int enqueue_back(rive_cuda_context* ctx,
                 const BatchLayout& L,
                 const BatchTables& B,
                 const Scratch& S,
                 uint32_t entries,
                 bool padded,
                 cudaStream_t stream,
                 bool guarded = false)
{
    uint32_t* const binError = S.binError ? S.binError : S.error;
    const uint32_t* sortedSlots = nullptr;
    if (entries && L.slots)
    {
        stage_begin(ctx, RIVE_CUDA_STAGE_BIN, stream);
        if (S.keys16)
        {
            uint16_t* keys = (uint16_t*)S.keys;
            if (padded)
                bin_fill16_kernel<<<(entries + 255) / 256, 256, 0, stream>>>(
                    S.offsets + L.slots, entries, L.tiles, keys);
            bin_scatter16_kernel<<<(L.slots + 255) / 256, 256, 0, stream>>>(
                L.slots, L.tileLog2, B.sceneTiles, S.tris, S.counts, S.masks, S.offsets, entries,
                binError, keys, S.vals);
        }
        else
        {
            uint32_t* keys = (uint32_t*)S.keys;
            if (padded)
                bin_fill_kernel<<<(entries + 255) / 256, 256, 0, stream>>>(
                    S.offsets + L.slots, entries, L.tiles, keys);
            if (L.winding)
                bin_scatter_winding_kernel<<<(L.slots + 255) / 256, 256, 0, stream>>>(
                    B, S.tris, S.counts, S.masks, S.offsets, L.slots, entries, binError, keys,
                    S.vals);
            else
                bin_scatter_kernel<<<(L.slots + 255) / 256, 256, 0, stream>>>(
                    L.slots, L.tileLog2, B.sceneTiles, S.tris, S.counts, S.masks, S.offsets, entries,
                    binError, keys, S.vals);
        }
        stage_end(ctx, stream);
        cub::DoubleBuffer<uint32_t> v(S.vals, S.valsAlt);
        size_t tempBytes = S.sortTempBytes;
        stage_begin(ctx, RIVE_CUDA_STAGE_SORT, stream);
        if (S.keys16)
        {
            cub::DoubleBuffer<uint16_t> k((uint16_t*)S.keys, (uint16_t*)S.keysAlt);
            CK(cub::DeviceRadixSort::SortPairs(S.sortTemp, tempBytes, k, v, (int)entries, 0,
                                               L.endBit(), stream));
            tile_ranges16_kernel<<<(entries + 255) / 256, 256, 0, stream>>>(entries, L.tiles,
                                                                          k.Current(), S.ranges);
        }
        else
        {
            cub::DoubleBuffer<uint32_t> k((uint32_t*)S.keys, (uint32_t*)S.keysAlt);
            CK(cub::DeviceRadixSort::SortPairs(S.sortTemp, tempBytes, k, v, (int)entries, 0,
                                               L.endBit(), stream));
            tile_ranges_kernel<<<(entries + 255) / 256, 256, 0, stream>>>(entries, L.tiles,
                                                                        k.Current(), S.ranges);
        }
        // A speculative pass whose total did not fit: every range emptied,
        // so the raster leaves the target as it was (or clears it) until the
        // back half runs again with exact bins.
        if (guarded)
            ranges_guard_kernel<<<(L.tiles + 255) / 256, 256, 0, stream>>>(S.offsets + L.slots,
                                                                          entries, S.ranges,
                                                                          L.tiles);
        stage_end(ctx, stream);
        sortedSlots = v.Current();
    }
    stage_begin(ctx, RIVE_CUDA_STAGE_RASTER, stream);
    if (L.tiles > L.mainTiles)
    {
        // The feather atlases first: the main raster's blits sample them.
        const uint32_t atlasTiles = L.tiles - L.mainTiles;
        if (L.tileLog2 == 3)
            raster_atlas8_kernel<<<atlasTiles, 64, 0, stream>>>(B, S.tris, sortedSlots, S.ranges,
                                                                L.mainTiles);
        else if (L.tileLog2 == 5)
            raster_atlas32_kernel<<<atlasTiles, 1024, 0, stream>>>(B, S.tris, sortedSlots,
                                                                   S.ranges, L.mainTiles);
        else
            raster_atlas_kernel<<<atlasTiles, 256, 0, stream>>>(B, S.tris, sortedSlots, S.ranges,
                                                                L.mainTiles);
    }
    if (ctx->rasterWait)
        CK(cudaStreamWaitEvent(stream, ctx->rasterWait, 0));
    int rc = launch_raster(ctx, L, B, S, S.tris, sortedSlots, S.ranges, stream);
    stage_end(ctx, stream);
    if (rc)
        return rc;
    CK(cudaGetLastError());
    return RIVE_CUDA_OK;
}

size_t scan_temp_bytes(uint32_t slots)
{
    size_t b = 0;
    cub::DeviceScan::InclusiveSum(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                  std::max(slots, 1u));
    return b;
}

// Temporary bytes of the work queue's sort of `tiles` tile indices.
size_t queue_temp_bytes(uint32_t tiles)
{
    size_t b = 0;
    cub::DoubleBuffer<uint32_t> k(nullptr, nullptr), v(nullptr, nullptr);
    cub::DeviceRadixSort::SortPairs(nullptr, b, k, v, (int)std::max(tiles, 1u), 0, 32);
    return b;
}

size_t sort_temp_bytes(uint32_t entries, int endBit, bool keys16 = false)
{
    size_t b = 0;
    cub::DoubleBuffer<uint32_t> v(nullptr, nullptr);
    if (keys16)
    {
        cub::DoubleBuffer<uint16_t> k(nullptr, nullptr);
        cub::DeviceRadixSort::SortPairs(nullptr, b, k, v, (int)std::max(entries, 1u), 0, endBit);
    }
    else
    {
        cub::DoubleBuffer<uint32_t> k(nullptr, nullptr);
        cub::DeviceRadixSort::SortPairs(nullptr, b, k, v, (int)std::max(entries, 1u), 0, endBit);
    }
    return b;
}

// Runs a batch of independent logical flushes (distinct targets) as one
// sequence of launches: every stage covers the work of all flushes at once.
// The bin-entry total is read back after the scan, so bins are sized exactly.
// The flush whose back half ran on speculative bins and whose bin-entry total
// has not been checked yet (at most one per context).
struct PendingFlush
{
    BatchLayout L;
    BatchTables B;
    Scratch S;
    uint32_t capacity = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t counted = nullptr;
    bool active = false;
    // Read-backs enqueued after it, to enqueue again after a re-run.
    std::vector<std::pair<rive_cuda_render_target*, void*>> reads;
};

// Reserves the sort keys/values and sort temporaries for `entries` bin
// entries and points S at them.
int reserve_bins(rive_cuda_context* ctx, const BatchLayout& L, uint32_t entries, Scratch& S)
{
    S.keys16 = L.keys16();
    const size_t keyBytes = S.keys16 ? 2 : 4;
    CK(ctx->keys.reserve((size_t)entries * keyBytes));
    CK(ctx->vals.reserve((size_t)entries * 4));
    CK(ctx->keysAlt.reserve((size_t)entries * keyBytes));
    CK(ctx->valsAlt.reserve((size_t)entries * 4));
    S.sortTempBytes = sort_temp_bytes(entries, L.endBit(), S.keys16);
    CK(ctx->sortTemp.reserve(S.sortTempBytes));
    S.keys = ctx->keys.ptr;
    S.vals = (uint32_t*)ctx->vals.ptr;
    S.keysAlt = ctx->keysAlt.ptr;
    S.valsAlt = (uint32_t*)ctx->valsAlt.ptr;
    S.sortTemp = ctx->sortTemp.ptr;
    return RIVE_CUDA_OK;
}

// Checks the pending speculative flush, if any: waits for its scanned total
// and, when the total did not fit its bins (the guarded raster then left the
// target untouched), runs its back half again with exact bins and repeats
// the read-backs enqueued after it. Every call that enqueues work on the
// context, reads its results or changes its configuration settles first.
int settle_pending(rive_cuda_context* ctx)
{
    PendingFlush* p = ctx->pending;
    if (!p || !p->active)
        return RIVE_CUDA_OK;
    p->active = false;
    CK(cudaSetDevice(ctx->device));
    CK(cudaEventSynchronize(p->counted));
    const uint32_t total = *ctx->hSpecTotal;
    ctx->binHighWater = std::max(ctx->binHighWater, total);
    ctx->stats.bin_entries = total;
    if (total > p->capacity)
    {
        // Read-backs already on the read stream finish first: the re-run
        // rewrites their target, and its own read-backs land after them.
        cudaEvent_t readsDone = nullptr;
        CK(cudaEventCreateWithFlags(&readsDone, cudaEventDisableTiming));
        CK(cudaEventRecord(readsDone, ctx->readStream));
        CK(cudaStreamWaitEvent(p->stream, readsDone, 0));
        CK(cudaEventDestroy(readsDone));
        Scratch S = p->S;
        S.binError = nullptr;
        int rc = reserve_bins(ctx, p->L, total, S);
        if (!rc)
            rc = enqueue_back(ctx, p->L, p->B, S, total, false, p->stream);
        if (!rc && ctx->lastDone)
        {
            CK(cudaEventRecord(ctx->lastDone, p->stream));
            ctx->lastStream = p->stream;
        }
        for (auto& r : p->reads)
            if (!rc)
            {
                cudaError_t e =
                    cudaMemcpyAsync(r.second, r.first->pixels,
                                    (size_t)r.first->width * r.first->height * 4,
                                    cudaMemcpyDeviceToHost, p->stream);
                if (e != cudaSuccess)
                    rc = cuda_fail(ctx, e, "read-back after a re-run");
            }
        p->reads.clear();
        return rc;
    }
    p->reads.clear();
    return RIVE_CUDA_OK;
}

int run_batch_body(rive_cuda_context* ctx,
                   const FlushInput* in,
                   uint32_t n,
                   cudaStream_t stream,
                   bool speculative)
{
    BatchLayout L;
    int rc = plan_batch(ctx, in, n, L);
    if (!rc)
        rc = prepare_raster(ctx);
    if (rc)
        return rc;
    // The staging slot's last tables may still be in flight.
    const int tslot = ctx->tableSlot;
    ctx->tableSlot = (tslot + 1) % rive_cuda_context::kTableRing;
    if (ctx->tablesCopied[tslot])
        CK(cudaEventSynchronize(ctx->tablesCopied[tslot]));
    CK(ctx->tess.reserve(L.tessBytes()));
    CK(ctx->grad.reserve(L.gradBytes()));
    CK(ctx->hTables[tslot].reserve(L.tableBytes));
    CK(ctx->dTables.reserve(L.tableBytes));
    CK(ctx->ranges.reserve((size_t)L.tiles * sizeof(uint2)));
    CK(ctx->tris.reserve((size_t)std::max(L.slots, 1u) * sizeof(TriRecord)));
    CK(ctx->tileCounts.reserve((size_t)std::max(L.slots, 1u) * 4));
    CK(ctx->tileMasks.reserve((size_t)std::max(L.slots, 1u)));
    CK(ctx->offsets.reserve((size_t)L.slots * 4 + 4));
    if (L.planes())
        CK(ctx->featherPlanes.reserve((size_t)L.slots * 2 * sizeof(float4)));
    if (L.atlasTexels)
        CK(ctx->atlas.reserve((size_t)L.atlasTexels * 2));
    if (L.imageSlots)
        CK(ctx->pathImage.reserve((size_t)std::max(L.paths, 1u) * 4));
    if (L.winding)
    {
        // The cell pool starts at four cells per tile of the batch and grows
        // to what the last flush asked for (cells past it leave those paths
        // on their fans).
        if (ctx->gridCapacity < L.tiles * 4u)
            ctx->gridCapacity = std::max(L.tiles * 4u, 1u << 16);
        CK(ctx->pathGrids.reserve((size_t)std::max(L.paths, 1u) * sizeof(PathGrid)));
        CK(ctx->gridWinding.reserve((size_t)ctx->gridCapacity * 4));
        CK(ctx->gridEdge.reserve(ctx->gridCapacity));
        CK(ctx->gridCounters.reserve(8));
    }
    const bool queue = ctx->rasterQueue && L.tileLog2 == 4;
    size_t queueBytes = 0;
    if (queue)
    {
        queueBytes = queue_temp_bytes(L.tiles);
        for (DeviceBuffer* b : {&ctx->queueKeys, &ctx->queueVals, &ctx->queueKeysAlt,
                                &ctx->queueValsAlt})
            CK(b->reserve((size_t)L.tiles * 4));
        CK(ctx->queueTemp.reserve(queueBytes));
        CK(ctx->queueCursor.reserve(4));
    }
    const size_t scanBytes = scan_temp_bytes(L.slots);
    CK(ctx->scanTemp.reserve(scanBytes));
    ctx->lastTessBytes = (size_t)kTessTextureWidth * std::max(in[0].d->tess_data_height, 1u) * 16;
    ctx->lastGradBytes = (size_t)kGradTextureWidth * std::max(in[0].d->grad_data_height, 1u) * 4;
    ctx->lastAtlasBytes = L.atlasScene[0] != ~0u ? (size_t)in[0].d->atlas_content_width *
                                                       in[0].d->atlas_content_height * 2
                                                 : 0;

    Scratch S;
    S.tables = (uint8_t*)ctx->dTables.ptr;
    S.tess = (uint4*)ctx->tess.ptr;
    S.grad = (uchar4*)ctx->grad.ptr;
    S.tris = (TriRecord*)ctx->tris.ptr;
    S.featherPlanes = L.planes() ? (float4*)ctx->featherPlanes.ptr : nullptr;
    S.atlas = L.atlasTexels ? (uint16_t*)ctx->atlas.ptr : nullptr;
    S.pathImage = L.imageSlots ? (uint32_t*)ctx->pathImage.ptr : nullptr;
    S.counts = (uint32_t*)ctx->tileCounts.ptr;
    S.masks = (uint8_t*)ctx->tileMasks.ptr;
    S.offsets = (uint32_t*)ctx->offsets.ptr;
    S.scanTemp = ctx->scanTemp.ptr;
    S.scanTempBytes = scanBytes;
    S.ranges = (uint2*)ctx->ranges.ptr;
    S.error = ctx->dError;
    if (L.winding)
    {
        S.pathGrids = (PathGrid*)ctx->pathGrids.ptr;
        S.gridWinding = (int32_t*)ctx->gridWinding.ptr;
        S.gridEdge = (uint8_t*)ctx->gridEdge.ptr;
        S.gridCounters = (uint32_t*)ctx->gridCounters.ptr;
        S.gridCapacity = ctx->gridCapacity;
    }
    if (queue)
    {
        S.qKeys = (uint32_t*)ctx->queueKeys.ptr;
        S.qVals = (uint32_t*)ctx->queueVals.ptr;
        S.qKeysAlt = (uint32_t*)ctx->queueKeysAlt.ptr;
        S.qValsAlt = (uint32_t*)ctx->queueValsAlt.ptr;
        S.qTemp = ctx->queueTemp.ptr;
        S.qTempBytes = queueBytes;
        S.qCursor = (uint32_t*)ctx->queueCursor.ptr;
    }
    BatchTables B = write_tables(ctx, in, L, S, (uint8_t*)ctx->hTables[tslot].ptr);
    CK(cudaMemcpyAsync(S.tables, ctx->hTables[tslot].ptr, L.tableBytes, cudaMemcpyHostToDevice,
                       stream));
    if (!ctx->tablesCopied[tslot])
        CK(cudaEventCreateWithFlags(&ctx->tablesCopied[tslot], cudaEventDisableTiming));
    CK(cudaEventRecord(ctx->tablesCopied[tslot], stream));

    rc = enqueue_front(ctx, L, B, S, stream);
    if (rc)
        return rc;
    // Speculative bins: a single flush on the context's stream, once a total
    // has been seen, without winding records (their cell counts are read
    // back too).
    if (speculative && ctx->speculate && n == 1 && L.slots && !L.winding && ctx->binHighWater)
    {
        if (!ctx->pending)
        {
            ctx->pending = new (std::nothrow) PendingFlush();
            if (!ctx->pending)
                return RIVE_CUDA_ERR_OUT_OF_MEMORY;
            CK(cudaEventCreateWithFlags(&ctx->pending->counted, cudaEventDisableTiming));
        }
        PendingFlush& p = *ctx->pending;
        const uint64_t cap = (uint64_t)ctx->binHighWater + ctx->binHighWater / 4 + 4096;
        p.capacity = (uint32_t)std::min<uint64_t>(cap, 0x7fffffffu);
        rc = reserve_bins(ctx, L, p.capacity, S);
        if (rc)
            return rc;
        S.binError = ctx->dSpecOverflow;
        CK(cudaMemcpyAsync(ctx->hSpecTotal, S.offsets + L.slots, 4, cudaMemcpyDeviceToHost,
                           stream));
        CK(cudaEventRecord(p.counted, stream));
        rc = enqueue_back(ctx, L, B, S, p.capacity, true, stream, true);
        if (rc)
            return rc;
        p.L = L;
        p.B = B;
        p.S = S;
        p.stream = stream;
        p.reads.clear();
        p.active = true;
        ctx->stats.tess_vertices = (uint64_t)L.tessRows * kTessTextureWidth;
        ctx->stats.patches = (uint64_t)L.items[0] + L.items[1] + L.items[3];
        ctx->stats.triangles = L.slots;
        ctx->stats.bin_entries = 0; // known when the flush settles
        ctx->stats.winding_entries = 0;
        ctx->stats.tiles = L.tiles;
        ctx->stats.kernel_launches = 1 + (L.gradSpans ? 1 : 0) + (L.tessSpans ? 1 : 0) + 1 + 5 +
                                     1 + (L.tiles > L.mainTiles ? 1 : 0);
        return RIVE_CUDA_OK;
    }
    uint32_t pairs = 0, windingEntries = 0;
    if (L.slots)
    {
        CK(cudaMemcpyAsync(ctx->hPairs, S.offsets + L.slots, 4, cudaMemcpyDeviceToHost, stream));
        if (L.winding)
            CK(cudaMemcpyAsync(ctx->hGridCounters, S.gridCounters, 8, cudaMemcpyDeviceToHost,
                               stream));
        CK(cudaStreamSynchronize(stream));
        pairs = *ctx->hPairs;
        ctx->binHighWater = std::max(ctx->binHighWater, pairs);
        if (L.winding)
        {
            windingEntries = ctx->hGridCounters[1];
            const uint32_t asked = ctx->hGridCounters[0];
            if (asked > ctx->gridCapacity)
                ctx->gridCapacity = asked + asked / 4; // for the next flush
        }
    }
    if (pairs)
    {
        rc = reserve_bins(ctx, L, pairs, S);
        if (rc)
            return rc;
    }
    rc = enqueue_back(ctx, L, B, S, pairs, false, stream);
    if (rc)
        return rc;
    ctx->stats.tess_vertices = (uint64_t)L.tessRows * kTessTextureWidth;
    ctx->stats.patches = (uint64_t)L.items[0] + L.items[1] + L.items[3];
    ctx->stats.triangles = L.slots;
    ctx->stats.bin_entries = pairs;
    ctx->stats.winding_entries = windingEntries;
    ctx->stats.tiles = L.tiles;
    ctx->stats.kernel_launches = 1 + (L.gradSpans ? 1 : 0) + (L.tessSpans ? 1 : 0) +
                                 (L.slots ? 1 : 0) + (pairs ? 3 : 0) + 1 +
                                 (L.tiles > L.mainTiles ? 1 : 0) +
                                 (L.winding ? 3 + (L.tessSpans ? 1 : 0) + 1 : 0);
    return RIVE_CUDA_OK;
}

// Runs a batch in order after the context's previous one: the flushes of one
// context share its intermediates (tessellation texture, triangle records,
// bins), so a batch on another stream waits for the last one's work first.
int run_batch(rive_cuda_context* ctx,
              const FlushInput* in,
              uint32_t n,
              cudaStream_t stream,
              bool speculative = false)
{
    if (n == 0)
        return RIVE_CUDA_OK;
    if (const int rc = settle_pending(ctx))
        return rc;
    if (ctx->lastDone && ctx->lastStream != stream)
        CK(cudaStreamWaitEvent(stream, ctx->lastDone, 0));
    const int rc = run_batch_body(ctx, in, n, stream, speculative);
    if (!ctx->lastDone)
        CK(cudaEventCreateWithFlags(&ctx->lastDone, cudaEventDisableTiming));
    CK(cudaEventRecord(ctx->lastDone, stream));
    ctx->lastStream = stream;
    return rc;
}

// Flushes into caller-given device memory cannot tell a target with a
// read-back in flight: while any is, their stream waits for the read stream.
int order_after_reads(rive_cuda_context* ctx, cudaStream_t s)
{
    if (!ctx->readsInFlight)
        return RIVE_CUDA_OK;
    cudaEvent_t ev = nullptr;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, ctx->readStream));
    CK(cudaStreamWaitEvent(s, ev, 0));
    CK(cudaEventDestroy(ev));
    return RIVE_CUDA_OK;
}

int run_flush(rive_cuda_context* ctx,
              const rive_cuda_flush_desc* d,
              const ResolvedBuffers& rb,
              uint32_t* fbDevice,
              cudaStream_t stream,
              bool speculative = false)
{
    FlushInput in{d, rb, fbDevice};
    return run_batch(ctx, &in, 1, stream, speculative);
}
} // namespace

extern "C" {

int rive_cuda_context_create(int device, rive_cuda_context** out_ctx)
{
    if (!out_ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out_ctx = nullptr;
    rive_cuda_context* ctx = new (std::nothrow) rive_cuda_context();
    if (!ctx)
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->copyStream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&ctx->readStream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&ctx->dError, 4);
    if (e == cudaSuccess)
        e = cudaMemset(ctx->dError, 0, 4);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->hError, 4);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->hPairs, 4);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->hGridCounters, 8);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->hSpecTotal, 4);
    if (e == cudaSuccess)
        e = cudaMalloc(&ctx->dSpecOverflow, 4);
    if (e == cudaSuccess)
        e = ensure_feather_lut(device);
    if (e != cudaSuccess)
    {
        fprintf(stderr, "rive_cuda_context_create: %s\n", cudaGetErrorString(e));
        rive_cuda_context_destroy(ctx);
        return RIVE_CUDA_ERR_CUDA;
    }
    *out_ctx = ctx;
    return RIVE_CUDA_OK;
}

void rive_cuda_context_destroy(rive_cuda_context* ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    settle_pending(ctx);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    if (ctx->copyStream)
        cudaStreamSynchronize(ctx->copyStream);
    if (ctx->readStream)
        cudaStreamSynchronize(ctx->readStream);
    if (ctx->pending)
    {
        if (ctx->pending->counted)
            cudaEventDestroy(ctx->pending->counted);
        delete ctx->pending;
    }
    if (ctx->hSpecTotal)
        cudaFreeHost(ctx->hSpecTotal);
    if (ctx->dSpecOverflow)
        cudaFree(ctx->dSpecOverflow);
    for (auto& r : ctx->rings)
    {
        for (int i = 0; i < kRingSize; ++i)
        {
            if (r.host[i])
                cudaFreeHost(r.host[i]);
            if (r.done[i])
                cudaEventDestroy(r.done[i]);
        }
        for (int i = 0; i < 2; ++i)
        {
            r.device[i].release();
            if (r.readDone[i])
                cudaEventDestroy(r.readDone[i]);
            if (r.copied[i])
                cudaEventDestroy(r.copied[i]);
        }
    }
    for (DeviceBuffer* b : {&ctx->tess, &ctx->grad, &ctx->tris, &ctx->tileCounts, &ctx->tileMasks,
                            &ctx->offsets, &ctx->featherPlanes,
                            &ctx->keys, &ctx->vals, &ctx->keysAlt, &ctx->valsAlt,
                            &ctx->sortTemp, &ctx->scanTemp, &ctx->ranges, &ctx->dTables,
                            &ctx->pathGrids, &ctx->gridWinding, &ctx->gridEdge,
                            &ctx->gridCounters, &ctx->queueKeys, &ctx->queueVals,
                            &ctx->queueKeysAlt, &ctx->queueValsAlt, &ctx->queueTemp,
                            &ctx->queueCursor, &ctx->atlas, &ctx->pathImage})
        b->release();
    for (int i = 0; i < rive_cuda_context::kTableRing; ++i)
    {
        ctx->hTables[i].release();
        if (ctx->tablesCopied[i])
            cudaEventDestroy(ctx->tablesCopied[i]);
    }
    if (ctx->hGridCounters)
        cudaFreeHost(ctx->hGridCounters);
    if (ctx->dError)
        cudaFree(ctx->dError);
    if (ctx->hError)
        cudaFreeHost(ctx->hError);
    if (ctx->hPairs)
        cudaFreeHost(ctx->hPairs);
    for (auto& v : ctx->stageEvents)
        for (auto& pr : v)
        {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    for (cudaEvent_t e : ctx->eventPool)
        cudaEventDestroy(e);
    if (ctx->stream)
        cudaStreamDestroy(ctx->stream);
    if (ctx->copyStream)
        cudaStreamDestroy(ctx->copyStream);
    if (ctx->readStream)
        cudaStreamDestroy(ctx->readStream);
    if (ctx->lastDone)
        cudaEventDestroy(ctx->lastDone);
    delete ctx;
}

int rive_cuda_last_error(const rive_cuda_context* ctx, char* buf, size_t len)
{
    if (!ctx || !buf || !len)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    snprintf(buf, len, "%s", ctx->lastError.c_str());
    return RIVE_CUDA_OK;
}

int rive_cuda_resize_buffer(rive_cuda_context* ctx, int kind, size_t bytes)
{
    if (!ctx || kind < 0 || kind >= RIVE_CUDA_BUFFER_KIND_COUNT)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "bad buffer kind %d", kind);
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    RecordRing& r = ctx->rings[kind];
    if (r.mapped)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "resize while mapped");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaStreamSynchronize(ctx->copyStream));
    for (int i = 0; i < kRingSize; ++i)
    {
        if (r.host[i])
            cudaFreeHost(r.host[i]);
        r.host[i] = nullptr;
    }
    r.capacity = 0;
    for (int i = 0; i < 2; ++i)
    {
        r.device[i].release();
        r.deviceValidBytes[i] = 0;
        if (!r.readDone[i])
            CK(cudaEventCreateWithFlags(&r.readDone[i], cudaEventDisableTiming));
        if (!r.copied[i])
            CK(cudaEventCreateWithFlags(&r.copied[i], cudaEventDisableTiming));
    }
    r.slot = 0;
    r.used = false;
    if (bytes == 0)
        return RIVE_CUDA_OK;
    for (int i = 0; i < kRingSize; ++i)
    {
        cudaError_t e = cudaHostAlloc(&r.host[i], bytes, cudaHostAllocWriteCombined);
        if (e != cudaSuccess)
            return set_error(ctx, RIVE_CUDA_ERR_OUT_OF_MEMORY, "pinned alloc of %zu bytes: %s", bytes,
                             cudaGetErrorString(e));
        if (!r.done[i])
            CK(cudaEventCreateWithFlags(&r.done[i], cudaEventDisableTiming));
    }
    for (int i = 0; i < 2; ++i)
        if (r.device[i].reserve(bytes) != cudaSuccess)
            return set_error(ctx, RIVE_CUDA_ERR_OUT_OF_MEMORY, "device alloc of %zu bytes", bytes);
    r.capacity = bytes;
    return RIVE_CUDA_OK;
}

void* rive_cuda_map_buffer(rive_cuda_context* ctx, int kind, size_t bytes)
{
    if (!ctx || kind < 0 || kind >= RIVE_CUDA_BUFFER_KIND_COUNT)
        return nullptr;
    RecordRing& r = ctx->rings[kind];
    if (r.mapped || bytes == 0 || bytes > r.capacity)
    {
        set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "map of %zu bytes (capacity %zu)", bytes,
                  r.capacity);
        return nullptr;
    }
    r.current = (r.current + 1) % kRingSize;
    // The ring slot may still be the source of an in-flight upload.
    if (cudaEventSynchronize(r.done[r.current]) != cudaSuccess)
    {
        set_error(ctx, RIVE_CUDA_ERR_CUDA, "ring wait failed");
        return nullptr;
    }
    r.mapped = true;
    return r.host[r.current];
}

int rive_cuda_unmap_buffer(rive_cuda_context* ctx, int kind, size_t bytes)
{
    if (!ctx || kind < 0 || kind >= RIVE_CUDA_BUFFER_KIND_COUNT)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "bad buffer kind %d", kind);
    RecordRing& r = ctx->rings[kind];
    if (!r.mapped)
        return set_error(ctx, RIVE_CUDA_ERR_NOT_MAPPED, "unmap of an unmapped buffer");
    r.mapped = false;
    if (bytes > r.capacity)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "unmap size too large");
    CK(cudaSetDevice(ctx->device));
    if (r.used)
    {
        // The current copy feeds flushes in flight: fill the other one once
        // the flushes that read it last are done.
        r.slot ^= 1;
        r.used = false;
        CK(cudaStreamWaitEvent(ctx->copyStream, r.readDone[r.slot], 0));
    }
    if (bytes)
        CK(cudaMemcpyAsync(r.device[r.slot].ptr, r.host[r.current], bytes, cudaMemcpyHostToDevice,
                           ctx->copyStream));
    CK(cudaEventRecord(r.done[r.current], ctx->copyStream));
    CK(cudaEventRecord(r.copied[r.slot], ctx->copyStream));
    r.deviceValidBytes[r.slot] = bytes;
    return RIVE_CUDA_OK;
}

int rive_cuda_resize_gradient_texture(rive_cuda_context* ctx, uint32_t width, uint32_t height)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    if (width && width != (uint32_t)kGradTextureWidth)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "gradient texture width must be 512");
    ctx->gradWidth = width;
    ctx->gradHeight = height;
    CK(cudaSetDevice(ctx->device));
    CK(ctx->grad.reserve((size_t)kGradTextureWidth * std::max(height, 1u) * 4));
    return RIVE_CUDA_OK;
}

int rive_cuda_resize_tessellation_texture(rive_cuda_context* ctx, uint32_t width, uint32_t height)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    if (width && width != (uint32_t)kTessTextureWidth)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                         "tessellation texture width must be 2048");
    ctx->tessWidth = width;
    ctx->tessHeight = height;
    CK(cudaSetDevice(ctx->device));
    CK(ctx->tess.reserve((size_t)kTessTextureWidth * std::max(height, 1u) * 16));
    return RIVE_CUDA_OK;
}

int rive_cuda_render_target_create(rive_cuda_context* ctx,
                                   uint32_t width,
                                   uint32_t height,
                                   rive_cuda_render_target** out)
{
    if (!ctx || !out || !width || !height || width > 16384 || height > 16384)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "bad render target size");
    *out = nullptr;
    auto* t = new (std::nothrow) rive_cuda_render_target();
    if (!t)
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    t->width = width;
    t->height = height;
    CK(cudaSetDevice(ctx->device));
    cudaError_t e = cudaMalloc(&t->pixels, (size_t)width * height * 4);
    if (e != cudaSuccess)
    {
        delete t;
        return cuda_fail(ctx, e, "render target alloc");
    }
    e = cudaMemset(t->pixels, 0, (size_t)width * height * 4);
    if (e != cudaSuccess)
    {
        cudaFree(t->pixels);
        delete t;
        return cuda_fail(ctx, e, "render target clear");
    }
    *out = t;
    return RIVE_CUDA_OK;
}

void rive_cuda_render_target_destroy(rive_cuda_context* ctx, rive_cuda_render_target* t)
{
    // A pending flush that may run again could still read it.
    if (ctx)
        settle_pending(ctx);
    if (!t)
        return;
    if (ctx)
    {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        cudaStreamSynchronize(ctx->readStream);
    }
    if (t->readDone)
        cudaEventDestroy(t->readDone);
    cudaFree(t->pixels);
    delete t;
}

void* rive_cuda_render_target_device_ptr(rive_cuda_render_target* t)
{
    return t ? t->pixels : nullptr;
}

int rive_cuda_render_target_read(rive_cuda_context* ctx,
                                 rive_cuda_render_target* t,
                                 void* dst,
                                 void* cuda_stream)
{
    if (!ctx || !t || !dst)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "bad read-back arguments");
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(dst, t->pixels, (size_t)t->width * t->height * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return RIVE_CUDA_OK;
}

int rive_cuda_render_target_read_async(rive_cuda_context* ctx,
                                        rive_cuda_render_target* t,
                                        void* dst,
                                        void* cuda_stream)
{
    if (!ctx || !t || !dst)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "bad read-back arguments");
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    // Behind a pending speculative flush on the same stream the copy is
    // enqueued at once and repeated should that flush run again; on another
    // stream the flush is settled first.
    const bool behindPending = ctx->pending && ctx->pending->active && ctx->pending->stream == s;
    if (!behindPending)
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    CK(cudaSetDevice(ctx->device));
    if (s == ctx->stream)
    {
        // On the read stream, after the flushes queued so far: the context's
        // stream goes on with the next flush's front half meanwhile, and only
        // the next raster into this target waits for the copy.
        if (!t->readDone)
            CK(cudaEventCreateWithFlags(&t->readDone, cudaEventDisableTiming));
        CK(cudaEventRecord(t->readDone, s));
        CK(cudaStreamWaitEvent(ctx->readStream, t->readDone, 0));
        CK(cudaMemcpyAsync(dst, t->pixels, (size_t)t->width * t->height * 4,
                           cudaMemcpyDeviceToHost, ctx->readStream));
        CK(cudaEventRecord(t->readDone, ctx->readStream));
        t->readPending = true;
        ctx->readsInFlight = true;
    }
    else
    {
        CK(cudaMemcpyAsync(dst, t->pixels, (size_t)t->width * t->height * 4,
                           cudaMemcpyDeviceToHost, s));
    }
    if (behindPending)
        ctx->pending->reads.emplace_back(t, dst);
    return RIVE_CUDA_OK;
}

int rive_cuda_flush(rive_cuda_context* ctx,
                    const rive_cuda_flush_desc* desc,
                    rive_cuda_render_target* target,
                    void* cuda_stream)
{
    if (!ctx || !desc || !target)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "NULL argument to flush");
    if (desc->render_target_width != target->width || desc->render_target_height != target->height)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "render target size mismatch");
    CK(cudaSetDevice(ctx->device));
    // A pending speculative flush settles first, so a re-run of it is queued
    // before anything this flush waits for.
    if (const int src = settle_pending(ctx))
        return src;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    if (s != ctx->stream)
    {
        // Work already queued on the context stream (texture and render
        // buffer uploads, earlier flushes) comes first.
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CK(cudaEventRecord(ev, ctx->stream));
        CK(cudaStreamWaitEvent(s, ev, 0));
        CK(cudaEventDestroy(ev));
    }
    ResolvedBuffers rb;
    for (int k = 0; k < kResolvedKinds; ++k)
    {
        RecordRing& r = ctx->rings[k];
        rb.ptr[k] = r.device[r.slot].ptr;
        rb.bytes[k] = r.deviceValidBytes[r.slot];
        if (r.copied[r.slot])
            CK(cudaStreamWaitEvent(s, r.copied[r.slot], 0));
    }
    // A read-back of this target still in flight: the raster waits for it.
    ctx->rasterWait = target->readPending ? target->readDone : nullptr;
    target->readPending = false;
    const int rc = run_flush(ctx, desc, rb, target->pixels, s, s == ctx->stream);
    ctx->rasterWait = nullptr;
    // The next upload of each kind goes to its other copy, after this flush.
    for (int k = 0; k < kResolvedKinds; ++k)
    {
        RecordRing& r = ctx->rings[k];
        if (r.readDone[r.slot])
        {
            CK(cudaEventRecord(r.readDone[r.slot], s));
            r.used = true;
        }
    }
    return rc;
}

int rive_cuda_flush_device(rive_cuda_context* ctx,
                           const rive_cuda_flush_desc* desc,
                           const rive_cuda_device_buffers* buffers,
                           void* target_pixels_device,
                           void* cuda_stream)
{
    if (!ctx || !desc || !buffers || !target_pixels_device)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "NULL argument to flush_device");
    CK(cudaSetDevice(ctx->device));
    const ResolvedBuffers rb = resolve_device_buffers(*buffers);
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    if (const int rc = order_after_reads(ctx, s))
        return rc;
    return run_flush(ctx, desc, rb, (uint32_t*)target_pixels_device, s);
}

namespace
{
void graph_free(rive_cuda_graph* g)
{
    if (g->exec)
        cudaGraphExecDestroy(g->exec);
    if (g->graph)
        cudaGraphDestroy(g->graph);
    for (DeviceBuffer* b : {&g->tables, &g->tess, &g->grad, &g->tris, &g->counts, &g->masks, &g->offsets,
                            &g->keys, &g->vals, &g->keysAlt, &g->valsAlt, &g->scanTemp,
                            &g->sortTemp, &g->ranges, &g->error, &g->featherPlanes,
                            &g->pathGrids, &g->gridWinding, &g->gridEdge, &g->gridCounters,
                            &g->queueKeys, &g->queueVals, &g->queueKeysAlt, &g->queueValsAlt,
                            &g->queueTemp, &g->queueCursor, &g->atlas, &g->pathImage})
        b->release();
    if (g->hError)
        cudaFreeHost(g->hError);
    if (g->stream)
        cudaStreamDestroy(g->stream);
    delete g;
}

int graph_build(rive_cuda_context* ctx,
                rive_cuda_graph* g,
                const FlushInput* in,
                uint32_t n,
                uint32_t capacity)
{
    BatchLayout L;
    int rc = plan_batch(ctx, in, n, L);
    if (rc)
        return rc;
    CK(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    CK(cudaMallocHost(&g->hError, 8)); // status word; cells the grids asked for
    CK(g->tables.reserve(L.tableBytes));
    CK(g->tess.reserve(L.tessBytes()));
    CK(g->grad.reserve(L.gradBytes()));
    CK(g->tris.reserve((size_t)std::max(L.slots, 1u) * sizeof(TriRecord)));
    CK(g->counts.reserve((size_t)std::max(L.slots, 1u) * 4));
    CK(g->masks.reserve((size_t)std::max(L.slots, 1u)));
    CK(g->offsets.reserve((size_t)L.slots * 4 + 4));
    if (L.planes())
        CK(g->featherPlanes.reserve((size_t)L.slots * 2 * sizeof(float4)));
    if (L.atlasTexels)
        CK(g->atlas.reserve((size_t)L.atlasTexels * 2));
    if (L.imageSlots)
        CK(g->pathImage.reserve((size_t)std::max(L.paths, 1u) * 4));
    CK(g->ranges.reserve((size_t)L.tiles * sizeof(uint2)));
    CK(g->error.reserve(4));
    const bool queue = ctx->rasterQueue && L.tileLog2 == 4;
    size_t queueBytes = 0;
    if (queue)
    {
        queueBytes = queue_temp_bytes(L.tiles);
        for (DeviceBuffer* b : {&g->queueKeys, &g->queueVals, &g->queueKeysAlt, &g->queueValsAlt})
            CK(b->reserve((size_t)L.tiles * 4));
        CK(g->queueTemp.reserve(queueBytes));
        CK(g->queueCursor.reserve(4));
    }
    const size_t scanBytes = scan_temp_bytes(L.slots);
    CK(g->scanTemp.reserve(scanBytes));
    CK(cudaMemset(g->error.ptr, 0, 4));

    Scratch S;
    S.tables = (uint8_t*)g->tables.ptr;
    S.tess = (uint4*)g->tess.ptr;
    S.grad = (uchar4*)g->grad.ptr;
    S.tris = (TriRecord*)g->tris.ptr;
    S.featherPlanes = L.planes() ? (float4*)g->featherPlanes.ptr : nullptr;
    S.atlas = L.atlasTexels ? (uint16_t*)g->atlas.ptr : nullptr;
    S.pathImage = L.imageSlots ? (uint32_t*)g->pathImage.ptr : nullptr;
    S.counts = (uint32_t*)g->counts.ptr;
    S.masks = (uint8_t*)g->masks.ptr;
    S.offsets = (uint32_t*)g->offsets.ptr;
    S.scanTemp = g->scanTemp.ptr;
    S.scanTempBytes = scanBytes;
    S.ranges = (uint2*)g->ranges.ptr;
    S.error = (uint32_t*)g->error.ptr;
    if (queue)
    {
        S.qKeys = (uint32_t*)g->queueKeys.ptr;
        S.qVals = (uint32_t*)g->queueVals.ptr;
        S.qKeysAlt = (uint32_t*)g->queueKeysAlt.ptr;
        S.qValsAlt = (uint32_t*)g->queueValsAlt.ptr;
        S.qTemp = g->queueTemp.ptr;
        S.qTempBytes = queueBytes;
        S.qCursor = (uint32_t*)g->queueCursor.ptr;
    }
    std::vector<uint8_t> h(L.tableBytes);
    // The graph's winding grids: a cell pool sized like the context's, grown
    // below if the measuring run asks for more.
    uint32_t gridCap = L.winding ? std::max({ctx->gridCapacity, L.tiles * 4u, 1u << 16}) : 0u;
    auto placeGrids = [&]() -> cudaError_t {
        if (!L.winding)
            return cudaSuccess;
        cudaError_t e = g->pathGrids.reserve((size_t)std::max(L.paths, 1u) * sizeof(PathGrid));
        if (e == cudaSuccess)
            e = g->gridWinding.reserve((size_t)gridCap * 4);
        if (e == cudaSuccess)
            e = g->gridEdge.reserve(gridCap);
        if (e == cudaSuccess)
            e = g->gridCounters.reserve(8);
        S.pathGrids = (PathGrid*)g->pathGrids.ptr;
        S.gridWinding = (int32_t*)g->gridWinding.ptr;
        S.gridEdge = (uint8_t*)g->gridEdge.ptr;
        S.gridCounters = (uint32_t*)g->gridCounters.ptr;
        S.gridCapacity = gridCap;
        return e;
    };
    CK(placeGrids());
    BatchTables B = write_tables(ctx, in, L, S, h.data());
    CK(cudaMemcpy(S.tables, h.data(), L.tableBytes, cudaMemcpyHostToDevice));

    const bool profiling = ctx->profiling;
    ctx->profiling = false; // stage events are not recorded inside a graph
    if (capacity == 0 && L.slots)
    {
        // Size the bins from one run of the front half: the exact total plus
        // an eighth of headroom for records that change between launches.
        // (The grids' cells too, with one more run if the pool was short.)
        for (int pass = 0; pass < 2; ++pass)
        {
            rc = enqueue_front(ctx, L, B, S, g->stream);
            if (rc)
            {
                ctx->profiling = profiling;
                return rc;
            }
            CK(cudaMemcpyAsync(g->hError, S.offsets + L.slots, 4, cudaMemcpyDeviceToHost,
                               g->stream));
            g->hError[1] = 0;
            if (L.winding)
                CK(cudaMemcpyAsync(g->hError + 1, S.gridCounters, 4, cudaMemcpyDeviceToHost,
                                   g->stream));
            CK(cudaStreamSynchronize(g->stream));
            g->measured = g->hError[0];
            const uint32_t asked = g->hError[1];
            if (asked <= gridCap)
                break;
            gridCap = asked + asked / 8;
            CK(placeGrids());
            B = write_tables(ctx, in, L, S, h.data());
            CK(cudaMemcpy(S.tables, h.data(), L.tableBytes, cudaMemcpyHostToDevice));
        }
        capacity = g->measured + g->measured / 8 + 4096;
    }
    if (!L.slots)
        capacity = 0;
    g->capacity = capacity;
    if (capacity)
    {
        for (DeviceBuffer* b : {&g->keys, &g->vals, &g->keysAlt, &g->valsAlt})
            CK(b->reserve((size_t)capacity * 4));
        S.keys = (uint32_t*)g->keys.ptr;
        S.vals = (uint32_t*)g->vals.ptr;
        S.keysAlt = (uint32_t*)g->keysAlt.ptr;
        S.valsAlt = (uint32_t*)g->valsAlt.ptr;
        S.sortTempBytes = sort_temp_bytes(capacity, L.endBit());
        CK(g->sortTemp.reserve(S.sortTempBytes));
        S.sortTemp = g->sortTemp.ptr;
    }
    rc = prepare_raster(ctx);
    if (rc)
    {
        ctx->profiling = profiling;
        return rc;
    }
    cudaError_t e = cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess)
    {
        rc = enqueue_front(ctx, L, B, S, g->stream);
        if (!rc)
            rc = enqueue_back(ctx, L, B, S, capacity, true, g->stream);
        e = cudaStreamEndCapture(g->stream, &g->graph);
    }
    ctx->profiling = profiling;
    if (rc)
        return rc;
    CK(e);
    CK(cudaGraphInstantiate(&g->exec, g->graph, 0));
    g->stats.tess_vertices = (uint64_t)L.tessRows * kTessTextureWidth;
    g->stats.patches = (uint64_t)L.items[0] + L.items[1] + L.items[3];
    g->stats.triangles = L.slots;
    g->stats.bin_entries = g->measured;
    g->stats.tiles = L.tiles;
    g->stats.kernel_launches = 1 + (L.gradSpans ? 1 : 0) + (L.tessSpans ? 1 : 0) +
                               (L.slots ? 2 : 0) + (capacity ? 4 : 0) + 1;
    return RIVE_CUDA_OK;
}
} // namespace

int rive_cuda_graph_create(rive_cuda_context* ctx,
                           const rive_cuda_batch_flush* flushes,
                           uint32_t count,
                           uint32_t bin_capacity,
                           rive_cuda_graph** out)
{
    if (!ctx || !out || !count || !flushes)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "NULL argument to graph_create");
    *out = nullptr;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    std::vector<FlushInput> in(count);
    for (uint32_t i = 0; i < count; ++i)
    {
        const rive_cuda_batch_flush& f = flushes[i];
        if (!f.desc || !f.target_pixels_device)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush %u: NULL desc or target",
                             i);
        in[i].d = f.desc;
        in[i].rb = resolve_device_buffers(f.buffers);
        in[i].fb = (uint32_t*)f.target_pixels_device;
    }
    CK(cudaSetDevice(ctx->device));
    auto* g = new (std::nothrow) rive_cuda_graph();
    if (!g)
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    g->ctx = ctx;
    int rc = graph_build(ctx, g, in.data(), count, bin_capacity);
    if (rc)
    {
        graph_free(g);
        return rc;
    }
    *out = g;
    return RIVE_CUDA_OK;
}

int rive_cuda_graph_launch(rive_cuda_graph* g, void* cuda_stream)
{
    if (!g)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    rive_cuda_context* ctx = g->ctx;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : g->stream;
    if (const int rc = order_after_reads(ctx, s))
        return rc;
    CK(cudaGraphLaunch(g->exec, s));
    return RIVE_CUDA_OK;
}

int rive_cuda_graph_check(rive_cuda_graph* g, void* cuda_stream)
{
    if (!g)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    rive_cuda_context* ctx = g->ctx;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : g->stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(g->hError, g->error.ptr, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const uint32_t err = *g->hError;
    if (err)
    {
        CK(cudaMemsetAsync(g->error.ptr, 0, 4, s));
        CK(cudaStreamSynchronize(s));
        return set_error(ctx, RIVE_CUDA_ERR_DEVICE_STATUS,
                         "graph device status 0x%x (32: more bin entries than the capacity %u)",
                         err, g->capacity);
    }
    return RIVE_CUDA_OK;
}

int rive_cuda_graph_stats(const rive_cuda_graph* g, rive_cuda_flush_stats* out)
{
    if (!g || !out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out = g->stats;
    return RIVE_CUDA_OK;
}

void rive_cuda_graph_destroy(rive_cuda_graph* g)
{
    if (!g)
        return;
    cudaSetDevice(g->ctx->device);
    if (g->stream)
        cudaStreamSynchronize(g->stream);
    graph_free(g);
}

int rive_cuda_flush_batch(rive_cuda_context* ctx,
                          const rive_cuda_batch_flush* flushes,
                          uint32_t count,
                          void* cuda_stream)
{
    if (!ctx || (count && !flushes))
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "NULL argument to flush_batch");
    std::vector<FlushInput> in(count);
    for (uint32_t i = 0; i < count; ++i)
    {
        const rive_cuda_batch_flush& f = flushes[i];
        if (!f.desc || !f.target_pixels_device)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush %u: NULL desc or target",
                             i);
        in[i].d = f.desc;
        in[i].rb = resolve_device_buffers(f.buffers);
        in[i].fb = (uint32_t*)f.target_pixels_device;
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    if (const int rc = order_after_reads(ctx, s))
        return rc;
    return run_batch(ctx, in.data(), count, s);
}

int rive_cuda_sync(rive_cuda_context* ctx, void* cuda_stream)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(ctx->hError, ctx->dError, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (s == ctx->stream)
    {
        CK(cudaStreamSynchronize(ctx->readStream)); // its asynchronous read-backs
        ctx->readsInFlight = false;
    }
    uint32_t err = *ctx->hError;
    if (err)
    {
        CK(cudaMemsetAsync(ctx->dError, 0, 4, s));
        CK(cudaStreamSynchronize(s));
        return set_error(ctx, RIVE_CUDA_ERR_DEVICE_STATUS,
                         "device status 0x%x (1 tess index, 2 contour, 4 path, "
                         "16 coordinate range, 32 bin overflow, 64 mesh index)",
                         err);
    }
    return RIVE_CUDA_OK;
}

int rive_cuda_read_tess_texture(rive_cuda_context* ctx, void* dst, size_t bytes)
{
    if (!ctx || !dst)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(dst, ctx->tess.ptr, std::min(bytes, ctx->lastTessBytes), cudaMemcpyDeviceToHost));
    return RIVE_CUDA_OK;
}

int rive_cuda_texture_create(rive_cuda_context* ctx,
                             uint32_t width,
                             uint32_t height,
                             uint32_t mip_levels,
                             const void* rgba_host,
                             rive_cuda_texture** out_texture)
{
    if (!ctx || !rgba_host || !out_texture || width == 0 || height == 0 || width > 16384 ||
        height > 16384 || mip_levels == 0)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    *out_texture = nullptr;
    uint32_t full = 0;
    for (uint32_t m = width | height; m; m >>= 1)
        ++full;
    if (mip_levels > full || mip_levels > (uint32_t)kMaxMipLevels)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                         "%u mip levels for a %ux%u image (at most %u)", mip_levels, width, height,
                         std::min(full, (uint32_t)kMaxMipLevels));
    CK(cudaSetDevice(ctx->device));
    rive_cuda_texture* t = new (std::nothrow) rive_cuda_texture();
    if (!t)
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    uint32_t total = 0;
    for (uint32_t l = 0; l < mip_levels; ++l)
    {
        t->desc.off[l] = total;
        total += std::max(width >> l, 1u) * std::max(height >> l, 1u);
    }
    cudaError_t e = cudaMalloc(&t->mem, (size_t)total * 4);
    if (e != cudaSuccess)
    {
        delete t;
        return cuda_fail(ctx, e, "cudaMalloc(texture)");
    }
    t->texels = total;
    t->desc.texels = (const uchar4*)t->mem;
    t->desc.width = width;
    t->desc.height = height;
    t->desc.levels = mip_levels;
    e = cudaMemcpyAsync(t->mem, rgba_host, (size_t)width * height * 4, cudaMemcpyHostToDevice,
                        ctx->stream);
    uchar4* base = (uchar4*)t->mem;
    for (uint32_t l = 1; l < mip_levels && e == cudaSuccess; ++l)
    {
        const uint32_t sw = std::max(width >> (l - 1), 1u), sh = std::max(height >> (l - 1), 1u);
        const uint32_t dw = std::max(width >> l, 1u), dh = std::max(height >> l, 1u);
        mip_level_kernel<<<(dw * dh + 255) / 256, 256, 0, ctx->stream>>>(
            base + t->desc.off[l - 1], sw, sh, base + t->desc.off[l], dw, dh);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
    {
        cudaFree(t->mem);
        delete t;
        return cuda_fail(ctx, e, "texture upload");
    }
    *out_texture = t;
    return RIVE_CUDA_OK;
}

void rive_cuda_texture_destroy(rive_cuda_context* ctx, rive_cuda_texture* texture)
{
    // A pending flush that may run again could still read it.
    if (ctx)
        settle_pending(ctx);
    if (!texture)
        return;
    if (ctx)
    {
        // Flushes still in flight may sample it.
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(texture->mem);
    delete texture;
}

int rive_cuda_render_buffer_create(rive_cuda_context* ctx,
                                   uint32_t type,
                                   size_t bytes,
                                   rive_cuda_render_buffer** out_buffer)
{
    if (!ctx || !out_buffer || type > RIVE_CUDA_RENDER_BUFFER_VERTEX || bytes == 0)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out_buffer = nullptr;
    CK(cudaSetDevice(ctx->device));
    rive_cuda_render_buffer* b = new (std::nothrow) rive_cuda_render_buffer();
    if (!b)
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    // Rounded up to 16 bytes so float2 and uint16 reads of the last element
    // stay inside the allocation.
    cudaError_t e = cudaMalloc(&b->mem, (bytes + 15) & ~(size_t)15);
    if (e == cudaSuccess)
        e = cudaMemset(b->mem, 0, (bytes + 15) & ~(size_t)15);
    if (e != cudaSuccess)
    {
        cudaFree(b->mem);
        delete b;
        return cuda_fail(ctx, e, "cudaMalloc(render buffer)");
    }
    b->bytes = bytes;
    b->type = type;
    *out_buffer = b;
    return RIVE_CUDA_OK;
}

int rive_cuda_render_buffer_write(rive_cuda_context* ctx,
                                  rive_cuda_render_buffer* buffer,
                                  size_t offset,
                                  const void* src_host,
                                  size_t bytes)
{
    if (!ctx || !buffer || (!src_host && bytes) || offset > buffer->bytes ||
        bytes > buffer->bytes - offset)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    if (!bytes)
        return RIVE_CUDA_OK;
    CK(cudaSetDevice(ctx->device));
    // After the flushes already queued (they may still read the old bytes).
    CK(cudaMemcpyAsync((uint8_t*)buffer->mem + offset, src_host, bytes, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return RIVE_CUDA_OK;
}

void rive_cuda_render_buffer_destroy(rive_cuda_context* ctx, rive_cuda_render_buffer* buffer)
{
    // A pending flush that may run again could still read it.
    if (ctx)
        settle_pending(ctx);
    if (!buffer)
        return;
    if (ctx)
    {
        // Flushes still in flight may read it.
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    cudaFree(buffer->mem);
    delete buffer;
}

int rive_cuda_texture_read(rive_cuda_context* ctx,
                           const rive_cuda_texture* texture,
                           uint32_t level,
                           void* dst_host,
                           size_t bytes)
{
    if (!ctx || !texture || !dst_host || level >= texture->desc.levels)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    const size_t n = (size_t)std::max(texture->desc.width >> level, 1u) *
                     std::max(texture->desc.height >> level, 1u) * 4;
    CK(cudaMemcpy(dst_host, (const uchar4*)texture->mem + texture->desc.off[level],
                  std::min(bytes, n), cudaMemcpyDeviceToHost));
    return RIVE_CUDA_OK;
}

int rive_cuda_read_atlas_texture(rive_cuda_context* ctx, void* dst, size_t bytes)
{
    if (!ctx || !dst)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    const size_t n = std::min(bytes, ctx->lastAtlasBytes);
    if (n)
        CK(cudaMemcpy(dst, ctx->atlas.ptr, n, cudaMemcpyDeviceToHost));
    return RIVE_CUDA_OK;
}

int rive_cuda_read_grad_texture(rive_cuda_context* ctx, void* dst, size_t bytes)
{
    if (!ctx || !dst)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(dst, ctx->grad.ptr, std::min(bytes, ctx->lastGradBytes), cudaMemcpyDeviceToHost));
    return RIVE_CUDA_OK;
}

int rive_cuda_feather_table(uint16_t* out)
{
    if (!out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    feather_table_f16(out);
    return RIVE_CUDA_OK;
}

int rive_cuda_inverse_feather_table(uint16_t* out)
{
    if (!out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    float table[kGaussianTableSize];
    build_inverse_feather_table(table);
    for (int i = 0; i < kGaussianTableSize; ++i)
        out[i] = __half_as_ushort(__float2half_rn(table[i]));
    return RIVE_CUDA_OK;
}

int rive_cuda_set_raster_config(rive_cuda_context* ctx, int tile_size, int ctas_per_sm)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    const int log2 = tile_size == 8 ? 3 : tile_size == 16 ? 4 : tile_size == 32 ? 5 : -1;
    if (log2 < 0)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "tile size %d (8, 16 or 32)",
                         tile_size);
    if (ctas_per_sm < 0 || ctas_per_sm > 32)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "ctas_per_sm %d", ctas_per_sm);
    ctx->tileLog2 = log2;
    ctx->rasterCtasPerSm = log2 == 5 ? 0 : ctas_per_sm;
    return RIVE_CUDA_OK;
}

int rive_cuda_get_raster_config(const rive_cuda_context* ctx, int* tile_size, int* ctas_per_sm)
{
    if (!ctx || !tile_size || !ctas_per_sm)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *tile_size = 1 << ctx->tileLog2;
    *ctas_per_sm = ctx->rasterCtasPerSm;
    return RIVE_CUDA_OK;
}

int rive_cuda_eval_tessellation_math(int fn, const float* in, float* out, size_t n)
{
    if (!((fn >= 0 && fn <= 5) || (fn >= 10 && fn <= 13)) || (n && (!in || !out)))
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    return run_tess_math(fn, in, out, n) == cudaSuccess ? RIVE_CUDA_OK : RIVE_CUDA_ERR_CUDA;
}

int rive_cuda_set_raster_queue(rive_cuda_context* ctx, int enabled)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    ctx->rasterQueue = enabled != 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_get_raster_queue(const rive_cuda_context* ctx, int* enabled)
{
    if (!ctx || !enabled)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *enabled = ctx->rasterQueue ? 1 : 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_set_winding_tiles(rive_cuda_context* ctx, int enabled)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    ctx->windingTiles = enabled != 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_set_bin_speculation(rive_cuda_context* ctx, int enabled)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    ctx->speculate = enabled != 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_get_bin_speculation(const rive_cuda_context* ctx, int* enabled)
{
    if (!ctx || !enabled)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *enabled = ctx->speculate ? 1 : 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_get_winding_tiles(const rive_cuda_context* ctx, int* enabled)
{
    if (!ctx || !enabled)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *enabled = ctx->windingTiles ? 1 : 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_set_profiling(rive_cuda_context* ctx, int enabled)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    ctx->profiling = enabled != 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_profile_collect(rive_cuda_context* ctx,
                              double ms[RIVE_CUDA_STAGE_COUNT],
                              uint64_t launches[RIVE_CUDA_STAGE_COUNT])
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    CK(cudaSetDevice(ctx->device));
    for (int st = 0; st < RIVE_CUDA_STAGE_COUNT; ++st)
    {
        double sum = 0;
        for (auto& pr : ctx->stageEvents[st])
        {
            CK(cudaEventSynchronize(pr.second));
            float t = 0;
            CK(cudaEventElapsedTime(&t, pr.first, pr.second));
            sum += t;
            ctx->eventPool.push_back(pr.first);
            ctx->eventPool.push_back(pr.second);
        }
        if (ms)
            ms[st] = sum;
        if (launches)
            launches[st] = ctx->stageEvents[st].size();
        ctx->stageEvents[st].clear();
    }
    return RIVE_CUDA_OK;
}

int rive_cuda_last_flush_stats(const rive_cuda_context* cctx, rive_cuda_flush_stats* out)
{
    // The bin-entry total of a pending speculative flush is read here.
    rive_cuda_context* ctx = const_cast<rive_cuda_context*>(cctx);
    if (ctx)
    {
        const int src = settle_pending(ctx);
        if (src)
            return src;
    }
    if (!ctx || !out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out = ctx->stats;
    return RIVE_CUDA_OK;
}

} // extern "C"
