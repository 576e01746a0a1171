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
//   color_ramp_kernel -> tessellate_kernel -> patch_setup_kernel ->
//   (scan) -> bin_scatter_kernel -> (radix sort by tile) ->
//   tile_ranges_kernel -> raster_tile_kernel.
#include "rive_cuda.h"
#include "rive_cuda_internal.cuh"

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
__global__ void patch_setup_kernel(BatchTables B, TriRecord* tris, uint32_t* tileCounts);
__global__ void bin_scatter_kernel(uint32_t slotCount,
                                   const uint2* sceneTiles,
                                   const TriRecord* tris,
                                   const uint32_t* tileCounts,
                                   const uint32_t* offsets,
                                   uint32_t* keys,
                                   uint32_t* vals);
__global__ void tile_ranges_kernel(uint32_t pairCount, const uint32_t* keys, uint2* ranges);
__global__ void raster_tile_kernel(BatchTables B,
                                   const TriRecord* tris,
                                   const uint32_t* sortedSlots,
                                   const uint2* ranges);
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
    DeviceBuffer device;
    size_t deviceValidBytes = 0;
};
} // namespace

struct rive_cuda_render_target
{
    uint32_t width = 0, height = 0;
    uint32_t* pixels = nullptr;
};

struct rive_cuda_context
{
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string lastError;
    RecordRing rings[RIVE_CUDA_BUFFER_KIND_COUNT];
    DeviceBuffer tess, grad;
    uint32_t tessWidth = 0, tessHeight = 0, gradWidth = 0, gradHeight = 0;
    DeviceBuffer tris, tileCounts, offsets;
    DeviceBuffer keys, vals, keysAlt, valsAlt, sortTemp, scanTemp, ranges;
    DeviceBuffer dTables;           // batch tables (device)
    HostBuffer hTables, hUniforms;  // pinned staging of tables and uniforms
    cudaEvent_t tablesCopied = nullptr;
    uint32_t* dError = nullptr;
    uint32_t* hError = nullptr;  // pinned
    uint32_t* hPairs = nullptr;  // pinned: scanned pair total
    rive_cuda_flush_stats stats = {};
    // Stage timing (rive_cuda_set_profiling).
    bool profiling = false;
    std::vector<cudaEvent_t> eventPool;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> stageEvents[RIVE_CUDA_STAGE_COUNT];
    cudaEvent_t openEvent = nullptr;
    int openStage = -1;
    // Last flush's texture extents (for debug read-backs).
    size_t lastTessBytes = 0, lastGradBytes = 0;
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

struct ResolvedBuffers
{
    const void* ptr[7];
    size_t bytes[7];
    // Host copy of the flush-uniform buffer when the caller staged it through
    // a mapped ring (read directly instead of copying it back).
    const void* hostUniforms = nullptr;
};

// One logical flush of a batch.
struct FlushInput
{
    const rive_cuda_flush_desc* d;
    ResolvedBuffers rb;
    uint32_t* fb;
};

// Host-side checks of one flush; counts its patch instances.
int validate_flush(rive_cuda_context* ctx, const rive_cuda_flush_desc* d, const ResolvedBuffers& rb,
                   uint64_t& instances)
{
    if (d->interlock_mode != 0)
        return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED,
                         "interlock mode %u not supported (rasterOrdering only)", d->interlock_mode);
    if (d->has_triangle_vertices)
        return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED,
                         "interior triangulation draws are not supported");
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
    instances = 0;
    for (uint32_t i = 0; i < d->draw_batch_count; ++i)
    {
        const rive_cuda_draw_batch& b = d->draw_batches[i];
        if (b.draw_type != RIVE_CUDA_DRAW_MIDPOINT_FAN_PATCHES)
            return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED, "draw type %u not supported",
                             b.draw_type);
        if (b.shader_features & SF_FEATHER)
            return set_error(ctx, RIVE_CUDA_ERR_UNSUPPORTED, "feathered draws not supported");
        if (((uint64_t)b.base_element + b.element_count) * kPatchSegmentSpan >
            (uint64_t)d->tess_data_height * kTessTextureWidth)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT,
                             "batch %u reads past the tessellation texture", i);
        instances += b.element_count;
    }
    return RIVE_CUDA_OK;
}

size_t align16(size_t n) { return (n + 15) & ~(size_t)15; }

// Runs a batch of independent logical flushes (distinct targets) as one
// sequence of launches: every stage covers the work of all flushes at once.
int run_batch(rive_cuda_context* ctx, const FlushInput* in, uint32_t n, cudaStream_t stream)
{
    if (n == 0)
        return RIVE_CUDA_OK;
    if (n > 65535)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "at most 65535 flushes per batch");
    std::vector<uint64_t> inst(n);
    uint64_t totalInstances = 0, segCount = 0;
    for (uint32_t i = 0; i < n; ++i)
    {
        int rc = validate_flush(ctx, in[i].d, in[i].rb, inst[i]);
        if (rc)
            return rc;
        if (!in[i].fb)
            return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "flush %u has no target", i);
        totalInstances += inst[i];
        for (uint32_t b = 0; b < in[i].d->draw_batch_count; ++b)
            segCount += in[i].d->draw_batches[b].element_count ? 1 : 0;
    }
    if (totalInstances * kPatchTriangleCount > 0xffffffffull)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "too many patches in one batch");
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

    // The previous batch's tables may still be in flight from the staging.
    if (ctx->tablesCopied)
        CK(cudaEventSynchronize(ctx->tablesCopied));

    // Flush uniforms (FlushUniforms, gpu.hpp:1466-1537): from the mapped ring
    // when staged there, else copied back from the device in one wait.
    CK(ctx->hUniforms.reserve((size_t)n * 256));
    uint8_t* uni = (uint8_t*)ctx->hUniforms.ptr;
    bool waitUniforms = false;
    for (uint32_t i = 0; i < n; ++i)
    {
        const rive_cuda_flush_desc* d = in[i].d;
        if (in[i].rb.hostUniforms)
            memcpy(uni + 256 * (size_t)i,
                   (const uint8_t*)in[i].rb.hostUniforms + d->flush_uniform_offset_bytes, 256);
        else
        {
            CK(cudaMemcpyAsync(uni + 256 * (size_t)i,
                               (const uint8_t*)in[i].rb.ptr[RIVE_CUDA_BUFFER_FLUSH_UNIFORM] +
                                   d->flush_uniform_offset_bytes,
                               256, cudaMemcpyDeviceToHost, stream));
            waitUniforms = true;
        }
    }
    if (waitUniforms)
        CK(cudaStreamSynchronize(stream));

    // Layout of the batch: per-flush texture rows, tiles, spans and slots.
    uint64_t tessRows = 0, gradRows = 0, tiles = 0, gradSpans = 0, tessSpans = 0;
    std::vector<uint64_t> tessRow0(n), gradRow0(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        const rive_cuda_flush_desc* d = in[i].d;
        tessRow0[i] = tessRows;
        gradRow0[i] = gradRows;
        tessRows += std::max(d->tess_data_height, 1u);
        gradRows += std::max(d->grad_data_height, 1u);
        const uint64_t tx = (d->render_target_width + kTileSize - 1) / kTileSize;
        const uint64_t ty = (d->render_target_height + kTileSize - 1) / kTileSize;
        tiles += tx * ty;
        gradSpans += d->grad_span_count;
        tessSpans += d->tess_span_count;
    }
    if (tiles > 0x7fffffffull || gradSpans > 0x7fffffffull || tessSpans * 32 > 0xffffffffull)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "batch too large");
    const size_t tessBytes = (size_t)kTessTextureWidth * tessRows * 16;
    const size_t gradBytes = (size_t)kGradTextureWidth * gradRows * 4;
    CK(ctx->tess.reserve(tessBytes));
    CK(ctx->grad.reserve(gradBytes));
    ctx->lastTessBytes = (size_t)kTessTextureWidth * std::max(in[0].d->tess_data_height, 1u) * 16;
    ctx->lastGradBytes = (size_t)kGradTextureWidth * std::max(in[0].d->grad_data_height, 1u) * 4;

    // Tables, staged in pinned memory and copied in one piece.
    const size_t oScenes = 0;
    const size_t oGradBase = align16(oScenes + sizeof(FlushParams) * n);
    const size_t oTessBase = align16(oGradBase + 4 * (n + 1));
    const size_t oTileBase = align16(oTessBase + 4 * (n + 1));
    const size_t oSceneTiles = align16(oTileBase + 4 * (n + 1));
    const size_t oSegments = align16(oSceneTiles + 8 * n);
    const size_t oSegBase = align16(oSegments + sizeof(PatchSegment) * std::max<uint64_t>(segCount, 1));
    const size_t tableBytes = align16(oSegBase + 4 * (segCount + 1));
    CK(ctx->hTables.reserve(tableBytes));
    CK(ctx->dTables.reserve(tableBytes));
    uint8_t* h = (uint8_t*)ctx->hTables.ptr;
    uint8_t* dT = (uint8_t*)ctx->dTables.ptr;
    auto* scenes = (FlushParams*)(h + oScenes);
    auto* gradBase = (uint32_t*)(h + oGradBase);
    auto* tessBase = (uint32_t*)(h + oTessBase);
    auto* tileBase = (uint32_t*)(h + oTileBase);
    auto* sceneTiles = (uint2*)(h + oSceneTiles);
    auto* segs = (PatchSegment*)(h + oSegments);
    auto* segBase = (uint32_t*)(h + oSegBase);
    uint32_t gAcc = 0, tAcc = 0, tileAcc = 0, segAcc = 0, instAcc = 0, slotAcc = 0;
    for (uint32_t i = 0; i < n; ++i)
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
        P.gradTextureHeight = d->grad_texture_height              ? d->grad_texture_height
                              : (n == 1 && ctx->gradHeight != 0u) ? ctx->gradHeight
                                                                  : d->grad_data_height;
        P.tessDataHeight = d->tess_data_height;
        P.width = d->render_target_width;
        P.height = d->render_target_height;
        P.wireframe = d->wireframe;
        P.loadClear = d->color_load_action == RIVE_CUDA_LOAD_CLEAR;
        P.clearColorPremulRGBA = premul_rgba8(d->color_clear_value);
        P.error = ctx->dError;
        P.fb = in[i].fb;
        P.tilesX = (d->render_target_width + kTileSize - 1) / kTileSize;
        const uint8_t* u = uni + 256 * (size_t)i;
        memcpy(&P.pathIDGranularity, u + 72, 4);
        memcpy(&P.ditherScale, u + 88, 4);
        memcpy(&P.ditherBias, u + 92, 4);
        if (P.pathIDGranularity == 0)
            P.pathIDGranularity = 1;
        P.tess = (uint4*)ctx->tess.ptr + (size_t)tessRow0[i] * kTessTextureWidth;
        P.grad = (uchar4*)ctx->grad.ptr + (size_t)gradRow0[i] * kGradTextureWidth;

        gradBase[i] = gAcc;
        tessBase[i] = tAcc;
        tileBase[i] = tileAcc;
        sceneTiles[i] = make_uint2(tileAcc, P.tilesX);
        gAcc += d->grad_span_count;
        tAcc += d->tess_span_count;
        tileAcc += P.tilesX * ((d->render_target_height + kTileSize - 1) / kTileSize);
        for (uint32_t b = 0; b < d->draw_batch_count; ++b)
        {
            const rive_cuda_draw_batch& db = d->draw_batches[b];
            if (!db.element_count)
                continue;
            segs[segAcc] = PatchSegment{i, db.base_element, db.shader_features, slotAcc};
            segBase[segAcc] = instAcc;
            ++segAcc;
            instAcc += db.element_count;
            slotAcc += db.element_count * kPatchTriangleCount;
        }
    }
    gradBase[n] = gAcc;
    tessBase[n] = tAcc;
    tileBase[n] = tileAcc;
    segBase[segAcc] = instAcc;
    CK(cudaMemcpyAsync(dT, h, tableBytes, cudaMemcpyHostToDevice, stream));
    if (!ctx->tablesCopied)
        CK(cudaEventCreateWithFlags(&ctx->tablesCopied, cudaEventDisableTiming));
    CK(cudaEventRecord(ctx->tablesCopied, stream));

    BatchTables B = {};
    B.scenes = (const FlushParams*)(dT + oScenes);
    B.gradSpanBase = (const uint32_t*)(dT + oGradBase);
    B.tessSpanBase = (const uint32_t*)(dT + oTessBase);
    B.tileBase = (const uint32_t*)(dT + oTileBase);
    B.sceneTiles = (const uint2*)(dT + oSceneTiles);
    B.segments = (const PatchSegment*)(dT + oSegments);
    B.segInstanceBase = (const uint32_t*)(dT + oSegBase);
    B.sceneCount = n;
    B.segmentCount = segAcc;
    B.totalGradSpans = gAcc;
    B.totalTessSpans = tAcc;
    B.totalInstances = instAcc;
    B.totalTiles = tileAcc;

    uint64_t launches = 0;
    // Pass 1: gradient ramps. Texels no span covers are never sampled; zero
    // them so the texture is deterministic.
    CK(cudaMemsetAsync(ctx->grad.ptr, 0, gradBytes, stream));
    if (gAcc)
    {
        stage_begin(ctx, RIVE_CUDA_STAGE_COLOR_RAMP, stream);
        color_ramp_kernel<<<gAcc, 128, 0, stream>>>(B);
        stage_end(ctx, stream);
        ++launches;
    }
    // Pass 2: tessellation.
    if (tAcc)
    {
        stage_begin(ctx, RIVE_CUDA_STAGE_TESSELLATE, stream);
        tessellate_kernel<<<(tAcc * 32u + 255u) / 256u, 256, 0, stream>>>(B);
        stage_end(ctx, stream);
        ++launches;
    }
    // Pass 3: patch set-up + tile counts, scan, binning, sort, raster.
    const uint32_t slots = slotAcc;
    CK(ctx->ranges.reserve((size_t)tileAcc * sizeof(uint2)));
    CK(cudaMemsetAsync(ctx->ranges.ptr, 0, (size_t)tileAcc * sizeof(uint2), stream));
    uint32_t pairs = 0;
    if (slots)
    {
        CK(ctx->tris.reserve((size_t)slots * sizeof(TriRecord)));
        CK(ctx->tileCounts.reserve((size_t)slots * 4));
        CK(ctx->offsets.reserve((size_t)slots * 4 + 4));
        stage_begin(ctx, RIVE_CUDA_STAGE_PATCH_SETUP, stream);
        patch_setup_kernel<<<(instAcc + 3) / 4, 128, 0, stream>>>(B, (TriRecord*)ctx->tris.ptr,
                                                                   (uint32_t*)ctx->tileCounts.ptr);
        stage_end(ctx, stream);
        ++launches;
        stage_begin(ctx, RIVE_CUDA_STAGE_BIN, stream);
        // Exclusive scan of tile counts -> pair offsets; slot `slots` holds
        // the total.
        size_t tempBytes = 0;
        uint32_t* counts = (uint32_t*)ctx->tileCounts.ptr;
        uint32_t* offs = (uint32_t*)ctx->offsets.ptr;
        CK(cub::DeviceScan::InclusiveSum(nullptr, tempBytes, counts, offs + 1, slots, stream));
        CK(ctx->scanTemp.reserve(tempBytes));
        CK(cudaMemsetAsync(offs, 0, 4, stream));
        CK(cub::DeviceScan::InclusiveSum(ctx->scanTemp.ptr, tempBytes, counts, offs + 1, slots,
                                         stream));
        stage_end(ctx, stream);
        CK(cudaMemcpyAsync(ctx->hPairs, offs + slots, 4, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        pairs = *ctx->hPairs;
    }
    const uint32_t* sortedSlots = nullptr;
    if (pairs)
    {
        CK(ctx->keys.reserve((size_t)pairs * 4));
        CK(ctx->vals.reserve((size_t)pairs * 4));
        CK(ctx->keysAlt.reserve((size_t)pairs * 4));
        CK(ctx->valsAlt.reserve((size_t)pairs * 4));
        stage_begin(ctx, RIVE_CUDA_STAGE_BIN, stream);
        bin_scatter_kernel<<<(slots + 255) / 256, 256, 0, stream>>>(
            slots, B.sceneTiles, (const TriRecord*)ctx->tris.ptr,
            (const uint32_t*)ctx->tileCounts.ptr, (const uint32_t*)ctx->offsets.ptr,
            (uint32_t*)ctx->keys.ptr, (uint32_t*)ctx->vals.ptr);
        stage_end(ctx, stream);
        ++launches;
        int endBit = 1;
        while ((1ull << endBit) < tileAcc)
            ++endBit;
        cub::DoubleBuffer<uint32_t> k((uint32_t*)ctx->keys.ptr, (uint32_t*)ctx->keysAlt.ptr);
        cub::DoubleBuffer<uint32_t> v((uint32_t*)ctx->vals.ptr, (uint32_t*)ctx->valsAlt.ptr);
        size_t tempBytes = 0;
        CK(cub::DeviceRadixSort::SortPairs(nullptr, tempBytes, k, v, (int)pairs, 0, endBit, stream));
        CK(ctx->sortTemp.reserve(tempBytes));
        stage_begin(ctx, RIVE_CUDA_STAGE_SORT, stream);
        CK(cub::DeviceRadixSort::SortPairs(ctx->sortTemp.ptr, tempBytes, k, v, (int)pairs, 0,
                                           endBit, stream));
        tile_ranges_kernel<<<(pairs + 255) / 256, 256, 0, stream>>>(pairs, k.Current(),
                                                                  (uint2*)ctx->ranges.ptr);
        stage_end(ctx, stream);
        ++launches;
        sortedSlots = v.Current();
    }
    stage_begin(ctx, RIVE_CUDA_STAGE_RASTER, stream);
    raster_tile_kernel<<<tileAcc, 256, 0, stream>>>(B, (const TriRecord*)ctx->tris.ptr, sortedSlots,
                                                    (const uint2*)ctx->ranges.ptr);
    stage_end(ctx, stream);
    ++launches;
    CK(cudaGetLastError());
    ctx->stats.tess_vertices = (uint64_t)tessRows * kTessTextureWidth;
    ctx->stats.patches = instAcc;
    ctx->stats.triangles = slots;
    ctx->stats.bin_entries = pairs;
    ctx->stats.tiles = tileAcc;
    ctx->stats.kernel_launches = launches;
    return RIVE_CUDA_OK;
}

int run_flush(rive_cuda_context* ctx,
              const rive_cuda_flush_desc* d,
              const ResolvedBuffers& rb,
              uint32_t* fbDevice,
              cudaStream_t stream)
{
    FlushInput in{d, rb, fbDevice};
    return run_batch(ctx, &in, 1, stream);
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
        e = cudaMalloc(&ctx->dError, 4);
    if (e == cudaSuccess)
        e = cudaMemset(ctx->dError, 0, 4);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->hError, 4);
    if (e == cudaSuccess)
        e = cudaMallocHost(&ctx->hPairs, 4);
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
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    for (auto& r : ctx->rings)
    {
        for (int i = 0; i < kRingSize; ++i)
        {
            if (r.host[i])
                cudaFreeHost(r.host[i]);
            if (r.done[i])
                cudaEventDestroy(r.done[i]);
        }
        r.device.release();
    }
    for (DeviceBuffer* b : {&ctx->tess, &ctx->grad, &ctx->tris, &ctx->tileCounts, &ctx->offsets,
                            &ctx->keys, &ctx->vals, &ctx->keysAlt, &ctx->valsAlt,
                            &ctx->sortTemp, &ctx->scanTemp, &ctx->ranges, &ctx->dTables})
        b->release();
    ctx->hTables.release();
    ctx->hUniforms.release();
    if (ctx->tablesCopied)
        cudaEventDestroy(ctx->tablesCopied);
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
    RecordRing& r = ctx->rings[kind];
    if (r.mapped)
        return set_error(ctx, RIVE_CUDA_ERR_INVALID_ARGUMENT, "resize while mapped");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < kRingSize; ++i)
    {
        if (r.host[i])
            cudaFreeHost(r.host[i]);
        r.host[i] = nullptr;
    }
    r.capacity = 0;
    r.device.release();
    r.deviceValidBytes = 0;
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
    if (r.device.reserve(bytes) != cudaSuccess)
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
    if (bytes)
        CK(cudaMemcpyAsync(r.device.ptr, r.host[r.current], bytes, cudaMemcpyHostToDevice,
                           ctx->stream));
    CK(cudaEventRecord(r.done[r.current], ctx->stream));
    r.deviceValidBytes = bytes;
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
    if (!t)
        return;
    if (ctx)
    {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
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
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(dst, t->pixels, (size_t)t->width * t->height * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
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
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    if (s != ctx->stream)
    {
        // Uploads were enqueued on the context stream; order them first.
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        CK(cudaEventRecord(ev, ctx->stream));
        CK(cudaStreamWaitEvent(s, ev, 0));
        CK(cudaEventDestroy(ev));
    }
    ResolvedBuffers rb;
    for (int k = 0; k < 7; ++k)
    {
        rb.ptr[k] = ctx->rings[k].device.ptr;
        rb.bytes[k] = ctx->rings[k].deviceValidBytes;
    }
    const RecordRing& ur = ctx->rings[RIVE_CUDA_BUFFER_FLUSH_UNIFORM];
    rb.hostUniforms = ur.host[ur.current];
    return run_flush(ctx, desc, rb, target->pixels, s);
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
    ResolvedBuffers rb;
    const void* p[7] = {buffers->flush_uniforms, buffers->paths, buffers->paints, buffers->paint_aux,
                        buffers->contours, buffers->grad_spans, buffers->tess_spans};
    for (int k = 0; k < 7; ++k)
    {
        rb.ptr[k] = p[k];
        rb.bytes[k] = p[k] ? (size_t)-1 / 2 : 0; // caller-sized; ranges come from desc
    }
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    return run_flush(ctx, desc, rb, (uint32_t*)target_pixels_device, s);
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
        const void* p[7] = {f.buffers.flush_uniforms, f.buffers.paths,    f.buffers.paints,
                            f.buffers.paint_aux,      f.buffers.contours, f.buffers.grad_spans,
                            f.buffers.tess_spans};
        in[i].d = f.desc;
        for (int k = 0; k < 7; ++k)
        {
            in[i].rb.ptr[k] = p[k];
            in[i].rb.bytes[k] = p[k] ? (size_t)-1 / 2 : 0; // caller-sized
        }
        in[i].fb = (uint32_t*)f.target_pixels_device;
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    return run_batch(ctx, in.data(), count, s);
}

int rive_cuda_sync(rive_cuda_context* ctx, void* cuda_stream)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    cudaStream_t s = cuda_stream ? (cudaStream_t)cuda_stream : ctx->stream;
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(ctx->hError, ctx->dError, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    uint32_t err = *ctx->hError;
    if (err)
    {
        CK(cudaMemsetAsync(ctx->dError, 0, 4, s));
        CK(cudaStreamSynchronize(s));
        return set_error(ctx, RIVE_CUDA_ERR_DEVICE_STATUS,
                         "device status 0x%x (1 tess index, 2 contour, 4 path, 8 feather, "
                         "16 coordinate range, 32 bin overflow)",
                         err);
    }
    return RIVE_CUDA_OK;
}

int rive_cuda_read_tess_texture(rive_cuda_context* ctx, void* dst, size_t bytes)
{
    if (!ctx || !dst)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(dst, ctx->tess.ptr, std::min(bytes, ctx->lastTessBytes), cudaMemcpyDeviceToHost));
    return RIVE_CUDA_OK;
}

int rive_cuda_read_grad_texture(rive_cuda_context* ctx, void* dst, size_t bytes)
{
    if (!ctx || !dst)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(dst, ctx->grad.ptr, std::min(bytes, ctx->lastGradBytes), cudaMemcpyDeviceToHost));
    return RIVE_CUDA_OK;
}

int rive_cuda_set_profiling(rive_cuda_context* ctx, int enabled)
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    ctx->profiling = enabled != 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_profile_collect(rive_cuda_context* ctx,
                              double ms[RIVE_CUDA_STAGE_COUNT],
                              uint64_t launches[RIVE_CUDA_STAGE_COUNT])
{
    if (!ctx)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
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

int rive_cuda_last_flush_stats(const rive_cuda_context* ctx, rive_cuda_flush_stats* out)
{
    if (!ctx || !out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out = ctx->stats;
    return RIVE_CUDA_OK;
}

} // extern "C"
