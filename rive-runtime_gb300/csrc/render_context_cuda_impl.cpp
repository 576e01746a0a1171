// RenderContextCUDAImpl (render_context_cuda_impl.hpp): each RenderContextImpl
// call becomes one rive_cuda.h call. Buffer kinds follow the order of the
// resize/map/unmap families in render_context_impl.hpp:108-174; the flush
// descriptor and draw list are copied field by field into
// rive_cuda_flush_desc / rive_cuda_draw_batch (gpu.hpp:1219-1282, 1320-1438)
// before RenderContext frees them (render_context.cpp:1028).
#include "render_context_cuda_impl.hpp"

#include "rive/renderer/gpu.hpp"
#include "rive/renderer/render_context.hpp"
#include "rive/renderer/texture.hpp"
#include "rive/gpu_texture_format.hpp"
#include "rive/renderer.hpp"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

namespace rive::gpu
{
// A RenderBuffer of image-mesh data (vertex positions, texture coordinates or
// indices): the app writes a host shadow between map and unmap; unmap copies
// it into the device buffer (rive_cuda_render_buffer_write), which the
// flushes of imageMesh batches then read.
class RenderBufferCUDA : public RenderBuffer
{
public:
    RenderBufferCUDA(rive_cuda_context* ctx,
                     RenderBufferType type,
                     RenderBufferFlags flags,
                     size_t bytes) :
        RenderBuffer(type, flags, bytes), m_ctx(ctx), m_shadow(bytes)
    {
        m_status = rive_cuda_render_buffer_create(
            ctx,
            type == RenderBufferType::index ? RIVE_CUDA_RENDER_BUFFER_INDEX
                                            : RIVE_CUDA_RENDER_BUFFER_VERTEX,
            bytes, &m_buffer);
    }
    ~RenderBufferCUDA() override { rive_cuda_render_buffer_destroy(m_ctx, m_buffer); }
    const rive_cuda_render_buffer* handle() const { return m_buffer; }
    int status() const { return m_status; }

protected:
    void* onMap() override { return m_shadow.data(); }
    void onUnmap() override
    {
        if (m_buffer)
            m_status = rive_cuda_render_buffer_write(m_ctx, m_buffer, 0, m_shadow.data(),
                                                     m_shadow.size());
    }

private:
    rive_cuda_context* m_ctx;
    std::vector<uint8_t> m_shadow;
    rive_cuda_render_buffer* m_buffer = nullptr;
    int m_status = RIVE_CUDA_OK;
};

RenderTargetCUDA::RenderTargetCUDA(rive_cuda_context* ctx,
                                   rive_cuda_render_target* target,
                                   uint32_t width,
                                   uint32_t height) :
    RenderTarget(width, height), m_ctx(ctx), m_target(target)
{}

RenderTargetCUDA::~RenderTargetCUDA() { rive_cuda_render_target_destroy(m_ctx, m_target); }

void* RenderTargetCUDA::devicePixels() const
{
    return rive_cuda_render_target_device_ptr(m_target);
}

int RenderTargetCUDA::readPixels(void* dstHost) const
{
    return rive_cuda_render_target_read(m_ctx, m_target, dstHost, nullptr);
}

std::unique_ptr<RenderContext> RenderContextCUDAImpl::MakeContext(int device)
{
    rive_cuda_context* ctx = nullptr;
    int rc = rive_cuda_context_create(device, &ctx);
    if (rc != RIVE_CUDA_OK)
    {
        fprintf(stderr, "RenderContextCUDAImpl: cannot open CUDA device %d (status %d)\n", device,
                rc);
        return nullptr;
    }
    std::unique_ptr<RenderContextCUDAImpl> impl(new RenderContextCUDAImpl(ctx));
    return std::make_unique<RenderContext>(std::move(impl));
}

RenderContextCUDAImpl::RenderContextCUDAImpl(rive_cuda_context* ctx) : m_ctx(ctx)
{
    // Only pixel-local-storage-style raster ordering is implemented; the
    // tile kernel gives the ordering guarantee that mode relies on.
    m_platformFeatures.supportsRasterOrderingMode = true;
}

RenderContextCUDAImpl::~RenderContextCUDAImpl() { rive_cuda_context_destroy(m_ctx); }

rcp<RenderTargetCUDA> RenderContextCUDAImpl::makeRenderTarget(uint32_t width, uint32_t height)
{
    rive_cuda_render_target* t = nullptr;
    int rc = rive_cuda_render_target_create(m_ctx, width, height, &t);
    note(rc);
    if (rc != RIVE_CUDA_OK)
        return nullptr;
    return rcp<RenderTargetCUDA>(new RenderTargetCUDA(m_ctx, t, width, height));
}

std::string RenderContextCUDAImpl::lastError() const
{
    char buf[512] = {};
    rive_cuda_last_error(m_ctx, buf, sizeof(buf));
    return buf;
}

int RenderContextCUDAImpl::syncAndCheck()
{
    int rc = rive_cuda_sync(m_ctx, nullptr);
    note(rc);
    return rc;
}

void RenderContextCUDAImpl::note(int status)
{
    if (status != RIVE_CUDA_OK)
        m_lastStatus = status;
}

rcp<RenderBuffer> RenderContextCUDAImpl::makeRenderBuffer(RenderBufferType type,
                                                          RenderBufferFlags flags,
                                                          size_t bytes)
{
    auto buffer = make_rcp<RenderBufferCUDA>(m_ctx, type, flags, bytes);
    note(buffer->status());
    return buffer->handle() ? buffer : nullptr;
}

// A texture in device memory with its mip chain (rive_cuda_texture_create).
class TextureCUDA : public Texture
{
public:
    TextureCUDA(rive_cuda_context* ctx, rive_cuda_texture* tex, uint32_t w, uint32_t h) :
        Texture(w, h), m_ctx(ctx), m_tex(tex)
    {}
    ~TextureCUDA() override { rive_cuda_texture_destroy(m_ctx, m_tex); }
    const rive_cuda_texture* handle() const { return m_tex; }
    void* nativeHandle() const override { return m_tex; }

private:
    rive_cuda_context* m_ctx;
    rive_cuda_texture* m_tex;
};

rcp<Texture> RenderContextCUDAImpl::makeImageTexture(uint32_t width,
                                                     uint32_t height,
                                                     uint32_t mipLevelCount,
                                                     GPUTextureFormat format,
                                                     const uint8_t imageData[],
                                                     uint8_t,
                                                     uint8_t,
                                                     bool,
                                                     bool generateRemainingMips)
{
    // Uncompressed RGBA (premultiplied, as the front end hands it over) only;
    // the other mip levels are made on the device.
    if (format != GPUTextureFormat::rgba32 || imageData == nullptr)
    {
        note(RIVE_CUDA_ERR_UNSUPPORTED);
        return nullptr;
    }
    rive_cuda_texture* tex = nullptr;
    int rc = rive_cuda_texture_create(m_ctx, width, height,
                                      generateRemainingMips ? mipLevelCount : 1u, imageData,
                                      &tex);
    note(rc);
    if (rc != RIVE_CUDA_OK)
        return nullptr;
    return make_rcp<TextureCUDA>(m_ctx, tex, width, height);
}

// RenderContextImpl::resize* "cannot fail" (render_context_impl.hpp:99-107):
// a failure is recorded and the next map of that buffer returns nullptr,
// which makes RenderContext skip the frame.
void RenderContextCUDAImpl::resize(int kind, size_t bytes)
{
    note(rive_cuda_resize_buffer(m_ctx, kind, bytes));
}

void* RenderContextCUDAImpl::map(int kind, size_t bytes)
{
    void* p = rive_cuda_map_buffer(m_ctx, kind, bytes);
    if (!p)
        note(RIVE_CUDA_ERR_NOT_MAPPED);
    return p;
}

void RenderContextCUDAImpl::unmap(int kind, size_t bytes)
{
    note(rive_cuda_unmap_buffer(m_ctx, kind, bytes));
}

void RenderContextCUDAImpl::resizeFlushUniformBuffer(size_t n) { resize(RIVE_CUDA_BUFFER_FLUSH_UNIFORM, n); }
void RenderContextCUDAImpl::resizePathBuffer(size_t n, StorageBufferStructure) { resize(RIVE_CUDA_BUFFER_PATH, n); }
void RenderContextCUDAImpl::resizePaintBuffer(size_t n, StorageBufferStructure) { resize(RIVE_CUDA_BUFFER_PAINT, n); }
void RenderContextCUDAImpl::resizePaintAuxBuffer(size_t n, StorageBufferStructure) { resize(RIVE_CUDA_BUFFER_PAINT_AUX, n); }
void RenderContextCUDAImpl::resizeContourBuffer(size_t n, StorageBufferStructure) { resize(RIVE_CUDA_BUFFER_CONTOUR, n); }
void RenderContextCUDAImpl::resizeGradSpanBuffer(size_t n) { resize(RIVE_CUDA_BUFFER_GRAD_SPAN, n); }
void RenderContextCUDAImpl::resizeTessVertexSpanBuffer(size_t n) { resize(RIVE_CUDA_BUFFER_TESS_SPAN, n); }
void RenderContextCUDAImpl::resizeTriangleVertexBuffer(size_t n) { resize(RIVE_CUDA_BUFFER_TRIANGLE, n); }
void RenderContextCUDAImpl::resizeImageDrawInstanceBuffer(size_t n) { resize(RIVE_CUDA_BUFFER_IMAGE_DRAW, n); }

void* RenderContextCUDAImpl::mapFlushUniformBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_FLUSH_UNIFORM, n); }
void* RenderContextCUDAImpl::mapPathBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_PATH, n); }
void* RenderContextCUDAImpl::mapPaintBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_PAINT, n); }
void* RenderContextCUDAImpl::mapPaintAuxBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_PAINT_AUX, n); }
void* RenderContextCUDAImpl::mapContourBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_CONTOUR, n); }
void* RenderContextCUDAImpl::mapGradSpanBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_GRAD_SPAN, n); }
void* RenderContextCUDAImpl::mapTessVertexSpanBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_TESS_SPAN, n); }
void* RenderContextCUDAImpl::mapTriangleVertexBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_TRIANGLE, n); }
void* RenderContextCUDAImpl::mapImageDrawInstanceBuffer(size_t n) { return map(RIVE_CUDA_BUFFER_IMAGE_DRAW, n); }

void RenderContextCUDAImpl::unmapFlushUniformBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_FLUSH_UNIFORM, n); }
void RenderContextCUDAImpl::unmapPathBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_PATH, n); }
void RenderContextCUDAImpl::unmapPaintBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_PAINT, n); }
void RenderContextCUDAImpl::unmapPaintAuxBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_PAINT_AUX, n); }
void RenderContextCUDAImpl::unmapContourBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_CONTOUR, n); }
void RenderContextCUDAImpl::unmapGradSpanBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_GRAD_SPAN, n); }
void RenderContextCUDAImpl::unmapTessVertexSpanBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_TESS_SPAN, n); }
void RenderContextCUDAImpl::unmapTriangleVertexBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_TRIANGLE, n); }
void RenderContextCUDAImpl::unmapImageDrawInstanceBuffer(size_t n) { unmap(RIVE_CUDA_BUFFER_IMAGE_DRAW, n); }

void RenderContextCUDAImpl::resizeGradientTexture(uint32_t width, uint32_t height)
{
    m_gradTextureHeight = height;
    note(rive_cuda_resize_gradient_texture(m_ctx, width, height));
}

void RenderContextCUDAImpl::resizeTessellationTexture(uint32_t width, uint32_t height)
{
    note(rive_cuda_resize_tessellation_texture(m_ctx, width, height));
}

// The atlas lives in the flush's intermediates, sized per flush from
// FlushDescriptor::featherAtlasContentWidth/Height; nothing to allocate here.
void RenderContextCUDAImpl::resizeFeatherAtlasTexture(uint32_t, uint32_t) {}

void RenderContextCUDAImpl::flush(const FlushDescriptor& d)
{
    rive_cuda_flush_desc o;
    memset(&o, 0, sizeof(o));
    o.render_target_width = d.renderTarget->width();
    o.render_target_height = d.renderTarget->height();
    o.interlock_mode = static_cast<uint32_t>(d.interlockMode);
    o.color_load_action = static_cast<uint32_t>(d.colorLoadAction);
    o.color_clear_value = d.colorClearValue;
    o.update_bounds[0] = d.renderTargetUpdateBounds.left;
    o.update_bounds[1] = d.renderTargetUpdateBounds.top;
    o.update_bounds[2] = d.renderTargetUpdateBounds.right;
    o.update_bounds[3] = d.renderTargetUpdateBounds.bottom;
    o.combined_shader_features = static_cast<uint32_t>(d.combinedShaderFeatures);
    o.dither_mode = static_cast<uint32_t>(d.ditherMode);
    o.flush_uniform_offset_bytes = static_cast<uint32_t>(d.flushUniformDataOffsetInBytes);
    o.path_count = d.pathCount;
    o.first_path = static_cast<uint32_t>(d.firstPath);
    o.first_paint = static_cast<uint32_t>(d.firstPaint);
    o.first_paint_aux = static_cast<uint32_t>(d.firstPaintAux);
    o.contour_count = d.contourCount;
    o.first_contour = static_cast<uint32_t>(d.firstContour);
    o.grad_span_count = d.gradSpanCount;
    o.first_grad_span = static_cast<uint32_t>(d.firstGradSpan);
    o.tess_span_count = d.tessVertexSpanCount;
    o.first_tess_span = static_cast<uint32_t>(d.firstTessVertexSpan);
    o.grad_data_height = d.gradDataHeight;
    o.tess_data_height = d.tessDataHeight;
    o.grad_texture_height = m_gradTextureHeight;
    o.wireframe = d.wireframe ? 1u : 0u;
    o.clockwise_fill_override = d.clockwiseFillOverride ? 1u : 0u;
    o.has_triangle_vertices = d.hasTriangleVertices ? 1u : 0u;

    std::vector<rive_cuda_draw_batch> batches;
    std::vector<rive_cuda_batch_image> images;
    std::vector<rive_cuda_batch_mesh> meshes;
    bool anyImage = false, anyMesh = false;
    if (d.drawList != nullptr)
    {
        for (const DrawBatch& b : *d.drawList)
        {
            rive_cuda_batch_image im = {};
            if (b.imageTexture != nullptr)
            {
                im.texture = static_cast<const TextureCUDA*>(b.imageTexture)->handle();
                im.sampler_key = b.imageSampler.asKey();
                anyImage = true;
            }
            images.push_back(im);
            // An imageMesh batch's buffers (gpu.hpp:1261-1264).
            rive_cuda_batch_mesh mesh = {};
            if (b.drawType == DrawType::imageMesh && b.vertexBuffer && b.uvBuffer &&
                b.indexBuffer)
            {
                mesh.vertices = static_cast<const RenderBufferCUDA*>(b.vertexBuffer)->handle();
                mesh.uvs = static_cast<const RenderBufferCUDA*>(b.uvBuffer)->handle();
                mesh.indices = static_cast<const RenderBufferCUDA*>(b.indexBuffer)->handle();
                mesh.index_count = b.indexCountPerInstance;
                anyMesh = true;
            }
            meshes.push_back(mesh);
            rive_cuda_draw_batch ob;
            ob.draw_type = static_cast<uint32_t>(b.drawType);
            ob.element_count = b.elementCount;
            ob.base_element = b.baseElement;
            ob.shader_features = static_cast<uint32_t>(b.shaderFeatures);
            ob.draw_contents = static_cast<uint32_t>(b.drawContents);
            ob.shader_misc_flags = static_cast<uint32_t>(b.shaderMiscFlags);
            ob.first_blend_mode = static_cast<uint32_t>(b.firstBlendMode);
            ob.barriers = static_cast<uint32_t>(b.barriers);
            batches.push_back(ob);
        }
    }
    o.draw_batch_count = static_cast<uint32_t>(batches.size());
    o.draw_batches = batches.empty() ? nullptr : batches.data();
    o.batch_images = anyImage ? images.data() : nullptr;
    o.batch_meshes = anyMesh ? meshes.data() : nullptr;

    // The feather atlas batches: fills, then strokes.
    std::vector<rive_cuda_atlas_batch> atlas;
    auto add_atlas = [&](const AtlasDrawBatch* b, size_t n) {
        for (size_t i = 0; i < n; ++i)
        {
            rive_cuda_atlas_batch a;
            a.scissor[0] = b[i].scissor.left;
            a.scissor[1] = b[i].scissor.top;
            a.scissor[2] = b[i].scissor.right;
            a.scissor[3] = b[i].scissor.bottom;
            a.patch_count = b[i].patchCount;
            a.base_patch = b[i].basePatch;
            atlas.push_back(a);
        }
    };
    add_atlas(d.featherAtlasFillBatches, d.featherAtlasFillBatchCount);
    add_atlas(d.featherAtlasStrokeBatches, d.featherAtlasStrokeBatchCount);
    o.atlas_texture_width = d.featherAtlasTextureWidth;
    o.atlas_texture_height = d.featherAtlasTextureHeight;
    o.atlas_content_width = d.featherAtlasContentWidth;
    o.atlas_content_height = d.featherAtlasContentHeight;
    o.atlas_fill_batch_count = static_cast<uint32_t>(d.featherAtlasFillBatchCount);
    o.atlas_stroke_batch_count = static_cast<uint32_t>(d.featherAtlasStrokeBatchCount);
    o.atlas_batches = atlas.empty() ? nullptr : atlas.data();

    auto* target = static_cast<RenderTargetCUDA*>(d.renderTarget);
    note(rive_cuda_flush(m_ctx, &o, target->handle(), d.externalCommandBuffer));
}

double RenderContextCUDAImpl::secondsNow() const
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}
} // namespace rive::gpu
