/*
 * capture_impl.hpp -- TEST INFRASTRUCTURE (oracle). The recording
 * RenderContextImpl shared by the capture tools: every buffer the reference's
 * RenderContext maps and unmaps is kept, every FlushDescriptor
 * (render_context_impl.hpp:217) with its draw batches is recorded, and
 * write_capture() stores them in the capture layout (see ref_capture.cpp).
 */
#pragma once

#include "rive/renderer/texture.hpp"
#include "common/render_context_null.hpp"
#include "rive/renderer/render_context.hpp"
#include "rive/renderer/gpu.hpp"

#include "rive_cuda.h"
#include "capture_format.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <utility>
#include <vector>

namespace capture
{
using namespace rive;
using namespace rive::gpu;
// Buffer ring whose unmap keeps a copy of the bytes the front end wrote.
class CaptureRing : public BufferRing
{
public:
    CaptureRing(size_t capacity, std::vector<uint8_t>* sink) :
        BufferRing(capacity), m_sink(sink)
    {}

private:
    // Zero the staging memory so padding the front end skips (alignment gaps,
    // unused record fields) is deterministic in the capture.
    void* onMapBuffer(int, size_t bytes) override
    {
        memset(shadowBuffer(), 0, bytes);
        return shadowBuffer();
    }
    void onUnmapAndSubmitBuffer(int, size_t bytes) override
    {
        m_sink->assign(shadowBuffer(), shadowBuffer() + bytes);
    }
    std::vector<uint8_t>* m_sink;
};

struct FlushRecord
{
    rive_cuda_flush_desc desc;
    std::vector<rive_cuda_draw_batch> batches;
    std::vector<rive_cuda_atlas_batch> atlasBatches; // fills, then strokes
    std::vector<uint32_t> images; // per batch: texture index (~0u: none), sampler key
    // Per batch: vertex, uv and index render-buffer indices (~0u: not a
    // mesh) and the index count; empty when no batch draws an image mesh.
    std::vector<uint32_t> meshes;
};

// A RenderBuffer the front end asked for (makeRenderBuffer): host bytes, and
// a version that each unmap advances, so a flush records the contents it
// drew.
class CaptureRenderBuffer : public RenderBuffer
{
public:
    CaptureRenderBuffer(RenderBufferType type, RenderBufferFlags flags, size_t bytes, uint64_t id) :
        RenderBuffer(type, flags, bytes), data(bytes), id(id)
    {}
    std::vector<uint8_t> data;
    uint64_t id;
    uint64_t version = 0;

protected:
    void* onMap() override { return data.data(); }
    void onUnmap() override { ++version; }
};

// An image texture the front end asked for (makeImageTexture): its index in
// the capture's texture table.
class CaptureTexture : public Texture
{
public:
    CaptureTexture(uint32_t w, uint32_t h, uint32_t index) : Texture(w, h), index(index) {}
    uint32_t index;
};

class CaptureImpl : public RenderContextNULL
{
public:
    // Buffers in rive_cuda.h kind order 0..8.
    std::vector<uint8_t> buffers[9];
    std::vector<FlushRecord> flushes;
    // Image textures: width, height, mip levels and level-0 texels.
    std::vector<uint32_t> textureDims;
    std::vector<std::vector<uint8_t>> textureTexels;
    // Render-buffer contents the flushes drew: type and bytes.
    std::vector<uint32_t> renderBufferTypes;
    std::vector<std::vector<uint8_t>> renderBufferData;

    rcp<RenderBuffer> makeRenderBuffer(RenderBufferType type,
                                       RenderBufferFlags flags,
                                       size_t bytes) override
    {
        return make_rcp<CaptureRenderBuffer>(type, flags, bytes, m_nextBufferID++);
    }

    // The render-buffer table index of a buffer's current contents.
    uint32_t snapshot(const RenderBuffer* b)
    {
        const auto* cb = static_cast<const CaptureRenderBuffer*>(b);
        const auto key = std::make_pair(cb->id, cb->version);
        auto it = m_snapshots.find(key);
        if (it != m_snapshots.end())
            return it->second;
        const uint32_t index = static_cast<uint32_t>(renderBufferData.size());
        renderBufferTypes.push_back(static_cast<uint32_t>(cb->type()));
        renderBufferData.push_back(cb->data);
        m_snapshots.emplace(key, index);
        return index;
    }

    rcp<Texture> makeImageTexture(uint32_t width,
                                  uint32_t height,
                                  uint32_t mipLevelCount,
                                  GPUTextureFormat format,
                                  const uint8_t imageData[],
                                  uint8_t,
                                  uint8_t,
                                  bool,
                                  bool) override
    {
        if (format != GPUTextureFormat::rgba32 || imageData == nullptr)
            return nullptr; // only uncompressed RGBA is recorded
        const uint32_t index = static_cast<uint32_t>(textureTexels.size());
        textureDims.insert(textureDims.end(), {width, height, mipLevelCount});
        textureTexels.emplace_back(imageData, imageData + (size_t)width * height * 4);
        return make_rcp<CaptureTexture>(width, height, index);
    }

    static std::unique_ptr<RenderContext> Make(CaptureImpl** out)
    {
        auto impl = std::make_unique<CaptureImpl>();
        *out = impl.get();
        return std::make_unique<RenderContext>(std::move(impl));
    }

private:
    // Sizes decide which ring a storage buffer belongs to; the helper impl
    // creates them in a fixed order, so route by call order instead.
    std::unique_ptr<BufferRing> makeUniformBufferRing(size_t cap) override
    {
        return std::make_unique<CaptureRing>(cap, &buffers[0]);
    }
    std::unique_ptr<BufferRing> makeStorageBufferRing(
        size_t cap,
        StorageBufferStructure) override
    {
        return std::make_unique<CaptureRing>(cap, m_nextStorageSink);
    }
    std::unique_ptr<BufferRing> makeVertexBufferRing(size_t cap) override
    {
        return std::make_unique<CaptureRing>(cap, m_nextVertexSink);
    }

public:
    // RenderContextHelperImpl::resize*Buffer call make*BufferRing; set the
    // sink before forwarding.
    void resizePathBuffer(size_t n, StorageBufferStructure s) override
    {
        m_nextStorageSink = &buffers[1];
        RenderContextHelperImpl::resizePathBuffer(n, s);
    }
    void resizePaintBuffer(size_t n, StorageBufferStructure s) override
    {
        m_nextStorageSink = &buffers[2];
        RenderContextHelperImpl::resizePaintBuffer(n, s);
    }
    void resizePaintAuxBuffer(size_t n, StorageBufferStructure s) override
    {
        m_nextStorageSink = &buffers[3];
        RenderContextHelperImpl::resizePaintAuxBuffer(n, s);
    }
    void resizeContourBuffer(size_t n, StorageBufferStructure s) override
    {
        m_nextStorageSink = &buffers[4];
        RenderContextHelperImpl::resizeContourBuffer(n, s);
    }
    void resizeGradSpanBuffer(size_t n) override
    {
        m_nextVertexSink = &buffers[5];
        RenderContextHelperImpl::resizeGradSpanBuffer(n);
    }
    void resizeTessVertexSpanBuffer(size_t n) override
    {
        m_nextVertexSink = &buffers[6];
        RenderContextHelperImpl::resizeTessVertexSpanBuffer(n);
    }
    void resizeTriangleVertexBuffer(size_t n) override
    {
        m_nextVertexSink = &buffers[7];
        RenderContextHelperImpl::resizeTriangleVertexBuffer(n);
    }
    void resizeImageDrawInstanceBuffer(size_t n) override
    {
        m_nextVertexSink = &buffers[8];
        RenderContextHelperImpl::resizeImageDrawInstanceBuffer(n);
    }

    void resizeGradientTexture(uint32_t width, uint32_t height) override
    {
        m_gradTextureHeight = height;
    }

    // PlatformFeatures::alwaysFeatherToAtlas (gpu.hpp:156-158): every
    // feathered draw renders through the feather atlas, whatever its radius.
    void setAlwaysFeatherToAtlas(bool on) { m_platformFeatures.alwaysFeatherToAtlas = on; }

    void flush(const FlushDescriptor& d) override
    {
        FlushRecord rec;
        memset(&rec.desc, 0, sizeof(rec.desc));
        rive_cuda_flush_desc& o = rec.desc;
        o.render_target_width = d.renderTarget->width();
        o.render_target_height = d.renderTarget->height();
        o.interlock_mode = static_cast<uint32_t>(d.interlockMode);
        o.color_load_action = static_cast<uint32_t>(d.colorLoadAction);
        o.color_clear_value = d.colorClearValue;
        o.update_bounds[0] = d.renderTargetUpdateBounds.left;
        o.update_bounds[1] = d.renderTargetUpdateBounds.top;
        o.update_bounds[2] = d.renderTargetUpdateBounds.right;
        o.update_bounds[3] = d.renderTargetUpdateBounds.bottom;
        o.combined_shader_features =
            static_cast<uint32_t>(d.combinedShaderFeatures);
        o.dither_mode = static_cast<uint32_t>(d.ditherMode);
        o.flush_uniform_offset_bytes =
            static_cast<uint32_t>(d.flushUniformDataOffsetInBytes);
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
        o.wireframe = d.wireframe;
        o.clockwise_fill_override = d.clockwiseFillOverride;
        o.has_triangle_vertices = d.hasTriangleVertices;
        if (d.drawList != nullptr)
        {
            for (const DrawBatch& b : *d.drawList)
            {
                rive_cuda_draw_batch ob;
                ob.draw_type = static_cast<uint32_t>(b.drawType);
                ob.element_count = b.elementCount;
                ob.base_element = b.baseElement;
                ob.shader_features = static_cast<uint32_t>(b.shaderFeatures);
                ob.draw_contents = static_cast<uint32_t>(b.drawContents);
                ob.shader_misc_flags =
                    static_cast<uint32_t>(b.shaderMiscFlags);
                ob.first_blend_mode = static_cast<uint32_t>(b.firstBlendMode);
                ob.barriers = static_cast<uint32_t>(b.barriers);
                rec.batches.push_back(ob);
                const auto* tex = static_cast<const CaptureTexture*>(b.imageTexture);
                rec.images.push_back(tex ? tex->index : ~0u);
                rec.images.push_back(b.imageSampler.asKey());
                if (b.drawType == DrawType::imageMesh)
                {
                    rec.meshes.push_back(snapshot(b.vertexBuffer));
                    rec.meshes.push_back(snapshot(b.uvBuffer));
                    rec.meshes.push_back(snapshot(b.indexBuffer));
                    rec.meshes.push_back(b.indexCountPerInstance);
                }
                else
                {
                    rec.meshes.insert(rec.meshes.end(), {~0u, ~0u, ~0u, 0u});
                }
            }
        }
        bool anyMesh = false;
        for (size_t i = 0; i < rec.meshes.size(); i += 4)
            anyMesh = anyMesh || rec.meshes[i] != ~0u;
        if (!anyMesh)
            rec.meshes.clear();
        bool anyImage = false;
        for (size_t i = 0; i < rec.images.size(); i += 2)
            anyImage = anyImage || rec.images[i] != ~0u;
        if (!anyImage)
            rec.images.clear();
        o.draw_batch_count = static_cast<uint32_t>(rec.batches.size());
        o.atlas_texture_width = d.featherAtlasTextureWidth;
        o.atlas_texture_height = d.featherAtlasTextureHeight;
        o.atlas_content_width = d.featherAtlasContentWidth;
        o.atlas_content_height = d.featherAtlasContentHeight;
        o.atlas_fill_batch_count = static_cast<uint32_t>(d.featherAtlasFillBatchCount);
        o.atlas_stroke_batch_count = static_cast<uint32_t>(d.featherAtlasStrokeBatchCount);
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
                rec.atlasBatches.push_back(a);
            }
        };
        add_atlas(d.featherAtlasFillBatches, d.featherAtlasFillBatchCount);
        add_atlas(d.featherAtlasStrokeBatches, d.featherAtlasStrokeBatchCount);
        flushes.push_back(std::move(rec));
    }

private:
    uint32_t m_gradTextureHeight = 0;
    std::vector<uint8_t>* m_nextStorageSink = &m_discard;
    std::vector<uint8_t>* m_nextVertexSink = &m_discard;
    std::vector<uint8_t> m_discard;
    uint64_t m_nextBufferID = 0;
    std::map<std::pair<uint64_t, uint64_t>, uint32_t> m_snapshots;
};

inline std::vector<uint8_t> read_file(const char* path)
{
    std::vector<uint8_t> data;
    FILE* f = fopen(path, "rb");
    if (!f)
        return data;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    data.resize(static_cast<size_t>(n));
    if (n > 0 && fread(data.data(), 1, static_cast<size_t>(n), f) !=
                     static_cast<size_t>(n))
        data.clear();
    fclose(f);
    return data;
}


// Writes the capture of a context's frame (layout in ref_capture.cpp).
inline bool write_capture(const char* path, const CaptureImpl& impl, uint32_t width,
                          uint32_t height)
{
    FILE* f = fopen(path, "wb");
    if (!f)
        return false;
    // Seven buffer kinds, eight when the frame has interior triangles, nine
    // when it has image draw instances.
    const uint32_t kinds = !impl.buffers[8].empty() ? 9u : impl.buffers[7].empty() ? 7u : 8u;
    bool v3 = !impl.renderBufferData.empty();
    for (const FlushRecord& r : impl.flushes)
        v3 = v3 || !r.meshes.empty();
    bool v2 = v3 || !impl.textureTexels.empty();
    for (const FlushRecord& r : impl.flushes)
        v2 = v2 || rive_capture_flush_has_atlas(&r.desc) || !r.images.empty();
    uint32_t head[4] = {v3   ? RIVE_CAPTURE_MAGIC_V3
                        : v2 ? RIVE_CAPTURE_MAGIC_V2
                             : RIVE_CAPTURE_MAGIC_V1,
                        width, height, kinds};
    fwrite(head, sizeof(head), 1, f);
    static const uint8_t zeros[8] = {};
    for (uint32_t k = 0; k < kinds; ++k)
    {
        uint64_t n = impl.buffers[k].size();
        fwrite(&n, sizeof(n), 1, f);
        if (n)
            fwrite(impl.buffers[k].data(), 1, n, f);
        fwrite(zeros, 1, (8 - (n & 7)) & 7, f);
    }
    uint32_t nf = static_cast<uint32_t>(impl.flushes.size());
    fwrite(&nf, sizeof(nf), 1, f);
    for (const FlushRecord& r : impl.flushes)
        rive_capture_write_flush(f, &r.desc, r.batches.data(), r.atlasBatches.data(),
                                 r.images.empty() ? nullptr : r.images.data(),
                                 r.meshes.empty() ? nullptr : r.meshes.data(), v2, v3);
    if (v2)
    {
        std::vector<const uint8_t*> texels;
        for (const auto& t : impl.textureTexels)
            texels.push_back(t.data());
        rive_capture_write_textures(f, static_cast<uint32_t>(texels.size()),
                                    impl.textureDims.data(), texels.data());
    }
    if (v3)
    {
        std::vector<const uint8_t*> data;
        std::vector<uint32_t> sizes;
        for (const auto& b : impl.renderBufferData)
        {
            data.push_back(b.data());
            sizes.push_back(static_cast<uint32_t>(b.size()));
        }
        rive_capture_write_render_buffers(f, static_cast<uint32_t>(data.size()),
                                          impl.renderBufferTypes.data(), sizes.data(),
                                          data.data());
    }
    fclose(f);
    return true;
}
} // namespace capture
