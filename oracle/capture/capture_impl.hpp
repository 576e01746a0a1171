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

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
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
};

class CaptureImpl : public RenderContextNULL
{
public:
    // Buffers in rive_cuda.h kind order 0..7.
    std::vector<uint8_t> buffers[8];
    std::vector<FlushRecord> flushes;

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
        m_nextVertexSink = &m_discard;
        RenderContextHelperImpl::resizeImageDrawInstanceBuffer(n);
    }

    void resizeGradientTexture(uint32_t width, uint32_t height) override
    {
        m_gradTextureHeight = height;
    }

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
            }
        }
        o.draw_batch_count = static_cast<uint32_t>(rec.batches.size());
        flushes.push_back(std::move(rec));
    }

private:
    uint32_t m_gradTextureHeight = 0;
    std::vector<uint8_t>* m_nextStorageSink = &m_discard;
    std::vector<uint8_t>* m_nextVertexSink = &m_discard;
    std::vector<uint8_t> m_discard;
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
    // Seven buffer kinds, or eight when the frame has interior triangles.
    const uint32_t kinds = impl.buffers[7].empty() ? 7u : 8u;
    uint32_t head[4] = {0x31504352u /*RCP1*/, width, height, kinds};
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
    {
        fwrite(&r.desc, sizeof(r.desc), 1, f);
        if (!r.batches.empty())
            fwrite(r.batches.data(), sizeof(rive_cuda_draw_batch), r.batches.size(), f);
    }
    fclose(f);
    return true;
}
} // namespace capture
