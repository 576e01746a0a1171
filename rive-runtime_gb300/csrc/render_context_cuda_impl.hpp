// RenderContextCUDAImpl: the rive::gpu::RenderContextImpl backend
// (renderer/include/rive/renderer/render_context_impl.hpp:26-243) that runs
// the flush on the sm_103a kernels behind include/rive_cuda.h.
//
// This file compiles inside a rive-runtime tree (it includes the renderer's
// own headers); a maintainer adds it as renderer/src/cuda/ beside the
// Metal/Vulkan/D3D/GL backends and links librive_cuda.so. RiveRenderer,
// RenderPath, RenderPaint and Factory are used unchanged:
//
//   auto ctx = rive::gpu::RenderContextCUDAImpl::MakeContext(/*device=*/0);
//   auto* impl = ctx->static_impl_cast<rive::gpu::RenderContextCUDAImpl>();
//   auto target = impl->makeRenderTarget(w, h);
//   ctx->beginFrame({.renderTargetWidth = w, .renderTargetHeight = h, ...});
//   rive::RiveRenderer renderer(ctx.get());
//   ... renderer.drawPath(path, paint) ...
//   ctx->flush({.renderTarget = target.get()});
//   target->readPixels(rgba);   // or target->devicePixels() for zero-copy
//
// Supported: InterlockMode::rasterOrdering with midpoint-fan patches, the
// center-AA midpoint fans of feathered fills, the feather atlas with its
// blits and, for large fills the front end triangulates, outer-curve patches
// plus interior triangles; i.e. fills (nonzero, even-odd, clockwise), strokes
// with every join and cap, feathers of any radius (fills and strokes), linear
// and radial gradients, clip paths (nested), clip rects, all blend modes,
// dither, image paints (drawImage draws a rectangle path with an image paint
// in this mode) and image meshes (drawImageMesh; RenderBuffers live on the
// device) on RGBA textures with their mip chains. A flush that needs anything
// else (atomic/MSAA/clockwise interlock modes) is not rendered: flush()
// records RIVE_CUDA_ERR_UNSUPPORTED in lastStatus().
#pragma once

// texture.hpp first: render_context_impl.hpp destroys rcp<Texture> inline.
#include "rive/renderer/texture.hpp"
#include "rive/renderer/render_context_impl.hpp"
#include "rive/renderer/render_target.hpp"

#include "rive_cuda.h"

#include <memory>
#include <string>

namespace rive::gpu
{
// A device-resident RGBA8 render target (premultiplied, R in the low byte).
class RenderTargetCUDA : public RenderTarget
{
public:
    ~RenderTargetCUDA() override;

    rive_cuda_render_target* handle() const { return m_target; }
    // Device pointer to width * height * 4 bytes, row-major, tightly packed.
    void* devicePixels() const;
    // Waits for outstanding flushes, then copies the pixels to host memory
    // (width * height * 4 bytes). Returns a rive_cuda.h status.
    int readPixels(void* dstHost) const;

private:
    friend class RenderContextCUDAImpl;
    RenderTargetCUDA(rive_cuda_context*, rive_cuda_render_target*, uint32_t width, uint32_t height);
    rive_cuda_context* m_ctx;
    rive_cuda_render_target* m_target;
};

class RenderContextCUDAImpl : public RenderContextImpl
{
public:
    // nullptr when the device cannot be opened (message on stderr).
    static std::unique_ptr<RenderContext> MakeContext(int device = 0);
    ~RenderContextCUDAImpl() override;

    rcp<RenderTargetCUDA> makeRenderTarget(uint32_t width, uint32_t height);

    // Status and message of the last failing call (flush() returns void).
    int lastStatus() const { return m_lastStatus; }
    std::string lastError() const;
    // Device-side status of the flushes since the last call (bin overflow,
    // coordinate range...): waits for the stream.
    int syncAndCheck();
    rive_cuda_context* handle() const { return m_ctx; }

#ifdef RIVE_CANVAS
    std::unique_ptr<rive::ore::Context> makeOreContext() override { return nullptr; }
#endif

    rcp<RenderBuffer> makeRenderBuffer(RenderBufferType, RenderBufferFlags, size_t) override;
    rcp<Texture> makeImageTexture(uint32_t width,
                                  uint32_t height,
                                  uint32_t mipLevelCount,
                                  GPUTextureFormat,
                                  const uint8_t imageData[],
                                  uint8_t blockWidth,
                                  uint8_t blockHeight,
                                  bool srgb,
                                  bool generateRemainingMips) override;

    void resizeFlushUniformBuffer(size_t sizeInBytes) override;
    void resizePathBuffer(size_t sizeInBytes, StorageBufferStructure) override;
    void resizePaintBuffer(size_t sizeInBytes, StorageBufferStructure) override;
    void resizePaintAuxBuffer(size_t sizeInBytes, StorageBufferStructure) override;
    void resizeContourBuffer(size_t sizeInBytes, StorageBufferStructure) override;
    void resizeGradSpanBuffer(size_t sizeInBytes) override;
    void resizeTessVertexSpanBuffer(size_t sizeInBytes) override;
    void resizeTriangleVertexBuffer(size_t sizeInBytes) override;
    void resizeImageDrawInstanceBuffer(size_t sizeInBytes) override;

    void* mapFlushUniformBuffer(size_t mapSizeInBytes) override;
    void* mapPathBuffer(size_t mapSizeInBytes) override;
    void* mapPaintBuffer(size_t mapSizeInBytes) override;
    void* mapPaintAuxBuffer(size_t mapSizeInBytes) override;
    void* mapContourBuffer(size_t mapSizeInBytes) override;
    void* mapGradSpanBuffer(size_t mapSizeInBytes) override;
    void* mapTessVertexSpanBuffer(size_t mapSizeInBytes) override;
    void* mapTriangleVertexBuffer(size_t mapSizeInBytes) override;
    void* mapImageDrawInstanceBuffer(size_t mapSizeInBytes) override;

    void unmapFlushUniformBuffer(size_t mapSizeInBytes) override;
    void unmapPathBuffer(size_t mapSizeInBytes) override;
    void unmapPaintBuffer(size_t mapSizeInBytes) override;
    void unmapPaintAuxBuffer(size_t mapSizeInBytes) override;
    void unmapContourBuffer(size_t mapSizeInBytes) override;
    void unmapGradSpanBuffer(size_t mapSizeInBytes) override;
    void unmapTessVertexSpanBuffer(size_t mapSizeInBytes) override;
    void unmapTriangleVertexBuffer(size_t mapSizeInBytes) override;
    void unmapImageDrawInstanceBuffer(size_t mapSizeInBytes) override;

    void resizeGradientTexture(uint32_t width, uint32_t height) override;
    void resizeTessellationTexture(uint32_t width, uint32_t height) override;
    void resizeFeatherAtlasTexture(uint32_t width, uint32_t height) override;

    // PlatformFeatures::alwaysFeatherToAtlas (gpu.hpp:156-158): render every
    // feathered draw through the feather atlas (off by default: only blurs
    // the front end scales to half resolution or less go there).
    void setAlwaysFeatherToAtlas(bool on) { m_platformFeatures.alwaysFeatherToAtlas = on; }

    // FlushDescriptor::externalCommandBuffer, when set, is the cudaStream_t
    // to enqueue on; otherwise the context's own stream is used.
    void flush(const FlushDescriptor&) override;

    double secondsNow() const override;

private:
    explicit RenderContextCUDAImpl(rive_cuda_context*);
    void resize(int kind, size_t bytes);
    void* map(int kind, size_t bytes);
    void unmap(int kind, size_t bytes);
    void note(int status);

    rive_cuda_context* m_ctx;
    uint32_t m_gradTextureHeight = 0;
    int m_lastStatus = RIVE_CUDA_OK;
};
} // namespace rive::gpu
