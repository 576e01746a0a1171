/*
 * scene_replay.hpp -- TEST INFRASTRUCTURE (oracle). Replays a rive_scene.h
 * recording through rive-runtime's own RiveRenderer into any RenderContext:
 * one frame, cleared, midpoint fans only (frameBudgetMs = 0), then flush.
 * Shared by ref_capture.cpp (recording RenderContextImpl),
 * adapter_capture.cpp (the product's RenderContextCUDAImpl) and
 * cmdbuf_capture.cpp (the reference's deferred command recorder).
 */
#pragma once

#include "rive/factory.hpp"
#include "rive/renderer.hpp"
#include "rive/renderer/render_context.hpp"
#include "rive/renderer/rive_renderer.hpp"
#include "rive/renderer/rive_render_image.hpp"
#include "rive/renderer/render_context_impl.hpp"
#include "rive/renderer/gpu.hpp"
#include "rive/math/raw_path.hpp"
#include "rive/shapes/paint/blend_mode.hpp"
#include "rive/shapes/paint/stroke_cap.hpp"
#include "rive/shapes/paint/stroke_join.hpp"

#include "rive_scene.h"

#include <cstring>
#include <limits>
#include <vector>

// The arrays of a rive_scene.h recording, in place.
struct SceneView
{
    rive_scene_header hdr;
    const rive_scene_path* paths;
    const rive_scene_paint* paints;
    const rive_scene_cmd* cmds;
    const uint8_t* verbs;
    const float* points;
    const rive_scene_stop* stops;
    // Images (only when the recording has an images section).
    std::vector<rive_scene_image> images;
    std::vector<const uint8_t*> imageTexels;
    // Meshes (only when the recording has a meshes section).
    struct Mesh
    {
        uint32_t vertexCount, indexCount;
        const float* xy;
        const float* uv;
        const uint16_t* indices;
    };
    std::vector<Mesh> meshes;
};

// Returns nullptr on success, else a message.
inline const char* parse_scene(const std::vector<uint8_t>& scene, SceneView* v)
{
    if (scene.size() < sizeof(rive_scene_header))
        return "cannot read scene";
    memcpy(&v->hdr, scene.data(), sizeof(v->hdr));
    const rive_scene_header& hdr = v->hdr;
    if (hdr.magic != RIVE_SCENE_MAGIC)
        return "bad scene magic";
    size_t off = sizeof(hdr);
    v->paths = reinterpret_cast<const rive_scene_path*>(scene.data() + off);
    off += sizeof(rive_scene_path) * hdr.path_count;
    v->paints = reinterpret_cast<const rive_scene_paint*>(scene.data() + off);
    off += sizeof(rive_scene_paint) * hdr.paint_count;
    v->cmds = reinterpret_cast<const rive_scene_cmd*>(scene.data() + off);
    off += sizeof(rive_scene_cmd) * hdr.cmd_count;
    v->verbs = scene.data() + off;
    off += (hdr.verb_count + 3u) & ~3u;
    v->points = reinterpret_cast<const float*>(scene.data() + off);
    off += sizeof(float) * 2 * hdr.point_count;
    v->stops = reinterpret_cast<const rive_scene_stop*>(scene.data() + off);
    off += sizeof(rive_scene_stop) * hdr.stop_count;
    if (off > scene.size())
        return "truncated scene";
    if (off + sizeof(rive_scene_images) <= scene.size())
    {
        rive_scene_images ih;
        memcpy(&ih, scene.data() + off, sizeof(ih));
        if (ih.magic != RIVE_SCENE_IMAGES_MAGIC)
            return "bad images magic";
        off += sizeof(ih);
        for (uint32_t i = 0; i < ih.count; ++i)
        {
            rive_scene_image im;
            if (off + sizeof(im) > scene.size())
                return "truncated images";
            memcpy(&im, scene.data() + off, sizeof(im));
            off += sizeof(im);
            const size_t bytes = (size_t)im.width * im.height * 4;
            if (im.width == 0 || im.height == 0 || off + bytes > scene.size())
                return "truncated image";
            v->images.push_back(im);
            v->imageTexels.push_back(scene.data() + off);
            off += bytes;
        }
    }
    if (off + sizeof(rive_scene_meshes) <= scene.size())
    {
        rive_scene_meshes mh;
        memcpy(&mh, scene.data() + off, sizeof(mh));
        if (mh.magic != RIVE_SCENE_MESHES_MAGIC)
            return "bad meshes magic";
        off += sizeof(mh);
        for (uint32_t i = 0; i < mh.count; ++i)
        {
            rive_scene_mesh m;
            if (off + sizeof(m) > scene.size())
                return "truncated meshes";
            memcpy(&m, scene.data() + off, sizeof(m));
            off += sizeof(m);
            const size_t vbytes = (size_t)m.vertex_count * 8;
            const size_t ibytes = ((size_t)m.index_count * 2 + 3) & ~(size_t)3;
            if (m.vertex_count == 0 || m.index_count == 0 || off + 2 * vbytes + ibytes > scene.size())
                return "truncated mesh";
            SceneView::Mesh mv;
            mv.vertexCount = m.vertex_count;
            mv.indexCount = m.index_count;
            mv.xy = reinterpret_cast<const float*>(scene.data() + off);
            mv.uv = reinterpret_cast<const float*>(scene.data() + off + vbytes);
            mv.indices = reinterpret_cast<const uint16_t*>(scene.data() + off + 2 * vbytes);
            v->meshes.push_back(mv);
            off += 2 * vbytes + ibytes;
        }
    }
    return nullptr;
}

// Mip levels of a full chain for an image of the given size: the index of
// the highest set bit of (height | width), counted from 1, as the
// reference's own image decoding asks makeImageTexture for
// (render_context.cpp:251).
inline uint32_t scene_image_mip_count(uint32_t w, uint32_t h)
{
    uint32_t n = 0;
    for (uint32_t m = w | h; m; m >>= 1)
        ++n;
    return n;
}

// The scene's paths and paints, made by `factory` (Factory::makeRenderPath,
// makeRenderPaint, make*Gradient).
struct SceneResources
{
    std::vector<rive::rcp<rive::RenderPath>> paths;
    std::vector<rive::rcp<rive::RenderPaint>> paints;
    std::vector<rive::rcp<rive::RenderImage>> images;
    struct Mesh
    {
        rive::rcp<rive::RenderBuffer> vertices, uvs, indices;
        uint32_t vertexCount, indexCount;
    };
    std::vector<Mesh> meshes;
};

// A RenderBuffer of `factory` holding `bytes` bytes (Factory::makeRenderBuffer,
// then map / copy / unmap, as an app fills one).
inline rive::rcp<rive::RenderBuffer> make_filled_buffer(rive::Factory* factory,
                                                        rive::RenderBufferType type,
                                                        const void* data,
                                                        size_t bytes)
{
    rive::rcp<rive::RenderBuffer> b =
        factory->makeRenderBuffer(type, rive::RenderBufferFlags::none, bytes);
    if (!b)
        return nullptr;
    void* p = b->map();
    memcpy(p, data, bytes);
    b->unmap();
    return b;
}

// The scene's meshes as RenderBuffers of `factory` (vertex, uv, index).
inline const char* make_scene_meshes(rive::Factory* factory,
                                     const SceneView& v,
                                     SceneResources* out)
{
    using namespace rive;
    for (const SceneView::Mesh& m : v.meshes)
    {
        SceneResources::Mesh r;
        r.vertexCount = m.vertexCount;
        r.indexCount = m.indexCount;
        r.vertices = make_filled_buffer(factory, RenderBufferType::vertex, m.xy,
                                        (size_t)m.vertexCount * 8);
        r.uvs = make_filled_buffer(factory, RenderBufferType::vertex, m.uv,
                                   (size_t)m.vertexCount * 8);
        r.indices = make_filled_buffer(factory, RenderBufferType::index, m.indices,
                                       (size_t)m.indexCount * 2);
        if (!r.vertices || !r.uvs || !r.indices)
            return "cannot make a mesh buffer";
        out->meshes.push_back(std::move(r));
    }
    return nullptr;
}

// The scene's images as textures of `impl` (RenderContextImpl::makeImageTexture
// with one level of RGBA8 texels and the rest generated), wrapped as the
// renderer's images.
inline const char* make_scene_images(rive::gpu::RenderContextImpl* impl,
                                     const SceneView& v,
                                     SceneResources* out)
{
    using namespace rive;
    for (size_t i = 0; i < v.images.size(); ++i)
    {
        const rive_scene_image& im = v.images[i];
        rcp<gpu::Texture> tex =
            impl->makeImageTexture(im.width, im.height, scene_image_mip_count(im.width, im.height),
                                   GPUTextureFormat::rgba32, v.imageTexels[i], 1, 1, false, true);
        if (!tex)
            return "cannot make an image texture";
        out->images.push_back(make_rcp<RiveRenderImage>(std::move(tex)));
    }
    return nullptr;
}

inline const char* make_scene_resources(rive::Factory* factory,
                                        const SceneView& v,
                                        SceneResources* out)
{
    using namespace rive;
    const rive_scene_header& hdr = v.hdr;
    for (uint32_t i = 0; i < hdr.path_count; ++i)
    {
        const rive_scene_path& p = v.paths[i];
        RawPath raw;
        const float* pts = v.points + 2 * p.point_offset;
        for (uint32_t k = 0; k < p.verb_count; ++k)
        {
            switch (v.verbs[p.verb_offset + k])
            {
                case RIVE_SCENE_VERB_MOVE:
                    raw.move({pts[0], pts[1]});
                    pts += 2;
                    break;
                case RIVE_SCENE_VERB_LINE:
                    raw.line({pts[0], pts[1]});
                    pts += 2;
                    break;
                case RIVE_SCENE_VERB_QUAD:
                    raw.quad({pts[0], pts[1]}, {pts[2], pts[3]});
                    pts += 4;
                    break;
                case RIVE_SCENE_VERB_CUBIC:
                    raw.cubic({pts[0], pts[1]}, {pts[2], pts[3]}, {pts[4], pts[5]});
                    pts += 6;
                    break;
                case RIVE_SCENE_VERB_CLOSE:
                    raw.close();
                    break;
                default:
                    return "bad verb";
            }
        }
        const auto fillRule = static_cast<FillRule>(p.fill_rule & RIVE_SCENE_FILL_RULE_MASK);
        if (p.fill_rule & RIVE_SCENE_PATH_APPENDED)
        {
            // As a replayed call stream builds it: no pruning.
            rcp<RenderPath> path = factory->makeEmptyRenderPath();
            path->fillRule(fillRule);
            path->addRawPath(raw);
            out->paths.push_back(path);
        }
        else
        {
            out->paths.push_back(factory->makeRenderPath(raw, fillRule));
        }
    }
    for (uint32_t i = 0; i < hdr.paint_count; ++i)
    {
        const rive_scene_paint& s = v.paints[i];
        rcp<RenderPaint> paint = factory->makeRenderPaint();
        paint->style(s.style == RIVE_SCENE_STYLE_FILL ? RenderPaintStyle::fill
                                                      : RenderPaintStyle::stroke);
        paint->color(s.color);
        paint->thickness(s.thickness);
        paint->join(static_cast<StrokeJoin>(s.join));
        paint->cap(static_cast<StrokeCap>(s.cap));
        paint->blendMode(static_cast<BlendMode>(s.blend_mode));
        if (s.feather != 0)
            paint->feather(s.feather);
        if (s.shader != RIVE_SCENE_SHADER_NONE)
        {
            std::vector<ColorInt> colors(s.stop_count);
            std::vector<float> pos(s.stop_count);
            for (uint32_t k = 0; k < s.stop_count; ++k)
            {
                colors[k] = v.stops[s.stop_offset + k].color;
                pos[k] = v.stops[s.stop_offset + k].position;
            }
            rcp<RenderShader> shader =
                s.shader == RIVE_SCENE_SHADER_LINEAR
                    ? factory->makeLinearGradient(s.g[0], s.g[1], s.g[2], s.g[3], colors.data(),
                                                  pos.data(), s.stop_count)
                    : factory->makeRadialGradient(s.g[0], s.g[1], s.g[2], colors.data(),
                                                  pos.data(), s.stop_count);
            paint->shader(shader);
        }
        out->paints.push_back(paint);
    }
    return nullptr;
}

// The scene's Renderer calls, in order.
inline const char* issue_scene_commands(rive::Renderer* renderer,
                                        const SceneView& v,
                                        const SceneResources& res)
{
    using namespace rive;
    for (uint32_t i = 0; i < v.hdr.cmd_count; ++i)
    {
        const rive_scene_cmd& c = v.cmds[i];
        switch (c.op)
        {
            case RIVE_SCENE_CMD_SAVE:
                renderer->save();
                break;
            case RIVE_SCENE_CMD_RESTORE:
                renderer->restore();
                break;
            case RIVE_SCENE_CMD_TRANSFORM:
                renderer->transform(Mat2D(c.m[0], c.m[1], c.m[2], c.m[3], c.m[4], c.m[5]));
                break;
            case RIVE_SCENE_CMD_DRAW_PATH:
                if (c.a >= res.paths.size() || c.b >= res.paints.size())
                    return "draw references a missing path or paint";
                renderer->drawPath(res.paths[c.a].get(), res.paints[c.b].get());
                break;
            case RIVE_SCENE_CMD_CLIP_PATH:
                if (c.a >= res.paths.size())
                    return "clip references a missing path";
                renderer->clipPath(res.paths[c.a].get());
                break;
            case RIVE_SCENE_CMD_MODULATE_OPACITY:
                renderer->modulateOpacity(c.m[0]);
                break;
            case RIVE_SCENE_CMD_DRAW_IMAGE:
                if (c.a >= res.images.size())
                    return "draw references a missing image";
                renderer->drawImage(res.images[c.a].get(),
                                    ImageSampler::SamplerFromKey(static_cast<uint8_t>(c.b >> 8)),
                                    static_cast<BlendMode>(c.b & 0xffu), c.m[0]);
                break;
            case RIVE_SCENE_CMD_DRAW_IMAGE_MESH:
            {
                const size_t mi = static_cast<size_t>(c.m[1]);
                if (c.a >= res.images.size() || mi >= res.meshes.size())
                    return "mesh draw references a missing image or mesh";
                const SceneResources::Mesh& m = res.meshes[mi];
                renderer->drawImageMesh(
                    res.images[c.a].get(), ImageSampler::SamplerFromKey(static_cast<uint8_t>(c.b >> 8)),
                    m.vertices, m.uvs, m.indices, m.vertexCount, m.indexCount,
                    static_cast<BlendMode>(c.b & 0xffu), c.m[0]);
                break;
            }
            default:
                return "bad command";
        }
    }
    return nullptr;
}

// The frame every capture tool renders: cleared to the scene's colour,
// midpoint fans for every fill, or (flag) every eligible fill triangulated;
// both are independent of timing.
inline rive::gpu::RenderContext::FrameDescriptor scene_frame(uint32_t width,
                                                             uint32_t height,
                                                             uint32_t clearColor,
                                                             uint32_t ditherMode,
                                                             uint32_t flags)
{
    using namespace rive::gpu;
    RenderContext::FrameDescriptor fd;
    fd.renderTargetWidth = width;
    fd.renderTargetHeight = height;
    fd.loadAction = LoadAction::clear;
    fd.clearColor = clearColor;
    fd.ditherMode = static_cast<DitherMode>(ditherMode);
    fd.triangulationThresholds.frameBudgetMs =
        (flags & RIVE_SCENE_FLAG_TRIANGULATE) ? std::numeric_limits<float>::infinity() : 0.f;
    return fd;
}

// Returns nullptr on success, else a message. `makeTarget(width, height)`
// returns the rcp<RenderTarget> to draw into.
template <class MakeTarget>
const char* replay_scene(rive::gpu::RenderContext* ctx,
                         const std::vector<uint8_t>& scene,
                         MakeTarget makeTarget,
                         rive::rcp<rive::gpu::RenderTarget>* outTarget = nullptr)
{
    using namespace rive;
    using namespace rive::gpu;
    SceneView v;
    if (const char* err = parse_scene(scene, &v))
        return err;
    SceneResources res;
    if (const char* err = make_scene_resources(ctx, v, &res))
        return err;
    if (const char* err = make_scene_images(ctx->impl(), v, &res))
        return err;
    if (const char* err = make_scene_meshes(ctx, v, &res))
        return err;
    rcp<RenderTarget> target = makeTarget(v.hdr.width, v.hdr.height);
    if (!target)
        return "cannot make the render target";
    ctx->beginFrame(
        scene_frame(v.hdr.width, v.hdr.height, v.hdr.clear_color, v.hdr.dither_mode, v.hdr.flags));
    {
        RiveRenderer renderer(ctx);
        if (const char* err = issue_scene_commands(&renderer, v, res))
            return err;
    }
    ctx->flush({.renderTarget = target.get()});
    if (outTarget)
        *outTarget = target;
    return nullptr;
}
