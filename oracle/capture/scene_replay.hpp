/*
 * scene_replay.hpp -- TEST INFRASTRUCTURE (oracle). Replays a rive_scene.h
 * recording through rive-runtime's own RiveRenderer into any RenderContext:
 * one frame, cleared, midpoint fans only (frameBudgetMs = 0), then flush.
 * Shared by ref_capture.cpp (recording RenderContextImpl) and
 * adapter_capture.cpp (the product's RenderContextCUDAImpl).
 */
#pragma once

#include "rive/renderer/render_context.hpp"
#include "rive/renderer/rive_renderer.hpp"
#include "rive/renderer/gpu.hpp"
#include "rive/math/raw_path.hpp"
#include "rive/shapes/paint/blend_mode.hpp"
#include "rive/shapes/paint/stroke_cap.hpp"
#include "rive/shapes/paint/stroke_join.hpp"

#include "rive_scene.h"

#include <cstring>
#include <limits>
#include <vector>

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
    if (scene.size() < sizeof(rive_scene_header))
        return "cannot read scene";
    rive_scene_header hdr;
    memcpy(&hdr, scene.data(), sizeof(hdr));
    if (hdr.magic != RIVE_SCENE_MAGIC)
        return ("bad scene magic");
    size_t off = sizeof(hdr);
    auto* paths = reinterpret_cast<const rive_scene_path*>(scene.data() + off);
    off += sizeof(rive_scene_path) * hdr.path_count;
    auto* paints = reinterpret_cast<const rive_scene_paint*>(scene.data() + off);
    off += sizeof(rive_scene_paint) * hdr.paint_count;
    auto* cmds = reinterpret_cast<const rive_scene_cmd*>(scene.data() + off);
    off += sizeof(rive_scene_cmd) * hdr.cmd_count;
    const uint8_t* verbs = scene.data() + off;
    off += (hdr.verb_count + 3u) & ~3u;
    auto* points = reinterpret_cast<const float*>(scene.data() + off);
    off += sizeof(float) * 2 * hdr.point_count;
    auto* stops = reinterpret_cast<const rive_scene_stop*>(scene.data() + off);
    off += sizeof(rive_scene_stop) * hdr.stop_count;
    if (off > scene.size())
        return ("truncated scene");


    std::vector<rcp<RenderPath>> renderPaths;
    for (uint32_t i = 0; i < hdr.path_count; ++i)
    {
        const rive_scene_path& p = paths[i];
        RawPath raw;
        const float* pts = points + 2 * p.point_offset;
        for (uint32_t v = 0; v < p.verb_count; ++v)
        {
            switch (verbs[p.verb_offset + v])
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
                    raw.cubic({pts[0], pts[1]},
                              {pts[2], pts[3]},
                              {pts[4], pts[5]});
                    pts += 6;
                    break;
                case RIVE_SCENE_VERB_CLOSE:
                    raw.close();
                    break;
                default:
                    return ("bad verb");
            }
        }
        renderPaths.push_back(
            ctx->makeRenderPath(raw, static_cast<FillRule>(p.fill_rule)));
    }

    std::vector<rcp<RenderPaint>> renderPaints;
    for (uint32_t i = 0; i < hdr.paint_count; ++i)
    {
        const rive_scene_paint& s = paints[i];
        rcp<RenderPaint> paint = ctx->makeRenderPaint();
        paint->style(s.style == RIVE_SCENE_STYLE_FILL ? RenderPaintStyle::fill
                                                      : RenderPaintStyle::stroke);
        paint->color(s.color);
        paint->thickness(s.thickness);
        paint->join(static_cast<StrokeJoin>(s.join));
        paint->cap(static_cast<StrokeCap>(s.cap));
        paint->blendMode(static_cast<BlendMode>(s.blend_mode));
        if (s.shader != RIVE_SCENE_SHADER_NONE)
        {
            std::vector<ColorInt> colors(s.stop_count);
            std::vector<float> pos(s.stop_count);
            for (uint32_t k = 0; k < s.stop_count; ++k)
            {
                colors[k] = stops[s.stop_offset + k].color;
                pos[k] = stops[s.stop_offset + k].position;
            }
            rcp<RenderShader> shader =
                s.shader == RIVE_SCENE_SHADER_LINEAR
                    ? ctx->makeLinearGradient(s.g[0],
                                              s.g[1],
                                              s.g[2],
                                              s.g[3],
                                              colors.data(),
                                              pos.data(),
                                              s.stop_count)
                    : ctx->makeRadialGradient(s.g[0],
                                              s.g[1],
                                              s.g[2],
                                              colors.data(),
                                              pos.data(),
                                              s.stop_count);
            paint->shader(shader);
        }
        renderPaints.push_back(paint);
    }

    rcp<RenderTarget> target = makeTarget(hdr.width, hdr.height);
    if (!target)
        return "cannot make the render target";
    RenderContext::FrameDescriptor fd;
    fd.renderTargetWidth = hdr.width;
    fd.renderTargetHeight = hdr.height;
    fd.loadAction = LoadAction::clear;
    fd.clearColor = hdr.clear_color;
    fd.ditherMode = static_cast<DitherMode>(hdr.dither_mode);
    // Midpoint fans for every fill, or (flag) triangulate every eligible fill;
    // both are independent of timing.
    fd.triangulationThresholds.frameBudgetMs =
        (hdr.flags & RIVE_SCENE_FLAG_TRIANGULATE) ? std::numeric_limits<float>::infinity() : 0.f;
    ctx->beginFrame(fd);
    {
        RiveRenderer renderer(ctx);
        for (uint32_t i = 0; i < hdr.cmd_count; ++i)
        {
            const rive_scene_cmd& c = cmds[i];
            switch (c.op)
            {
                case RIVE_SCENE_CMD_SAVE:
                    renderer.save();
                    break;
                case RIVE_SCENE_CMD_RESTORE:
                    renderer.restore();
                    break;
                case RIVE_SCENE_CMD_TRANSFORM:
                    renderer.transform(
                        Mat2D(c.m[0], c.m[1], c.m[2], c.m[3], c.m[4], c.m[5]));
                    break;
                case RIVE_SCENE_CMD_DRAW_PATH:
                    renderer.drawPath(renderPaths[c.a].get(),
                                      renderPaints[c.b].get());
                    break;
                case RIVE_SCENE_CMD_CLIP_PATH:
                    renderer.clipPath(renderPaths[c.a].get());
                    break;
                case RIVE_SCENE_CMD_MODULATE_OPACITY:
                    renderer.modulateOpacity(c.m[0]);
                    break;
                default:
                    return ("bad command");
            }
        }
    }
    ctx->flush({.renderTarget = target.get()});
    if (outTarget)
        *outTarget = target;
    return nullptr;
}
