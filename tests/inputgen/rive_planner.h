/*
 * rive_planner.h -- TEST AND BENCH INFRASTRUCTURE (not part of the product):
 * a host-side stand-in for the reference front end that turns a rive_scene.h
 * recording into the records a RenderContextImpl receives for one frame.
 *
 * It restates, for InterlockMode::rasterOrdering with midpoint-fan
 * tessellation (no feathers, images or interior triangulation), the CPU work
 * of rive-runtime's RiveRenderer and RenderContext:
 *   RiveRenderer::drawPath/clipPath/applyClip (renderer/src/rive_renderer.cpp),
 *   PathDraw::Make/initForMidpointFan/pushMidpointFanTessellationData
 *     (renderer/src/draw.cpp),
 *   LogicalFlush::pushDraws/allocateGradient/layoutResources/writeResources,
 *   TessellationWriter (renderer/src/render_context.cpp),
 *   PathData/PaintData/PaintAuxData/FlushUniforms (renderer/src/gpu.cpp).
 * Its output is byte-compared against the reference's own output on the same
 * scene in the tests.
 *
 * Output: a flush capture (the buffers of the frame plus one
 * rive_cuda_flush_desc + rive_cuda_draw_batch[] per logical flush), in the
 * layout documented in rive-runtime_gb300/capture.py.
 */
#ifndef RIVE_PLANNER_H
#define RIVE_PLANNER_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Plans one frame. On success returns 0 and a malloc'd capture in *out
 * (free with rive_plan_free). On failure returns nonzero and writes a message
 * into err (if non-NULL). */
int rive_plan_scene(const void* scene,
                    size_t scene_bytes,
                    void** out,
                    size_t* out_bytes,
                    char* err,
                    size_t err_len);

void rive_plan_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* RIVE_PLANNER_H */
