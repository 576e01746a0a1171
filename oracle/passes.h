/*
 * passes.h -- TEST INFRASTRUCTURE. CPU restatement of rive-runtime's GPU
 * passes for InterlockMode::rasterOrdering, used only as the parity checker
 * (tests, smoke check, and the timed CPU baseline of the benchmark). Never
 * linked into the product library.
 *
 *   pass 1  color ramps     renderer/src/shaders/color_ramp.glsl:40-107
 *   pass 2  tessellation    renderer/src/shaders/tessellate.glsl:61-567
 *   pass 3  draw + resolve  renderer/src/shaders/draw_path.vert:96-549,
 *                           draw_path_common.glsl:275-789,
 *                           draw_raster_order_path.frag:14-238,
 *                           advanced_blend.glsl:94-327, common.glsl:185-336
 *
 * Rasterisation follows the Vulkan rules the reference backend runs under
 * (render_context_vulkan_impl.cpp, draw_pipeline_vulkan.cpp:333-334):
 * pixel-centre sampling, 8 sub-pixel bits, top-left fill rule, clockwise front
 * faces with counterclockwise faces culled (gpu.cpp:1552-1567), no-perspective
 * barycentric interpolation.
 *
 * Parity pin: the inputs (records) are pinned by the reference's own front
 * end; the pixel arithmetic is pinned only by this restatement (no graphics
 * API exists to run the reference shaders), with the reference's own shader
 * known-answer tests re-run against it.
 */
#ifndef RIVE_ORACLE_PASSES_H
#define RIVE_ORACLE_PASSES_H

#include <stddef.h>
#include <stdint.h>

#include "rive_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The frame's record buffers, each at element 0 (desc->first_* index in). */
typedef struct oracle_buffers
{
    const void* flush_uniforms;
    size_t flush_uniforms_bytes;
    const void* paths;
    size_t paths_bytes;
    const void* paints;
    size_t paints_bytes;
    const void* paint_aux;
    size_t paint_aux_bytes;
    const void* contours;
    size_t contours_bytes;
    const void* grad_spans;
    size_t grad_spans_bytes;
    const void* tess_spans;
    size_t tess_spans_bytes;
    const void* triangles; /* gpu::TriangleVertex, 12 B each (interior triangulation) */
    size_t triangles_bytes;
    const void* image_draws; /* gpu::ImageDrawInstance, 64 B each (image meshes) */
    size_t image_draws_bytes;
} oracle_buffers;

/* A RenderBuffer for the passes: in a flush descriptor given to the oracle,
 * each rive_cuda_batch_mesh buffer pointer points at one of these (host
 * bytes and their size). */
typedef struct oracle_render_buffer
{
    const void* data;
    size_t bytes;
} oracle_render_buffer;

/* Pass 1 into grad (512 x grad_data_height RGBA8). Returns 0 on success. */
int oracle_color_ramps(const rive_cuda_flush_desc* d,
                       const oracle_buffers* b,
                       uint8_t* grad);

/* Pass 2 into tess (2048 x tess_data_height uint4). fp32 arithmetic. */
int oracle_tessellate(const rive_cuda_flush_desc* d,
                      const oracle_buffers* b,
                      uint32_t* tess);

/* Pass 2 evaluated in double precision (same algorithm): the FP64 twin the
 * tessellated-vertex tolerance is measured against. Flags and theta words
 * are produced the same way; x,y are written as floats rounded from double. */
int oracle_tessellate_f64(const rive_cuda_flush_desc* d,
                          const oracle_buffers* b,
                          double* xy /* 2 per texel */,
                          uint32_t* tess_flags /* 1 per texel */);

/* Pass 3 into fb (width x height RGBA8, row 0 at top), reading the textures
 * of passes 1 and 2. threads <= 0 uses all cores. */
int oracle_draw(const rive_cuda_flush_desc* d,
                const oracle_buffers* b,
                const uint32_t* tess,
                const uint8_t* grad,
                uint8_t* fb,
                int threads);

/* All three passes of one logical flush. */
int oracle_flush(const rive_cuda_flush_desc* d,
                 const oracle_buffers* b,
                 uint8_t* fb,
                 int threads);

/* An image texture for the passes: level-0 RGBA8 premultiplied texels (row 0
 * at the top) and, after oracle_texture_prepare, its whole mip chain. A
 * flush's rive_cuda_batch_image entries point at these (in place of the
 * library's rive_cuda_texture). */
typedef struct oracle_texture
{
    uint32_t width, height, levels;
    const uint8_t* rgba;
    uint8_t* mips;      /* every level; owned, freed by oracle_texture_release */
    uint32_t off[16];   /* texel offset of each level in mips */
} oracle_texture;

/* Makes the mip chain: each texel of level l the rounded mean of the (up to)
 * 2x2 texels of level l - 1 it covers, edges clamped. */
int oracle_texture_prepare(oracle_texture* t);
void oracle_texture_release(oracle_texture* t);

/* The feather atlas pass of one logical flush (tessellation included) into
 * out, atlas_content_width x atlas_content_height fp16 texels, row-major. */
int oracle_atlas(const rive_cuda_flush_desc* d,
                 const oracle_buffers* b,
                 uint16_t* out,
                 int threads);

/* The mip level an image-mesh triangle samples, from the squared texel-space
 * length rho2 of its steeper texture-coordinate derivative, the LOD bias and
 * the texture's level count. */
int oracle_mesh_mip_level(float rho2, float bias, uint32_t levels);

/* Counters of the last oracle_draw (triangles after culling, fragments). */
void oracle_last_stats(uint64_t* triangles, uint64_t* fragments);

/* The fp32 elementary functions the tessellation pass and kernel share
 * (rive-runtime_gb300/csrc/rive_fp32_math.h) over n inputs: fn 0 sin, 1 cos,
 * 2 acos, 3 cube root. Returns -1 for an unknown fn. */
int oracle_math_eval(int fn, const float* x, float* out, size_t n);

/* The tessellation pass's cubic functions on n items (fn 0 clamped_divide,
 * 1 max height, 2 local curvature, 3 De Casteljau point, 4 Wang's segment
 * count, 5 end tangents; see passes.c for the layouts). -1 for an unknown fn. */
int oracle_cubic_eval(int fn, const float* in, float* out, size_t n);

/* Half-float helpers exposed for known-answer tests. */
uint16_t oracle_f32_to_f16(float f);
/* The 512-entry fp16 feather (Gaussian integral) table. */
void oracle_feather_table(uint16_t* out);
/* Its 512-entry fp16 inverse (the height at which the integral reaches x). */
void oracle_inverse_feather_table(uint16_t* out);
float oracle_f16_to_f32(uint16_t h);

/* Blend coefficients of one mode (advanced_blend.glsl:156-301). */
void oracle_advanced_blend_coeffs(const float src[3],
                                  const float dst_premul[4],
                                  int mode,
                                  float out_rgb[3]);

/* Advanced blend of one unmultiplied src over a premultiplied dst
 * (advanced_blend.glsl:156-327), exposed for known-answer tests. */
void oracle_advanced_blend(const float src[3],
                           const float dst_premul[4],
                           int mode,
                           float out_rgb[3]);

#ifdef __cplusplus
}
#endif

#endif
