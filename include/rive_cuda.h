/*
 * rive_cuda.h -- C ABI of the GB300 (sm_103a) flush backend for the Rive
 * vector renderer.
 *
 * This is the drop-in seam for rive-runtime's backend interface,
 * `rive::gpu::RenderContextImpl`
 * (renderer/include/rive/renderer/render_context_impl.hpp:26-243). A C++
 * `RenderContextCUDAImpl` (see rive-runtime_gb300/csrc/render_context_cuda_impl.hpp)
 * forwards each virtual to one call below; any other host language binds the
 * same symbols over its FFI. Signatures use plain pointers, sizes and PODs only.
 *
 * Every entry point returns an int status (RIVE_CUDA_OK == 0). On failure the
 * context keeps a message, readable through rive_cuda_last_error(). No call
 * throws and none aborts the process.
 */
#ifndef RIVE_CUDA_H
#define RIVE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RIVE_CUDA_ABI_VERSION 2 /* 2: image meshes (render buffers, batch_meshes, image_draws) */

/* Status codes. */
enum
{
    RIVE_CUDA_OK = 0,
    RIVE_CUDA_ERR_INVALID_ARGUMENT = 1,
    RIVE_CUDA_ERR_UNSUPPORTED = 2,   /* a draw type / interlock mode this
                                        backend does not implement */
    RIVE_CUDA_ERR_OUT_OF_MEMORY = 3,
    RIVE_CUDA_ERR_CUDA = 4,          /* a CUDA runtime call failed */
    RIVE_CUDA_ERR_DEVICE_STATUS = 5, /* a kernel reported an overflow or a
                                        bounded wait that ran out */
    RIVE_CUDA_ERR_NOT_MAPPED = 6,
};

/*
 * Buffer kinds. One per `RenderContextImpl::resize*Buffer/map*Buffer/
 * unmap*Buffer` triple (render_context_impl.hpp:108-174).
 */
enum
{
    RIVE_CUDA_BUFFER_FLUSH_UNIFORM = 0, /* gpu::FlushUniforms, 256 B each      */
    RIVE_CUDA_BUFFER_PATH = 1,          /* gpu::PathData, 64 B each            */
    RIVE_CUDA_BUFFER_PAINT = 2,         /* gpu::PaintData, 8 B each            */
    RIVE_CUDA_BUFFER_PAINT_AUX = 3,     /* gpu::PaintAuxData, 128 B each       */
    RIVE_CUDA_BUFFER_CONTOUR = 4,       /* gpu::ContourData, 16 B each         */
    RIVE_CUDA_BUFFER_GRAD_SPAN = 5,     /* gpu::GradientSpan, 16 B each        */
    RIVE_CUDA_BUFFER_TESS_SPAN = 6,     /* gpu::TessVertexSpan, 64 B each      */
    RIVE_CUDA_BUFFER_TRIANGLE = 7,      /* gpu::TriangleVertex, 12 B each      */
    RIVE_CUDA_BUFFER_IMAGE_DRAW = 8,    /* gpu::ImageDrawInstance, 64 B each   */
    RIVE_CUDA_BUFFER_KIND_COUNT = 9,
};

/* gpu::LoadAction (gpu.hpp:774). */
enum
{
    RIVE_CUDA_LOAD_CLEAR = 0,
    RIVE_CUDA_LOAD_PRESERVE = 1,
    RIVE_CUDA_LOAD_DONT_CARE = 2,
};

/* gpu::DrawType values this backend executes (gpu.hpp:657-668). */
enum
{
    RIVE_CUDA_DRAW_MIDPOINT_FAN_PATCHES = 0,
    RIVE_CUDA_DRAW_MIDPOINT_FAN_CENTER_AA_PATCHES = 1, /* feathered fills */
    RIVE_CUDA_DRAW_OUTER_CURVE_PATCHES = 2,   /* interior triangulation: the curves */
    RIVE_CUDA_DRAW_INTERIOR_TRIANGULATION = 3, /* ... and the interior triangles  */
    RIVE_CUDA_DRAW_FEATHER_ATLAS_BLIT = 4,     /* a path's coverage from the atlas */
};

/*
 * One gpu::AtlasDrawBatch (gpu.hpp:827-833): `patch_count` patch instances
 * from `base_patch`, drawn into the feather atlas within the scissor
 * [left, right) x [top, bottom) (atlas pixels). Fill batches draw center-AA
 * midpoint-fan patches, stroke batches the border of midpoint-fan patches.
 */
typedef struct rive_cuda_atlas_batch
{
    uint16_t scissor[4]; /* left, top, right, bottom */
    uint32_t patch_count;
    uint32_t base_patch;
} rive_cuda_atlas_batch;

/*
 * An image texture (RenderContextImpl::makeImageTexture,
 * render_context_impl.hpp:60-70): RGBA8 premultiplied texels in device
 * memory with their mip chain. Created and destroyed with
 * rive_cuda_texture_create / rive_cuda_texture_destroy.
 */
typedef struct rive_cuda_texture rive_cuda_texture;

/*
 * The image a draw batch samples (gpu::DrawBatch::imageTexture and
 * imageSampler, gpu.hpp:1257-1259): a texture and an ImageSampler key
 * (wrapX + 3 wrapY + 9 filter; include/rive/shapes/paint/image_sampler.hpp).
 */
typedef struct rive_cuda_batch_image
{
    const rive_cuda_texture* texture; /* NULL: the batch draws no image */
    uint32_t sampler_key;
    uint32_t reserved;
} rive_cuda_batch_image;

/*
 * A RenderBuffer (RenderContextImpl::makeRenderBuffer,
 * render_context_impl.hpp:36-39): the vertex, texture-coordinate or index data
 * of image meshes, in device memory. Created, written and destroyed with
 * rive_cuda_render_buffer_create / _write / _destroy.
 */
typedef struct rive_cuda_render_buffer rive_cuda_render_buffer;

/* rive::RenderBufferType (include/rive/renderer.hpp:37-41). */
enum
{
    RIVE_CUDA_RENDER_BUFFER_INDEX = 0,
    RIVE_CUDA_RENDER_BUFFER_VERTEX = 1,
};

/*
 * The mesh an imageMesh draw batch draws (gpu::DrawBatch::vertexBuffer,
 * uvBuffer, indexBuffer and indexCountPerInstance, gpu.hpp:1257-1264;
 * RiveRenderer::drawImageMesh, rive_renderer.cpp:448-495): float2 positions
 * in the draw's local space, float2 texture coordinates, and a uint16
 * triangle list. The batch's ImageDrawInstance (its base_element) carries the
 * matrix, opacity, clip and blend mode; its rive_cuda_batch_image the texture
 * and sampler.
 */
typedef struct rive_cuda_batch_mesh
{
    const rive_cuda_render_buffer* vertices; /* NULL: the batch draws no mesh */
    const rive_cuda_render_buffer* uvs;
    const rive_cuda_render_buffer* indices;
    uint32_t index_count;
    uint32_t reserved;
} rive_cuda_batch_mesh;

/*
 * One gpu::DrawBatch (gpu.hpp:1219-1282), flattened. The reference keeps the
 * batches in a linked list owned by a per-frame allocator; the caller flattens
 * it into an array in list order.
 */
typedef struct rive_cuda_draw_batch
{
    uint32_t draw_type;         /* gpu::DrawType                          */
    uint32_t element_count;     /* patch instances                        */
    uint32_t base_element;      /* first patch instance                   */
    uint32_t shader_features;   /* gpu::ShaderFeatures bits of this batch */
    uint32_t draw_contents;     /* gpu::DrawContents bits                 */
    uint32_t shader_misc_flags; /* gpu::ShaderMiscFlags bits              */
    uint32_t first_blend_mode;  /* rive::BlendMode of the first draw      */
    uint32_t barriers;          /* gpu::BarrierFlags                      */
} rive_cuda_draw_batch;

/*
 * The fields of gpu::FlushDescriptor (gpu.hpp:1320-1438) that a
 * rasterOrdering backend reads. `first_*` are element offsets into the frame's
 * mapped buffers, exactly as RenderContext::LogicalFlush::layoutResources
 * (render_context.cpp:1116-1392) computes them.
 */
typedef struct rive_cuda_flush_desc
{
    uint32_t render_target_width;
    uint32_t render_target_height;
    uint32_t interlock_mode;       /* gpu::InterlockMode; 0 = rasterOrdering */
    uint32_t color_load_action;    /* RIVE_CUDA_LOAD_*                       */
    uint32_t color_clear_value;    /* rive::ColorInt (0xAARRGGBB)            */
    int32_t update_bounds[4];      /* renderTargetUpdateBounds l,t,r,b       */
    uint32_t combined_shader_features;
    uint32_t dither_mode;          /* gpu::DitherMode                        */
    uint32_t flush_uniform_offset_bytes;
    uint32_t path_count;
    uint32_t first_path;
    uint32_t first_paint;
    uint32_t first_paint_aux;
    uint32_t contour_count;
    uint32_t first_contour;
    uint32_t grad_span_count;
    uint32_t first_grad_span;
    uint32_t tess_span_count;
    uint32_t first_tess_span;
    uint32_t grad_data_height;
    uint32_t tess_data_height;
    /* Height the gradient texture was last sized to
     * (RenderContextImpl::resizeGradientTexture, render_context_impl.hpp:177).
     * PaintData's gradient row coordinate is normalised to it (gpu.cpp:906-917,
     * render_context.cpp:1442-1443). 0 means grad_data_height. */
    uint32_t grad_texture_height;
    uint32_t wireframe;
    uint32_t clockwise_fill_override;
    uint32_t has_triangle_vertices;
    uint32_t draw_batch_count;
    const rive_cuda_draw_batch* draw_batches; /* host array, list order */
    /* The feather atlas (gpu.hpp:1361-1368, 1418-1426): feathered paths whose
     * blur is wide enough render their coverage into an offscreen fp16
     * texture first (fills add, strokes take the maximum), and a
     * featherAtlasBlit draw of each then samples it. All zero when the flush
     * has no atlas draws. */
    uint32_t atlas_texture_width;  /* featherAtlasTextureWidth/Height */
    uint32_t atlas_texture_height;
    uint32_t atlas_content_width;  /* featherAtlasContentWidth/Height */
    uint32_t atlas_content_height;
    uint32_t atlas_fill_batch_count;
    uint32_t atlas_stroke_batch_count;
    const rive_cuda_atlas_batch* atlas_batches; /* fill batches, then stroke batches */
    /* Images: NULL, or one entry per draw batch (the batch's texture and
     * sampler; paths with an image paint, ENABLE_MODULATED_IMAGE). */
    const rive_cuda_batch_image* batch_images;
    /* Image meshes: NULL, or one entry per draw batch (the mesh of each
     * imageMesh batch; others NULL). */
    const rive_cuda_batch_mesh* batch_meshes;
} rive_cuda_flush_desc;

typedef struct rive_cuda_context rive_cuda_context;

/* Creates a context bound to CUDA device `device`. */
int rive_cuda_context_create(int device, rive_cuda_context** out_ctx);
void rive_cuda_context_destroy(rive_cuda_context* ctx);

/* Copies the last error message (NUL-terminated, truncated) into buf. */
int rive_cuda_last_error(const rive_cuda_context* ctx, char* buf, size_t len);

/*
 * RenderContextImpl::resize*Buffer (render_context_impl.hpp:108-120). Sizes
 * the ring of pinned host staging buffers and the device copy. A size of 0
 * frees the buffer. "Cannot fail" in the reference; here a failed allocation
 * returns RIVE_CUDA_ERR_OUT_OF_MEMORY and the next map returns NULL.
 */
int rive_cuda_resize_buffer(rive_cuda_context* ctx, int kind, size_t bytes);

/*
 * RenderContextImpl::map*Buffer (render_context_impl.hpp:155-164). Returns a
 * write-only pointer into pinned host memory, valid until the matching unmap,
 * or NULL (the reference then skips the frame, render_context.cpp:1012-1016).
 */
void* rive_cuda_map_buffer(rive_cuda_context* ctx, int kind, size_t bytes);

/*
 * RenderContextImpl::unmap*Buffer (render_context_impl.hpp:165-174). Enqueues
 * the host->device copy of the mapped bytes on the context's upload stream.
 */
int rive_cuda_unmap_buffer(rive_cuda_context* ctx, int kind, size_t bytes);

/* RenderContextImpl::resizeGradientTexture / resizeTessellationTexture
 * (render_context_impl.hpp:177-178). */
int rive_cuda_resize_gradient_texture(rive_cuda_context* ctx,
                                      uint32_t width,
                                      uint32_t height);
int rive_cuda_resize_tessellation_texture(rive_cuda_context* ctx,
                                          uint32_t width,
                                          uint32_t height);

/*
 * RenderContextImpl::makeImageTexture (render_context_impl.hpp:60-70) for an
 * RGBA8 premultiplied image: uploads level 0 (width * height * 4 bytes, row 0
 * at the top) and, with mip_levels > 1, makes the other levels on the device
 * (each texel the rounded mean of the 2x2 texels above it; edges clamp).
 * mip_levels is at most the full chain's length. The texture belongs to the
 * context and is valid until destroyed or the context is.
 */
int rive_cuda_texture_create(rive_cuda_context* ctx,
                             uint32_t width,
                             uint32_t height,
                             uint32_t mip_levels,
                             const void* rgba_host,
                             rive_cuda_texture** out_texture);
void rive_cuda_texture_destroy(rive_cuda_context* ctx, rive_cuda_texture* texture);
/* Copies mip level `level` of the texture to host memory (debug/parity). */
int rive_cuda_texture_read(rive_cuda_context* ctx,
                           const rive_cuda_texture* texture,
                           uint32_t level,
                           void* dst_host,
                           size_t bytes);

/*
 * RenderContextImpl::makeRenderBuffer (render_context_impl.hpp:36-39): a
 * device buffer of `bytes` bytes (zeroed) of type RIVE_CUDA_RENDER_BUFFER_*.
 * rive_cuda_render_buffer_write copies bytes from host memory into it at
 * `offset` (RenderBuffer::unmap), ordered after the work already queued on
 * the context's stream, and returns once they are on the device. Destroying
 * a buffer waits for the context's stream first.
 */
int rive_cuda_render_buffer_create(rive_cuda_context* ctx,
                                   uint32_t type,
                                   size_t bytes,
                                   rive_cuda_render_buffer** out_buffer);
int rive_cuda_render_buffer_write(rive_cuda_context* ctx,
                                  rive_cuda_render_buffer* buffer,
                                  size_t offset,
                                  const void* src_host,
                                  size_t bytes);
void rive_cuda_render_buffer_destroy(rive_cuda_context* ctx, rive_cuda_render_buffer* buffer);

/*
 * Render targets (gpu::RenderTarget, render_target.hpp): an RGBA8 image in
 * device memory, rows of width*4 bytes, row 0 at the top.
 */
typedef struct rive_cuda_render_target rive_cuda_render_target;
int rive_cuda_render_target_create(rive_cuda_context* ctx,
                                   uint32_t width,
                                   uint32_t height,
                                   rive_cuda_render_target** out_target);
void rive_cuda_render_target_destroy(rive_cuda_context* ctx,
                                     rive_cuda_render_target* target);
/* Device address of the target's pixels (for zero-copy consumers, after
 * rive_cuda_sync). */
void* rive_cuda_render_target_device_ptr(rive_cuda_render_target* target);
/* Copies the target's pixels to host memory (width*height*4 bytes). */
int rive_cuda_render_target_read(rive_cuda_context* ctx,
                                  rive_cuda_render_target* target,
                                  void* dst_host,
                                  void* cuda_stream);
/*
 * The same copy, enqueued after the flushes already on the stream (the
 * context's when NULL), without waiting for it: a caller that pipelines
 * frames writes frame k+1's records into the mapped rings while frame k
 * renders and reads back. dst_host should be page-locked for the copy to run
 * asynchronously, and must stay valid until rive_cuda_sync on that stream
 * returns. Later flushes overwrite the target only after this copy. With the
 * context's stream the copy runs on a read stream of its own, so the next
 * flush's front half overlaps it and only its raster into this target
 * waits; flushes into caller-given device memory wait for it too.
 */
int rive_cuda_render_target_read_async(rive_cuda_context* ctx,
                                        rive_cuda_render_target* target,
                                        void* dst_host,
                                        void* cuda_stream);

/*
 * RenderContextImpl::flush(const gpu::FlushDescriptor&)
 * (render_context_impl.hpp:217). Runs, in stream order, the gradient-ramp,
 * tessellation and draw/resolve kernels of one logical flush over the buffers
 * last unmapped, into `target`. `cuda_stream` carries the role of
 * FlushDescriptor::externalCommandBuffer (gpu.hpp:1416): a cudaStream_t, or
 * NULL for the context's own stream. Returns once the work is enqueued;
 * device-side overflow is reported by rive_cuda_sync(). The flushes of one
 * context run in the order they are issued, whatever their streams (a flush
 * on another stream than the previous one waits for it).
 */
int rive_cuda_flush(rive_cuda_context* ctx,
                    const rive_cuda_flush_desc* desc,
                    rive_cuda_render_target* target,
                    void* cuda_stream);

/*
 * Same as rive_cuda_flush, but the record buffers are device pointers the
 * caller already holds (each at element 0 of the frame's buffer; desc->first_*
 * still index into them). No host staging is touched. Used by batched and
 * serving callers that keep path buffers resident in HBM.
 */
typedef struct rive_cuda_device_buffers
{
    const void* flush_uniforms;
    const void* paths;
    const void* paints;
    const void* paint_aux;
    const void* contours;
    const void* grad_spans;
    const void* tess_spans;
    const void* triangle_vertices; /* gpu::TriangleVertex, 12 B each; may be NULL */
    const void* image_draws;       /* gpu::ImageDrawInstance, 64 B each; may be NULL */
} rive_cuda_device_buffers;

int rive_cuda_flush_device(rive_cuda_context* ctx,
                           const rive_cuda_flush_desc* desc,
                           const rive_cuda_device_buffers* buffers,
                           void* target_pixels_device,
                           void* cuda_stream);

/*
 * Batched form (no counterpart in the reference, whose backends flush one
 * render target at a time): `count` independent logical flushes, each with
 * its own records (device pointers, as in rive_cuda_flush_device) and its own
 * target, rendered by ONE sequence of launches whose every stage covers all
 * of them. Each target receives exactly what rive_cuda_flush_device would
 * have written. Targets must be distinct within a batch; the logical flushes
 * of one multi-flush frame go in successive batches. Up to 65535 flushes.
 */
typedef struct rive_cuda_batch_flush
{
    const rive_cuda_flush_desc* desc;
    rive_cuda_device_buffers buffers;
    void* target_pixels_device; /* RGBA8, width * height * 4 bytes */
} rive_cuda_batch_flush;

int rive_cuda_flush_batch(rive_cuda_context* ctx,
                          const rive_cuda_batch_flush* flushes,
                          uint32_t count,
                          void* cuda_stream);

/*
 * A batch captured as a CUDA graph (no counterpart in the reference). Takes
 * the same flushes as rive_cuda_flush_batch and captures the whole batch --
 * every pass of every flush -- into one graph that owns all intermediates.
 * A launch replays it with no host synchronisation and no allocation: the
 * records are read through the device pointers given here, so the caller may
 * rewrite their contents between launches as long as every count and offset
 * in the descriptors stays the same.
 *
 * `bin_capacity` fixes the number of tile bin entries the graph holds; 0 runs
 * the set-up once at creation and takes the measured total plus an eighth.
 * A launch that needs more drops the excess and sets a device status, which
 * rive_cuda_graph_check (waits for the stream) returns as
 * RIVE_CUDA_ERR_DEVICE_STATUS. Launches on one graph must not overlap in
 * time (they share its intermediates); NULL stream: the graph's own stream.
 */
typedef struct rive_cuda_graph rive_cuda_graph;
int rive_cuda_graph_create(rive_cuda_context* ctx,
                           const rive_cuda_batch_flush* flushes,
                           uint32_t count,
                           uint32_t bin_capacity,
                           rive_cuda_graph** out_graph);
int rive_cuda_graph_launch(rive_cuda_graph* graph, void* cuda_stream);
int rive_cuda_graph_check(rive_cuda_graph* graph, void* cuda_stream);
void rive_cuda_graph_destroy(rive_cuda_graph* graph);

/*
 * No-allocation flush (no counterpart in the reference). Same inputs and
 * result as rive_cuda_flush_device, without a context: every intermediate
 * lives in one fixed device pool of RIVE_CUDA_NOALLOC_POOL_BYTES per device,
 * a file-scope __device__ array that exists while the library's module is
 * loaded, so the call itself never allocates or frees memory. With CUDA's
 * lazy module loading (the default) the module, and with it the pool, is
 * loaded on the first call on each device: that first call is where the
 * pool's memory is reserved, and it can fail if the device has no room for
 * it. A caller with a fixed budget makes one small call at start-up. It is for callers that may not allocate while they render: a
 * render thread with a frame deadline (cudaFree waits for the whole device),
 * or an embedder whose device memory budget is fixed up front. It draws
 * midpoint-fan batches only, feathered strokes included; flushes with other
 * draw types (interior triangulation, the center-AA fans of feathered fills)
 * return RIVE_CUDA_ERR_UNSUPPORTED.
 *
 * Limits (larger flushes return RIVE_CUDA_ERR_INVALID_ARGUMENT with a message
 * naming the limit, before anything is launched or written): render target
 * up to RIVE_CUDA_NOALLOC_MAX_WIDTH x RIVE_CUDA_NOALLOC_MAX_HEIGHT, up to
 * RIVE_CUDA_NOALLOC_MAX_TESS_ROWS tessellation rows (so up to
 * RIVE_CUDA_NOALLOC_MAX_PATCHES patches), RIVE_CUDA_NOALLOC_MAX_GRAD_ROWS
 * gradient rows, 256 draw batches and RIVE_CUDA_NOALLOC_MAX_BIN_ENTRIES tile
 * bin entries (this one is known only after set-up; the call then returns
 * without writing the target).
 *
 * The call clears what must start at zero (status word, tile ranges,
 * gradient rows in use) itself. It waits for `cuda_stream` (NULL: the legacy
 * default stream) twice, to read the bin total and at the end, and
 * returns after the whole flush has run, with the device status checked
 * (RIVE_CUDA_ERR_DEVICE_STATUS as rive_cuda_sync reports it). The first call
 * on each device also uploads the feather tables; make it before any stream
 * capture begins. Every call looks up the pool's address
 * (cudaGetSymbolAddress), so a pointer cached from an earlier CUDA context
 * is never used; the feather tables, though, are uploaded once per device
 * and process, so a cudaDeviceReset after the first call is not supported. There is one pool per
 * device and process: calls that overlap in time, from two threads or on two
 * streams of one device, race on it and must be serialised by the caller.
 * `err` (may be NULL) receives a message on failure.
 */
#define RIVE_CUDA_NOALLOC_MAX_WIDTH 1024u
#define RIVE_CUDA_NOALLOC_MAX_HEIGHT 1024u
#define RIVE_CUDA_NOALLOC_MAX_TESS_ROWS 32u
#define RIVE_CUDA_NOALLOC_MAX_PATCHES 8192u /* 32 rows x 2048 vertices / 8 */
#define RIVE_CUDA_NOALLOC_MAX_GRAD_ROWS 64u
#define RIVE_CUDA_NOALLOC_MAX_BIN_ENTRIES 1048576u
#define RIVE_CUDA_NOALLOC_POOL_BYTES 42903552u /* about 40.9 MiB */
int rive_cuda_flush_device_noalloc(const rive_cuda_flush_desc* desc,
                                   const rive_cuda_device_buffers* buffers,
                                   void* target_pixels_device,
                                   void* cuda_stream,
                                   char* err,
                                   size_t err_len);

/*
 * Waits for the stream and returns RIVE_CUDA_ERR_DEVICE_STATUS if any kernel
 * since the last sync reported an overflow; the message names it.
 */
int rive_cuda_sync(rive_cuda_context* ctx, void* cuda_stream);

/*
 * Debug/parity read-backs of the intermediate textures of the last flush:
 * the tessellation texture (uint4 per vertex, 2048 per row) and the gradient
 * texture (RGBA8, 512 per row).
 */
int rive_cuda_read_tess_texture(rive_cuda_context* ctx,
                                void* dst_host,
                                size_t bytes);
int rive_cuda_read_grad_texture(rive_cuda_context* ctx,
                                void* dst_host,
                                size_t bytes);
/* ... and the feather atlas the last flush rendered (fp16 texels,
 * atlas_content_width per row). */
int rive_cuda_read_atlas_texture(rive_cuda_context* ctx,
                                 void* dst_host,
                                 size_t bytes);

/*
 * The tessellation pass's device functions evaluated on n host items (no
 * counterpart in the reference; for parity tests of the kernel's building
 * blocks against the oracle and the reference's unit-test properties). By fn,
 * floats in / out per item:
 *   0 clamped_divide(a, b) 2/1; 1 cubic max height (p0..p3) 8/2 (height, T);
 *   2 local curvature (p0..p3, T, spread) 10/1; 3 De Casteljau point at T
 *   9/2; 4 Wang's segment count under a 2x2 matrix 12/1; 5 end tangents 8/4;
 *   10 sin, 11 cos, 12 acos, 13 cube root 1/1.
 * Synchronous on the current device; allocates its own temporaries.
 */
int rive_cuda_eval_tessellation_math(int fn, const float* in, float* out, size_t n);

/* Counters of the last flush (triangles set up, tile bin entries, ...). */
typedef struct rive_cuda_flush_stats
{
    uint64_t tess_vertices;
    uint64_t patches;
    uint64_t triangles;
    uint64_t bin_entries;
    uint64_t tiles;
    uint64_t kernel_launches;
    uint64_t winding_entries; /* bin entries that are interior-tile windings */
} rive_cuda_flush_stats;
int rive_cuda_last_flush_stats(const rive_cuda_context* ctx,
                               rive_cuda_flush_stats* out);
/* Counters of a graph's batch (bin_entries as measured at creation). */
int rive_cuda_graph_stats(const rive_cuda_graph* graph, rive_cuda_flush_stats* out);

/*
 * The 512 fp16 entries of the feather table the passes sample (the integral of
 * the normal distribution over -3..+3 standard deviations; the reference ships
 * the same table as gpu::g_gaussianIntegralTableF16, gpu.hpp:2083-2091).
 * Feathers below the feather atlas's 32-pixel radius are rendered: strokes
 * in midpoint-fan batches and fills in midpointFanCenterAAPatches batches
 * (draw type 1), both with ENABLE_FEATHER. The feather atlas (larger
 * feathers) is not built.
 */
int rive_cuda_feather_table(uint16_t* out);
/* Its 512-entry fp16 inverse (gpu::g_inverseGaussianIntegralTableF16,
 * gpu.hpp:2090), which feathered-fill tessellation samples. */
int rive_cuda_inverse_feather_table(uint16_t* out);

/*
 * Raster configuration of the context's later flushes, batches and graphs
 * (no counterpart in the reference): the tile size (8, 16 or 32 pixels; 16
 * by default) and, for 8 and 16, a limit on resident raster CTAs per SM (0:
 * as many as fit). The results are the same within the image tolerance for
 * every choice; only the speed differs, so an autotuner may pick per workload.
 */
int rive_cuda_set_raster_config(rive_cuda_context* ctx, int tile_size, int ctas_per_sm);
int rive_cuda_get_raster_config(const rive_cuda_context* ctx, int* tile_size, int* ctas_per_sm);

/*
 * Raster schedule (no counterpart in the reference; off by default, an
 * autotuner knob; 16-pixel tiles): with it on, the raster runs as a
 * persistent grid of resident CTAs that take tiles from an atomic cursor over
 * the batch's tiles sorted by bin entries, heaviest first, instead of one CTA
 * launched per tile. The image is the same either way.
 */
int rive_cuda_set_raster_queue(rive_cuda_context* ctx, int enabled);
int rive_cuda_get_raster_queue(const rive_cuda_context* ctx, int* enabled);

/*
 * Interior tiles as winding records (no counterpart in the reference; off by
 * default, an autotuner knob). Inside a fill, every midpoint-fan triangle has
 * coverage +1 or -1, so on a tile that no contour edge, AA ramp or contour
 * midpoint comes within 2 px of, the path's coverage count is the same
 * integer at every pixel: the winding number of the fan's boundary. With this
 * on, such tiles get one winding entry per path instead of every fan
 * triangle that crosses them (fills that are not nested clip updates, whose
 * contour is short enough for their box to have interior tiles, in batches
 * without feathers). It pays on large filled shapes; on scribbles and small
 * flushes its extra passes cost more than they save. The image is
 * bit-identical either way.
 */
int rive_cuda_set_winding_tiles(rive_cuda_context* ctx, int enabled);
int rive_cuda_get_winding_tiles(const rive_cuda_context* ctx, int* enabled);

/*
 * Speculative bins (no counterpart in the reference; on by default). A flush
 * on the context's own stream sizes its bins from the largest bin-entry total
 * the context has seen (plus a quarter) instead of waiting for the scan's
 * total, so rive_cuda_flush returns without waiting for the device and the
 * caller can write the next frame's records while this one renders. The
 * total is checked at the next call into the context; when it did not fit,
 * the flush's back half runs again with exact bins before anything else, and
 * read-backs enqueued after it are repeated. The image is the same either
 * way. A caller that reads a target's device memory itself
 * (rive_cuda_render_target_device_ptr) calls rive_cuda_sync first, which
 * settles it. Flushes on a caller's stream and batches always size bins
 * exactly.
 */
int rive_cuda_set_bin_speculation(rive_cuda_context* ctx, int enabled);
int rive_cuda_get_bin_speculation(const rive_cuda_context* ctx, int* enabled);

/*
 * Per-stage device timing with CUDA events recorded on the flush stream
 * (off by default; no counterpart in the reference, whose backends time
 * nothing). Stages of one flush, in launch order:
 */
enum
{
    RIVE_CUDA_STAGE_COLOR_RAMP = 0,  /* color_ramp_kernel                 */
    RIVE_CUDA_STAGE_TESSELLATE = 1,  /* tessellate_kernel                 */
    RIVE_CUDA_STAGE_PATCH_SETUP = 2, /* patch_setup_kernel                */
    RIVE_CUDA_STAGE_BIN = 3,         /* scan + bin_scatter_kernel         */
    RIVE_CUDA_STAGE_SORT = 4,        /* radix sort + tile_ranges_kernel   */
    RIVE_CUDA_STAGE_RASTER = 5,      /* raster_tile_kernel                */
    RIVE_CUDA_STAGE_COUNT = 6,
};
int rive_cuda_set_profiling(rive_cuda_context* ctx, int enabled);
/* Waits for the recorded events, returns the summed milliseconds and launch
 * counts per stage since the last collect, and clears them. */
int rive_cuda_profile_collect(rive_cuda_context* ctx,
                              double ms[RIVE_CUDA_STAGE_COUNT],
                              uint64_t launches[RIVE_CUDA_STAGE_COUNT]);

#ifdef __cplusplus
}
#endif

#endif /* RIVE_CUDA_H */
