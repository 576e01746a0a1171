/*
 * capture_format.h -- TEST INFRASTRUCTURE (oracle). The flush part of the
 * capture layout, shared by ref_capture / cmdbuf_capture (capture_impl.hpp)
 * and the product-adapter recorder (abi_recorder.c), so that both write the
 * same bytes for the same flushes.
 *
 * Per flush:
 *   the rive_cuda_flush_desc fields up to and including draw_batches
 *   (RIVE_CAPTURE_DESC_BYTES, the pointer written as 0),
 *   rive_cuda_draw_batch[draw_batch_count],
 * and, in an 'RCP2' capture (one whose frame renders into the feather atlas
 * or draws images):
 *   u32 atlas_texture_width, atlas_texture_height, atlas_content_width,
 *   atlas_content_height, atlas_fill_batch_count, atlas_stroke_batch_count,
 *   rive_cuda_atlas_batch[fill + stroke],
 *   u32 image_count (draw_batch_count, or 0 when no batch draws an image),
 *   image_count x { u32 texture index (0xffffffff: none), u32 sampler key }.
 * After the flushes an RCP2 capture lists its textures:
 *   u32 texture_count,
 *   texture_count x { u32 width, u32 height, u32 mip_levels,
 *                     uint8_t rgba[width * height * 4] (level 0) }.
 * An 'RCP3' capture (a frame that draws image meshes) is an RCP2 capture with,
 * per flush after its images:
 *   u32 mesh_count (draw_batch_count, or 0 when no batch draws a mesh),
 *   mesh_count x { u32 vertex buffer, u32 uv buffer, u32 index buffer
 *                  (render-buffer indices, 0xffffffff: not a mesh),
 *                  u32 index count },
 * and after the textures the render buffers the flushes drew:
 *   u32 buffer_count,
 *   buffer_count x { u32 type (rive::RenderBufferType), u32 bytes,
 *                    uint8_t data[bytes] (padded to 4 bytes) }.
 * A frame without atlas draws or images keeps the 'RCP1' layout byte for byte.
 */
#ifndef RIVE_CAPTURE_FORMAT_H
#define RIVE_CAPTURE_FORMAT_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "rive_cuda.h"

#define RIVE_CAPTURE_MAGIC_V1 0x31504352u /* "RCP1" */
#define RIVE_CAPTURE_MAGIC_V2 0x32504352u /* "RCP2": with feather atlas batches */
#define RIVE_CAPTURE_MAGIC_V3 0x33504352u /* "RCP3": RCP2 with image meshes */
#define RIVE_CAPTURE_DESC_BYTES offsetof(rive_cuda_flush_desc, atlas_texture_width)

static inline int rive_capture_flush_has_atlas(const rive_cuda_flush_desc* d)
{
    return d->atlas_fill_batch_count != 0 || d->atlas_stroke_batch_count != 0 ||
           d->atlas_content_width != 0 || d->atlas_content_height != 0;
}

/* Writes one flush (`d`'s pointers are ignored; the arrays come separately). */
static inline void rive_capture_write_flush(FILE* f,
                                            const rive_cuda_flush_desc* d,
                                            const rive_cuda_draw_batch* batches,
                                            const rive_cuda_atlas_batch* atlas,
                                            const uint32_t* images, /* 2 per batch, or NULL */
                                            const uint32_t* meshes, /* 4 per batch, or NULL */
                                            int v2,
                                            int v3)
{
    rive_cuda_flush_desc o;
    memcpy(&o, d, sizeof(o));
    o.draw_batches = NULL;
    o.atlas_batches = NULL;
    o.batch_images = NULL;
    fwrite(&o, RIVE_CAPTURE_DESC_BYTES, 1, f);
    if (d->draw_batch_count)
        fwrite(batches, sizeof(rive_cuda_draw_batch), d->draw_batch_count, f);
    if (v2)
    {
        const uint32_t a[6] = {d->atlas_texture_width,   d->atlas_texture_height,
                               d->atlas_content_width,   d->atlas_content_height,
                               d->atlas_fill_batch_count, d->atlas_stroke_batch_count};
        fwrite(a, sizeof(a), 1, f);
        const uint32_t na = d->atlas_fill_batch_count + d->atlas_stroke_batch_count;
        if (na)
            fwrite(atlas, sizeof(rive_cuda_atlas_batch), na, f);
        const uint32_t ni = images ? d->draw_batch_count : 0u;
        fwrite(&ni, 4, 1, f);
        if (ni)
            fwrite(images, 8, ni, f);
    }
    if (v3)
    {
        const uint32_t nm = meshes ? d->draw_batch_count : 0u;
        fwrite(&nm, 4, 1, f);
        if (nm)
            fwrite(meshes, 16, nm, f);
    }
}

/* The texture table at the end of an RCP2 capture. */
static inline void rive_capture_write_textures(FILE* f,
                                               uint32_t count,
                                               const uint32_t* dims, /* w, h, levels per texture */
                                               const uint8_t* const* texels)
{
    fwrite(&count, 4, 1, f);
    for (uint32_t i = 0; i < count; ++i)
    {
        fwrite(dims + 3 * i, 4, 3, f);
        fwrite(texels[i], 1, (size_t)dims[3 * i] * dims[3 * i + 1] * 4, f);
    }
}

/* The render-buffer table at the end of an RCP3 capture. */
static inline void rive_capture_write_render_buffers(FILE* f,
                                                     uint32_t count,
                                                     const uint32_t* types,
                                                     const uint32_t* sizes,
                                                     const uint8_t* const* data)
{
    static const uint8_t zeros[4] = {0, 0, 0, 0};
    fwrite(&count, 4, 1, f);
    for (uint32_t i = 0; i < count; ++i)
    {
        const uint32_t head[2] = {types[i], sizes[i]};
        fwrite(head, 4, 2, f);
        if (sizes[i])
            fwrite(data[i], 1, sizes[i], f);
        fwrite(zeros, 1, (4 - (sizes[i] & 3)) & 3, f);
    }
}

#endif /* RIVE_CAPTURE_FORMAT_H */
