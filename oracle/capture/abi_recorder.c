/*
 * abi_recorder.c -- TEST INFRASTRUCTURE (oracle). A recording stand-in for
 * the rive_cuda.h entry points that RenderContextCUDAImpl calls: it runs no
 * GPU work, keeps the bytes each record buffer holds at unmap and every
 * flush descriptor with its draw batches, and writes them in the capture
 * layout of ref_capture.cpp. Linked with the reference front end and the
 * product's RenderContextCUDAImpl, it shows that the backend hands the
 * C ABI exactly what the reference's RenderContext produced.
 */
#include "rive_cuda.h"
#include "capture_format.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define KINDS RIVE_CUDA_BUFFER_KIND_COUNT
#define CAPTURED_KINDS 7 /* flush uniforms .. tess spans (+ triangle vertices, image draws) */
#define MAX_FLUSHES 256
#define MAX_TEXTURES 4096
#define MAX_SNAPSHOTS 4096

struct rive_cuda_texture
{
    uint32_t index; /* in the context's texture table */
};

/* A render buffer: its bytes, and a version each write advances. */
struct rive_cuda_render_buffer
{
    uint32_t type;
    size_t bytes;
    unsigned char* data;
    uint64_t id, version;
};

struct rive_cuda_context
{
    unsigned char* staging[KINDS];
    size_t capacity[KINDS];
    unsigned char* data[KINDS]; /* bytes at the last unmap */
    size_t bytes[KINDS];
    uint32_t flush_count;
    rive_cuda_flush_desc descs[MAX_FLUSHES];
    rive_cuda_draw_batch* batches[MAX_FLUSHES];
    rive_cuda_atlas_batch* atlas[MAX_FLUSHES];
    uint32_t* images[MAX_FLUSHES]; /* 2 per batch, or NULL */
    uint32_t texture_count;
    uint32_t texture_dims[3 * MAX_TEXTURES];
    unsigned char* texture_texels[MAX_TEXTURES];
    rive_cuda_texture* textures[MAX_TEXTURES];
    uint32_t* meshes[MAX_FLUSHES]; /* 4 per batch, or NULL */
    /* Render-buffer contents the flushes drew (one per buffer and version). */
    uint32_t snapshot_count;
    uint64_t snapshot_id[MAX_SNAPSHOTS], snapshot_version[MAX_SNAPSHOTS];
    uint32_t snapshot_type[MAX_SNAPSHOTS], snapshot_bytes[MAX_SNAPSHOTS];
    unsigned char* snapshot_data[MAX_SNAPSHOTS];
    uint64_t next_buffer_id;
    uint32_t width, height;
    int failed;
};

struct rive_cuda_render_target
{
    uint32_t width, height;
};

static rive_cuda_context* g_last; /* the context abi_recorder_write dumps */

int rive_cuda_context_create(int device, rive_cuda_context** out)
{
    (void)device;
    if (!out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out = (rive_cuda_context*)calloc(1, sizeof(rive_cuda_context));
    g_last = *out;
    return *out ? RIVE_CUDA_OK : RIVE_CUDA_ERR_OUT_OF_MEMORY;
}

void rive_cuda_context_destroy(rive_cuda_context* ctx)
{
    if (!ctx)
        return;
    for (int k = 0; k < KINDS; ++k)
    {
        free(ctx->staging[k]);
        free(ctx->data[k]);
    }
    for (uint32_t i = 0; i < ctx->flush_count; ++i)
    {
        free(ctx->batches[i]);
        free(ctx->atlas[i]);
        free(ctx->images[i]);
        free(ctx->meshes[i]);
    }
    for (uint32_t i = 0; i < ctx->snapshot_count; ++i)
        free(ctx->snapshot_data[i]);
    for (uint32_t i = 0; i < ctx->texture_count; ++i)
    {
        free(ctx->texture_texels[i]);
        free(ctx->textures[i]);
    }
    if (g_last == ctx)
        g_last = NULL;
    free(ctx);
}

int rive_cuda_texture_create(rive_cuda_context* ctx,
                             uint32_t width,
                             uint32_t height,
                             uint32_t mip_levels,
                             const void* rgba_host,
                             rive_cuda_texture** out)
{
    if (!ctx || !out || !rgba_host || ctx->texture_count >= MAX_TEXTURES)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    const uint32_t i = ctx->texture_count;
    const size_t bytes = (size_t)width * height * 4;
    rive_cuda_texture* t = (rive_cuda_texture*)malloc(sizeof(rive_cuda_texture));
    unsigned char* texels = (unsigned char*)malloc(bytes ? bytes : 1);
    if (!t || !texels)
    {
        free(t);
        free(texels);
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    }
    memcpy(texels, rgba_host, bytes);
    t->index = i;
    ctx->texture_dims[3 * i] = width;
    ctx->texture_dims[3 * i + 1] = height;
    ctx->texture_dims[3 * i + 2] = mip_levels;
    ctx->texture_texels[i] = texels;
    ctx->textures[i] = t;
    ctx->texture_count = i + 1;
    *out = t;
    return RIVE_CUDA_OK;
}

/* Textures stay recorded until the context goes (the capture lists them). */
void rive_cuda_texture_destroy(rive_cuda_context* ctx, rive_cuda_texture* texture)
{
    (void)ctx, (void)texture;
}

int rive_cuda_render_buffer_create(rive_cuda_context* ctx,
                                   uint32_t type,
                                   size_t bytes,
                                   rive_cuda_render_buffer** out)
{
    if (!ctx || !out || bytes == 0)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    rive_cuda_render_buffer* b = (rive_cuda_render_buffer*)calloc(1, sizeof(*b));
    unsigned char* data = (unsigned char*)calloc(1, bytes);
    if (!b || !data)
    {
        free(b);
        free(data);
        return RIVE_CUDA_ERR_OUT_OF_MEMORY;
    }
    b->type = type;
    b->bytes = bytes;
    b->data = data;
    b->id = ctx->next_buffer_id++;
    *out = b;
    return RIVE_CUDA_OK;
}

int rive_cuda_render_buffer_write(rive_cuda_context* ctx,
                                  rive_cuda_render_buffer* b,
                                  size_t offset,
                                  const void* src,
                                  size_t bytes)
{
    if (!ctx || !b || offset > b->bytes || bytes > b->bytes - offset || (!src && bytes))
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    if (bytes)
        memcpy(b->data + offset, src, bytes);
    ++b->version;
    return RIVE_CUDA_OK;
}

void rive_cuda_render_buffer_destroy(rive_cuda_context* ctx, rive_cuda_render_buffer* b)
{
    (void)ctx;
    if (!b)
        return;
    free(b->data);
    free(b);
}

/* The snapshot index of a buffer's current contents (recorded on first use). */
static uint32_t snapshot(rive_cuda_context* ctx, const rive_cuda_render_buffer* b)
{
    for (uint32_t i = 0; i < ctx->snapshot_count; ++i)
        if (ctx->snapshot_id[i] == b->id && ctx->snapshot_version[i] == b->version)
            return i;
    if (ctx->snapshot_count >= MAX_SNAPSHOTS)
    {
        ctx->failed = 1;
        return 0xffffffffu;
    }
    const uint32_t i = ctx->snapshot_count++;
    ctx->snapshot_id[i] = b->id;
    ctx->snapshot_version[i] = b->version;
    ctx->snapshot_type[i] = b->type;
    ctx->snapshot_bytes[i] = (uint32_t)b->bytes;
    ctx->snapshot_data[i] = (unsigned char*)malloc(b->bytes);
    if (ctx->snapshot_data[i])
        memcpy(ctx->snapshot_data[i], b->data, b->bytes);
    else
        ctx->failed = 1;
    return i;
}

int rive_cuda_texture_read(rive_cuda_context* ctx,
                           const rive_cuda_texture* texture,
                           uint32_t level,
                           void* dst_host,
                           size_t bytes)
{
    (void)ctx, (void)texture, (void)level, (void)dst_host, (void)bytes;
    return RIVE_CUDA_ERR_UNSUPPORTED;
}

int rive_cuda_last_error(const rive_cuda_context* ctx, char* buf, size_t len)
{
    (void)ctx;
    if (buf && len)
        buf[0] = 0;
    return RIVE_CUDA_OK;
}

int rive_cuda_resize_buffer(rive_cuda_context* ctx, int kind, size_t bytes)
{
    if (!ctx || kind < 0 || kind >= KINDS)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    free(ctx->staging[kind]);
    ctx->staging[kind] = bytes ? (unsigned char*)malloc(bytes) : NULL;
    ctx->capacity[kind] = bytes;
    return RIVE_CUDA_OK;
}

void* rive_cuda_map_buffer(rive_cuda_context* ctx, int kind, size_t bytes)
{
    if (!ctx || kind < 0 || kind >= KINDS || bytes > ctx->capacity[kind] || !ctx->staging[kind])
        return NULL;
    /* Zeroed, as ref_capture's rings are, so skipped padding compares equal. */
    memset(ctx->staging[kind], 0, bytes);
    return ctx->staging[kind];
}

int rive_cuda_unmap_buffer(rive_cuda_context* ctx, int kind, size_t bytes)
{
    if (!ctx || kind < 0 || kind >= KINDS)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    free(ctx->data[kind]);
    ctx->data[kind] = (unsigned char*)malloc(bytes ? bytes : 1);
    if (bytes)
        memcpy(ctx->data[kind], ctx->staging[kind], bytes);
    ctx->bytes[kind] = bytes;
    return RIVE_CUDA_OK;
}

int rive_cuda_resize_gradient_texture(rive_cuda_context* ctx, uint32_t w, uint32_t h)
{
    (void)ctx, (void)w, (void)h;
    return RIVE_CUDA_OK;
}

int rive_cuda_resize_tessellation_texture(rive_cuda_context* ctx, uint32_t w, uint32_t h)
{
    (void)ctx, (void)w, (void)h;
    return RIVE_CUDA_OK;
}

int rive_cuda_render_target_create(rive_cuda_context* ctx,
                                   uint32_t width,
                                   uint32_t height,
                                   rive_cuda_render_target** out)
{
    if (!ctx || !out)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    *out = (rive_cuda_render_target*)calloc(1, sizeof(rive_cuda_render_target));
    (*out)->width = width;
    (*out)->height = height;
    ctx->width = width;
    ctx->height = height;
    return RIVE_CUDA_OK;
}

void rive_cuda_render_target_destroy(rive_cuda_context* ctx, rive_cuda_render_target* t)
{
    (void)ctx;
    free(t);
}

void* rive_cuda_render_target_device_ptr(rive_cuda_render_target* t)
{
    (void)t;
    return NULL;
}

int rive_cuda_render_target_read(rive_cuda_context* ctx,
                                 rive_cuda_render_target* t,
                                 void* dst,
                                 void* stream)
{
    (void)ctx, (void)t, (void)dst, (void)stream;
    return RIVE_CUDA_ERR_UNSUPPORTED;
}

int rive_cuda_flush(rive_cuda_context* ctx,
                    const rive_cuda_flush_desc* desc,
                    rive_cuda_render_target* target,
                    void* stream)
{
    (void)target, (void)stream;
    if (!ctx || !desc || ctx->flush_count >= MAX_FLUSHES)
        return RIVE_CUDA_ERR_INVALID_ARGUMENT;
    uint32_t i = ctx->flush_count++;
    ctx->descs[i] = *desc;
    ctx->descs[i].draw_batches = NULL;
    size_t n = desc->draw_batch_count;
    ctx->batches[i] = (rive_cuda_draw_batch*)malloc(n ? n * sizeof(rive_cuda_draw_batch) : 1);
    if (n)
        memcpy(ctx->batches[i], desc->draw_batches, n * sizeof(rive_cuda_draw_batch));
    size_t na = (size_t)desc->atlas_fill_batch_count + desc->atlas_stroke_batch_count;
    ctx->descs[i].atlas_batches = NULL;
    ctx->atlas[i] = (rive_cuda_atlas_batch*)malloc(na ? na * sizeof(rive_cuda_atlas_batch) : 1);
    if (na)
        memcpy(ctx->atlas[i], desc->atlas_batches, na * sizeof(rive_cuda_atlas_batch));
    ctx->descs[i].batch_images = NULL;
    ctx->images[i] = NULL;
    if (desc->batch_images && n)
    {
        int any = 0;
        uint32_t* im = (uint32_t*)malloc(n * 8);
        if (!im)
            return RIVE_CUDA_ERR_OUT_OF_MEMORY;
        for (size_t b = 0; b < n; ++b)
        {
            const rive_cuda_texture* t = desc->batch_images[b].texture;
            im[2 * b] = t ? t->index : 0xffffffffu;
            im[2 * b + 1] = desc->batch_images[b].sampler_key;
            any = any || t != NULL;
        }
        if (any)
            ctx->images[i] = im;
        else
            free(im);
    }
    ctx->descs[i].batch_meshes = NULL;
    ctx->meshes[i] = NULL;
    if (desc->batch_meshes && n)
    {
        int any = 0;
        uint32_t* me = (uint32_t*)malloc(n * 16);
        if (!me)
            return RIVE_CUDA_ERR_OUT_OF_MEMORY;
        for (size_t b = 0; b < n; ++b)
        {
            const rive_cuda_batch_mesh* m = &desc->batch_meshes[b];
            if (m->vertices && m->uvs && m->indices)
            {
                me[4 * b] = snapshot(ctx, m->vertices);
                me[4 * b + 1] = snapshot(ctx, m->uvs);
                me[4 * b + 2] = snapshot(ctx, m->indices);
                me[4 * b + 3] = m->index_count;
                any = 1;
            }
            else
            {
                me[4 * b] = me[4 * b + 1] = me[4 * b + 2] = 0xffffffffu;
                me[4 * b + 3] = 0;
            }
        }
        if (any)
            ctx->meshes[i] = me;
        else
            free(me);
    }
    return RIVE_CUDA_OK;
}

int rive_cuda_sync(rive_cuda_context* ctx, void* stream)
{
    (void)ctx, (void)stream;
    return RIVE_CUDA_OK;
}

/* Writes the recording of the most recently created context. */
int abi_recorder_write(const char* path)
{
    rive_cuda_context* ctx = g_last;
    if (!ctx)
        return 1;
    FILE* f = fopen(path, "wb");
    if (!f)
        return 1;
    /* Seven kinds, eight when the frame has interior triangles, nine when it
     * has image draw instances. */
    const uint32_t kinds = ctx->bytes[CAPTURED_KINDS + 1]  ? CAPTURED_KINDS + 2
                           : ctx->bytes[CAPTURED_KINDS] ? CAPTURED_KINDS + 1
                                                        : CAPTURED_KINDS;
    if (ctx->failed)
    {
        fclose(f);
        return 1;
    }
    int v3 = ctx->snapshot_count != 0;
    for (uint32_t i = 0; i < ctx->flush_count; ++i)
        v3 = v3 || ctx->meshes[i] != NULL;
    int v2 = v3 || ctx->texture_count != 0;
    for (uint32_t i = 0; i < ctx->flush_count; ++i)
        v2 = v2 || rive_capture_flush_has_atlas(&ctx->descs[i]) || ctx->images[i] != NULL;
    uint32_t head[4] = {v3   ? RIVE_CAPTURE_MAGIC_V3
                        : v2 ? RIVE_CAPTURE_MAGIC_V2
                             : RIVE_CAPTURE_MAGIC_V1,
                        ctx->width, ctx->height, kinds};
    fwrite(head, sizeof(head), 1, f);
    static const unsigned char zeros[8] = {0};
    for (uint32_t k = 0; k < kinds; ++k)
    {
        uint64_t n = ctx->bytes[k];
        fwrite(&n, sizeof(n), 1, f);
        if (n)
            fwrite(ctx->data[k], 1, n, f);
        fwrite(zeros, 1, (8 - (n & 7)) & 7, f);
    }
    fwrite(&ctx->flush_count, sizeof(uint32_t), 1, f);
    for (uint32_t i = 0; i < ctx->flush_count; ++i)
        rive_capture_write_flush(f, &ctx->descs[i], ctx->batches[i], ctx->atlas[i], ctx->images[i],
                                 ctx->meshes[i], v2, v3);
    if (v2)
        rive_capture_write_textures(f, ctx->texture_count, ctx->texture_dims,
                                    (const uint8_t* const*)ctx->texture_texels);
    if (v3)
        rive_capture_write_render_buffers(f, ctx->snapshot_count, ctx->snapshot_type,
                                          ctx->snapshot_bytes,
                                          (const uint8_t* const*)ctx->snapshot_data);
    fclose(f);
    return 0;
}
