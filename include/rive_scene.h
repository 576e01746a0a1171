/*
 * rive_scene.h -- a flat, pointer-free recording of the rive::Renderer /
 * rive::Factory calls that make one frame (include/rive/renderer.hpp:212-236,
 * include/rive/factory.hpp:35-87).
 *
 * It is the input format of the planner (rive-runtime_gb300/csrc/planner) and
 * of the reference front-end replay that pins it. Python's scene generator
 * writes it. All fields are little-endian and 4-byte aligned.
 *
 *   rive_scene_header
 *   rive_scene_path[path_count]
 *   rive_scene_paint[paint_count]
 *   rive_scene_cmd[cmd_count]
 *   uint8_t verbs[verb_count]          (padded to a multiple of 4 bytes)
 *   float   points[point_count * 2]
 *   rive_scene_stop stops[stop_count]
 * and, only when the frame draws images:
 *   rive_scene_images { magic "RSI1", count }
 *   count x { rive_scene_image, uint8_t rgba[width * height * 4] }
 * and after them, only when the frame draws image meshes:
 *   rive_scene_meshes { magic "RSM1", count }
 *   count x { rive_scene_mesh, float xy[vertex_count * 2],
 *             float uv[vertex_count * 2],
 *             uint16_t indices[index_count] (padded to 4 bytes) }
 */
#ifndef RIVE_SCENE_H
#define RIVE_SCENE_H

#include <stdint.h>

#define RIVE_SCENE_MAGIC 0x31435352u /* "RSC1" */

/* rive::PathVerb (include/rive/math/path_types.hpp). */
enum
{
    RIVE_SCENE_VERB_MOVE = 0,
    RIVE_SCENE_VERB_LINE = 1,
    RIVE_SCENE_VERB_QUAD = 2,
    RIVE_SCENE_VERB_CUBIC = 4,
    RIVE_SCENE_VERB_CLOSE = 5,
};

/* Renderer calls. */
enum
{
    RIVE_SCENE_CMD_SAVE = 0,
    RIVE_SCENE_CMD_RESTORE = 1,
    RIVE_SCENE_CMD_TRANSFORM = 2, /* m[6] = xx, xy, yx, yy, tx, ty */
    RIVE_SCENE_CMD_DRAW_PATH = 3, /* a = path index, b = paint index */
    RIVE_SCENE_CMD_CLIP_PATH = 4, /* a = path index */
    RIVE_SCENE_CMD_MODULATE_OPACITY = 5, /* m[0] = opacity (Renderer::modulateOpacity) */
    /* Renderer::drawImage (renderer.hpp:216-219): a = image index, b = blend
     * mode | ImageSampler key << 8, m[0] = opacity. The image covers the unit
     * square scaled to its size under the current transform. */
    RIVE_SCENE_CMD_DRAW_IMAGE = 6,
    /* Renderer::drawImageMesh (renderer.hpp:222-230): a = image index, b =
     * blend mode | ImageSampler key << 8, m[0] = opacity, m[1] = mesh index
     * (an integer held exactly in the float). The mesh's vertex, uv and index
     * data become three RenderBuffers. */
    RIVE_SCENE_CMD_DRAW_IMAGE_MESH = 7,
};

/* rive::RenderPaintStyle / gradient kinds. */
enum
{
    RIVE_SCENE_STYLE_STROKE = 0,
    RIVE_SCENE_STYLE_FILL = 1,
    RIVE_SCENE_SHADER_NONE = 0,
    RIVE_SCENE_SHADER_LINEAR = 1,
    RIVE_SCENE_SHADER_RADIAL = 2,
};

typedef struct rive_scene_header
{
    uint32_t magic;
    uint32_t width;
    uint32_t height;
    uint32_t clear_color; /* rive::ColorInt 0xAARRGGBB */
    uint32_t path_count;
    uint32_t paint_count;
    uint32_t cmd_count;
    uint32_t verb_count;
    uint32_t point_count;
    uint32_t stop_count;
    uint32_t dither_mode; /* gpu::DitherMode: 0 none, 1 IGN */
    uint32_t flags;       /* RIVE_SCENE_FLAG_* */
} rive_scene_header;

/* Let the front end triangulate the interiors of large fills: the frame is
 * recorded with TriangulationThresholds::frameBudgetMs = infinity (every
 * eligible path, independent of timing; triangulation_controller.cpp), so it
 * draws outer-curve patches plus interior triangles for them. Without it,
 * frameBudgetMs = 0 and every fill is a midpoint fan. */
#define RIVE_SCENE_FLAG_TRIANGULATE 1u

/* Draw every feathered path through the feather atlas, whatever its radius:
 * the frame is recorded with PlatformFeatures::alwaysFeatherToAtlas
 * (gpu.hpp:156-158). Without it only blurs the front end scales to half
 * resolution or less go to the atlas (radius x scale >= 32 px). */
#define RIVE_SCENE_FLAG_FEATHER_ATLAS 2u

/* In rive_scene_path.fill_rule: the path was built the way a replayed call
 * stream builds it, Factory::makeEmptyRenderPath + RenderPath::addRawPath,
 * which keeps empty segments; without it the path is made by
 * Factory::makeRenderPath, which prunes them (RiveRenderPath's constructor,
 * renderer/src/rive_render_path.cpp:16-21). */
#define RIVE_SCENE_PATH_APPENDED 0x100u
#define RIVE_SCENE_FILL_RULE_MASK 0xffu

typedef struct rive_scene_path
{
    uint32_t verb_offset;
    uint32_t verb_count;
    uint32_t point_offset;
    uint32_t point_count;
    uint32_t fill_rule; /* rive::FillRule: 0 nonZero, 1 evenOdd, 2 clockwise,
                           | RIVE_SCENE_PATH_APPENDED */
} rive_scene_path;

typedef struct rive_scene_paint
{
    uint32_t style;      /* RIVE_SCENE_STYLE_* */
    uint32_t color;      /* rive::ColorInt */
    float thickness;
    uint32_t join;       /* rive::StrokeJoin: 0 miter, 1 round, 2 bevel */
    uint32_t cap;        /* rive::StrokeCap: 0 butt, 1 round, 2 square */
    uint32_t blend_mode; /* rive::BlendMode enum value (3 = srcOver) */
    uint32_t shader;     /* RIVE_SCENE_SHADER_* */
    float g[4];          /* linear: sx, sy, ex, ey; radial: cx, cy, r, 0 */
    uint32_t stop_offset;
    uint32_t stop_count;
    float feather;       /* RenderPaint::feather (blur width; 0 = none) */
} rive_scene_paint;

typedef struct rive_scene_cmd
{
    uint32_t op;
    uint32_t a;
    uint32_t b;
    float m[6];
} rive_scene_cmd;

typedef struct rive_scene_stop
{
    float position;
    uint32_t color; /* rive::ColorInt */
} rive_scene_stop;

#define RIVE_SCENE_IMAGES_MAGIC 0x31495352u /* "RSI1" */

typedef struct rive_scene_images
{
    uint32_t magic;
    uint32_t count;
} rive_scene_images;

/* An image: RGBA8 premultiplied texels, row 0 at the top, handed to
 * RenderContextImpl::makeImageTexture as one level; the backend makes the
 * other mip levels (generateRemainingMips). */
typedef struct rive_scene_image
{
    uint32_t width;
    uint32_t height;
} rive_scene_image;

#define RIVE_SCENE_MESHES_MAGIC 0x314d5352u /* "RSM1" */

typedef struct rive_scene_meshes
{
    uint32_t magic;
    uint32_t count;
} rive_scene_meshes;

/* A mesh: local positions, texture coordinates (normalised; the sampler
 * wraps them) and a triangle list. */
typedef struct rive_scene_mesh
{
    uint32_t vertex_count;
    uint32_t index_count;
} rive_scene_mesh;

#endif /* RIVE_SCENE_H */
