"""Regenerates the golden flush captures in this directory.

Each fixture pair is <name>.scene (a seeded rive_scene.h recording written by
the scene generator) and <name>.cap: what rive-runtime's own, unmodified CPU
front end (RiveRenderer -> RenderContext, compiled from its sources by
oracle/Makefile into oracle/_ref/ref_capture) hands its RenderContextImpl for
that scene (for the silver_* fixtures, a frame of one of the reference's
recorded .sriv animations). Needs the reference sources, so it runs only where
they exist:

    python tests/golden/make_golden.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from conftest import load_package  # noqa: E402

pkg = load_package()
from rive_runtime_gb300 import scene  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle  # noqa: E402

SCENES = {
    # The plain small workload at full size: 512x512, 200 closed 8-cubic fills.
    "plain_small_s1": lambda: scene.plain_small(seed=1),
    # Full-feature distribution, shrunk: fills (nonzero/even-odd), strokes
    # (all joins and caps), gradients, blend modes, nested clips.
    "full_small_s7": lambda: scene.full_feature(seed=7, width=256, height=256, n_paths=40,
                                                max_cubics=12, scale_range=(0.5, 2.0)),
    # Odd canvas size (not a multiple of the tile), heavier blend/clip mix.
    "full_odd_s11": lambda: scene.full_feature(seed=11, width=300, height=200, n_paths=50,
                                               max_cubics=8, p_gradient=0.5, p_blend=0.5,
                                               p_clip=0.4, scale_range=(0.5, 2.0)),
    # Strokes only: every join and cap, thin to thick.
    "strokes_s3": lambda: scene.full_feature(seed=3, width=256, height=256, n_paths=40,
                                             max_cubics=6, p_fill=0.0, p_gradient=0.2,
                                             p_blend=0.0, p_clip=0.0, scale_range=(0.5, 2.0)),
    # Tessellation stress: cusps, near-degenerate cubics, round joins/caps.
    "stroke_stress_s5": lambda: scene.stroke_stress(seed=5, width=256, height=256, n_strokes=60),
    # Deep nested clipping.
    "clips_s13": lambda: scene.full_feature(seed=13, width=192, height=192, n_paths=30,
                                            max_cubics=6, p_clip=1.0, p_gradient=0.3,
                                            p_blend=0.2, scale_range=(0.75, 1.5)),
    # Interior triangulation (the front end's default for large fills): outer
    # curve patches plus interior triangles, on canvas-wide plain fills.
    "tri_fills_s21": lambda: _triangulated(scene.plain_canvas(
        __import__("numpy").random.default_rng(21), 640, 480, 10)),
    # ... and on scaled-up full-feature paths (even-odd, gradients, blend
    # modes, triangulated clip paths).
    "tri_full_s23": lambda: _triangulated(scene.full_feature(
        seed=23, width=512, height=512, n_paths=24, max_cubics=10, p_fill=0.8, p_clip=0.3,
        p_blend=0.3, scale_range=(6.0, 9.0))),
    # More complex gradients than the gradient texture has rows (2,048): the
    # front end splits the frame into two logical flushes
    # (LogicalFlush::pushDraws, render_context.cpp:509-586), and the second
    # loads the target the first wrote (render_context.cpp:1218-1222).
    "multiflush_s41": lambda: scene.full_feature(
        seed=41, width=256, height=256, n_paths=2450, max_contours=1, min_cubics=2,
        max_cubics=2, p_fill=0.85, p_gradient=1.0, p_clip=0.05, p_blend=0.1,
        scale_range=(0.15, 0.5)),
}


# Feathered strokes (RenderPaint::feather on strokes, radius x scale below the
# reference's 32-pixel feather-atlas threshold): ENABLE_FEATHER batches.
SCENES["feather_strokes_s31"] = lambda: scene.feathered_strokes(seed=31)
# Feathered fills and strokes (clockwise feathered fills, radius x scale below
# the atlas threshold): midpointFanCenterAAPatches batches beside the fans.
SCENES["feathered_s33"] = lambda: scene.feathered(seed=33)

# Frames of real content: the reference's own silver renderer-call streams
# (tests/unit_tests/silvers/*.sriv, recorded by its SerializingFactory while
# .riv artboards animate), read by rive_runtime_gb300.sriv. Their fills are
# mostly clockwise (FillRule::clockwise), with clip rects, nested clips,
# gradients, blend modes and modulated opacity. Image draws are left out of the
# scenes (not part of this path), and so are feathered draws except in the
# FEATHERED_SILVERS frames below.
SILVERS = {
    "silver_hunter_x_f0": ("hunter_x_demo", 0),
    "silver_rewards_f10": ("rewards_demo", 10),
    "silver_spotify_kids_f31": ("spotify_kids_demo", 31),
    "silver_echo_show_f0": ("echo_show_demo", 0),
    "silver_path_opacity_f30": ("script_path_opacity", 30),
    "silver_artboards_opacity_f30": ("script_artboards_opacity", 30),
}
SILVER_DIR = os.path.join(oracle.REFERENCE_SOURCES, "tests", "unit_tests", "silvers")


# Real frames whose feathered draws all stay below the feather atlas
# threshold, feathered draws kept: the reference front end draws their
# feathered fills as midpointFanCenterAAPatches batches.
FEATHERED_SILVERS = {
    "silver_path_effect_feathers_f30": ("path_effect_with_feathers", 30),
    "silver_text_feather_falloff_f30": ("text_feather_falloff", 30),
    "silver_police_files_f60": ("game_menu_ad_police_files", 60),
}


# Wide feathers through the feather atlas (radius x scale >= 32 px; the
# reference renders their coverage offscreen and blits it,
# render_context.cpp:676-744, 2255-2345, 3515-3534), beside direct feathers.
SCENES["feather_atlas_s35"] = lambda: scene.feathered_atlas(seed=35)
# feathered_s33 again, every feather through the atlas
# (PlatformFeatures::alwaysFeatherToAtlas): renders the same image as the
# direct feathers of feathered_s33, within the image tolerance.
SCENES["feathered_atlas_s33"] = lambda: _atlas_always(scene.feathered(seed=33))

# Images drawn with Renderer::drawImage (a rectangle path with an image paint
# in rasterOrdering, rive_renderer.cpp:383-446): every ImageSampler, magnified
# and minified (mip levels), opacity, blend modes, clips.
SCENES["images_s41"] = lambda: scene.images(seed=41)

# Image meshes drawn with Renderer::drawImageMesh (rive_renderer.cpp:448-495;
# draw_image_mesh.vert, draw_mesh.frag): warped grids and overlapping
# triangle soups, both windings, every ImageSampler, implicit mip levels,
# opacity, blend modes, clip paths and clip rects, beside drawImage draws.
SCENES["image_meshes_s43"] = lambda: scene.image_meshes(seed=43)
# Two overlapping mesh triangles of opposite windings: both are drawn and
# both blend where they overlap (a known answer).
SCENES["mesh_overlap"] = lambda: scene.mesh_overlap()

# Real frames whose wide feathers the reference front end sends through the
# feather atlas (feathered draws kept).
ATLAS_SILVERS = {
    "silver_data_viz_f6": ("data_viz_demo", 6),
    "silver_bankcard_f10": ("bankcard", 10),
    "silver_rewards_atlas_f10": ("rewards_demo", 10),
}


# Real frames with their images: the recorded PNG / JPEG bytes decoded
# (image_decode) and premultiplied as RenderContext::decodeImage does;
# drawImage draws and, in image_fit_alignment_2, a drawImageMesh with the
# RenderBuffer contents the stream recorded.
IMAGE_SILVERS = {
    "silver_image_mesh_f10": ("image_fit_alignment_2", 10),
    "silver_clipping_images_f6": ("clipping_and_draw_order", 6),
    "silver_superbowl_images_f5": ("superbowl", 5),
}


def _atlas_always(sc):
    sc.flags = scene.FLAG_FEATHER_ATLAS
    return sc


def _silver(stream, frame, keep_feathered=False, images=False):
    from rive_runtime_gb300 import sriv
    with open(os.path.join(SILVER_DIR, stream + ".sriv"), "rb") as f:
        st = sriv.read_sriv(f.read())
    return st.frame_scene(frame, keep_feathered=keep_feathered, images=images)[0]


for _name, (_stream, _frame) in SILVERS.items():
    SCENES[_name] = (lambda s=_stream, k=_frame: _silver(s, k))
for _name, (_stream, _frame) in FEATHERED_SILVERS.items():
    SCENES[_name] = (lambda s=_stream, k=_frame: _silver(s, k, keep_feathered=True))
for _name, (_stream, _frame) in ATLAS_SILVERS.items():
    SCENES[_name] = (lambda s=_stream, k=_frame: _silver(s, k, keep_feathered=True))
for _name, (_stream, _frame) in IMAGE_SILVERS.items():
    SCENES[_name] = (lambda s=_stream, k=_frame: _silver(s, k, keep_feathered=True, images=True))


def _triangulated(sc):
    sc.flags = scene.FLAG_TRIANGULATE
    return sc


def main(only=None):
    for name, make in SCENES.items():
        if only and name not in only:
            continue
        sc = make()
        sb = sc.to_bytes()
        cb = oracle.reference_capture(sb)
        with open(os.path.join(HERE, name + ".scene"), "wb") as f:
            f.write(sb)
        with open(os.path.join(HERE, name + ".cap"), "wb") as f:
            f.write(cb)
        print(f"{name}: scene {len(sb)} B, capture {len(cb)} B")


if __name__ == "__main__":
    main(sys.argv[1:])
