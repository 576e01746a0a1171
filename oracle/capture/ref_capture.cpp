/*
 * ref_capture -- TEST INFRASTRUCTURE (oracle). Never linked into the product.
 *
 * Replays a rive_scene.h recording through rive-runtime's own, unmodified CPU
 * front end (RiveRenderer -> RenderContext, renderer/src/rive_renderer.cpp and
 * renderer/src/render_context.cpp) into a RenderContextImpl that records every
 * buffer it is handed and every FlushDescriptor (render_context_impl.hpp:217).
 * The recording ("capture") is the golden INPUT of the device passes and the
 * golden OUTPUT of this project's own planner.
 *
 * Built by oracle/Makefile from the reference sources where they lie; the
 * binary lands in oracle/_ref/ and is never committed.
 *
 * Usage: ref_capture <scene.bin> <capture.bin>
 *
 * Capture file layout (little-endian):
 *   u32 magic 'RCP1' ('RCP2' when the frame renders into the feather atlas),
 *   u32 width, u32 height, u32 buffer_kinds (7, or 8 when the frame has
 *   interior triangles or atlas blits)
 *   buffer_kinds x { u64 bytes, bytes of data, zero pad to 8 }  in rive_cuda.h order
 *   u32 flush_count
 *   flush_count x { the flush (capture_format.h) }
 */
#include "capture_impl.hpp"
#include "scene_replay.hpp"

using namespace capture;

namespace
{
int fail(const char* msg)
{
    fprintf(stderr, "ref_capture: %s\n", msg);
    return 1;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc != 3)
        return fail("usage: ref_capture <scene.bin> <capture.bin>");
    std::vector<uint8_t> scene = read_file(argv[1]);
    if (scene.size() < sizeof(rive_scene_header))
        return fail("cannot read scene");
    CaptureImpl* impl = nullptr;
    std::unique_ptr<RenderContext> ctx = CaptureImpl::Make(&impl);
    rive_scene_header hdr;
    memcpy(&hdr, scene.data(), sizeof(hdr));
    impl->setAlwaysFeatherToAtlas((hdr.flags & RIVE_SCENE_FLAG_FEATHER_ATLAS) != 0);
    const char* err = replay_scene(ctx.get(), scene, [&](uint32_t w, uint32_t h) {
        return rcp<RenderTarget>(impl->makeRenderTarget(w, h));
    });
    if (err)
        return fail(err);

    if (!write_capture(argv[2], *impl, hdr.width, hdr.height))
        return fail("cannot open output");
    return 0;
}
