/*
 * adapter_capture -- TEST INFRASTRUCTURE (oracle). Replays a rive_scene.h
 * recording through the reference's own RiveRenderer and RenderContext into
 * the product's RenderContextCUDAImpl, linked against abi_recorder.c instead
 * of librive_cuda.so, and writes what reached the C ABI in the capture
 * layout of ref_capture. The two captures of one scene must be identical.
 *
 * Usage: adapter_capture <scene.bin> <capture.bin>
 */
#include "render_context_cuda_impl.hpp"
#include "scene_replay.hpp"

#include <cstdio>
#include <cstring>
#include <vector>

extern "C" int abi_recorder_write(const char* path);

int main(int argc, char** argv)
{
    if (argc != 3)
    {
        fprintf(stderr, "usage: adapter_capture <scene.bin> <capture.bin>\n");
        return 1;
    }
    std::vector<uint8_t> scene;
    if (FILE* f = fopen(argv[1], "rb"))
    {
        fseek(f, 0, SEEK_END);
        scene.resize(static_cast<size_t>(ftell(f)));
        fseek(f, 0, SEEK_SET);
        if (fread(scene.data(), 1, scene.size(), f) != scene.size())
            scene.clear();
        fclose(f);
    }
    std::unique_ptr<rive::gpu::RenderContext> ctx = rive::gpu::RenderContextCUDAImpl::MakeContext(0);
    if (!ctx)
        return 1;
    auto* impl = ctx->static_impl_cast<rive::gpu::RenderContextCUDAImpl>();
    if (scene.size() >= sizeof(rive_scene_header))
    {
        rive_scene_header hdr;
        memcpy(&hdr, scene.data(), sizeof(hdr));
        impl->setAlwaysFeatherToAtlas((hdr.flags & RIVE_SCENE_FLAG_FEATHER_ATLAS) != 0);
    }
    const char* err = replay_scene(ctx.get(), scene, [&](uint32_t w, uint32_t h) {
        return rive::rcp<rive::gpu::RenderTarget>(impl->makeRenderTarget(w, h));
    });
    if (err)
    {
        fprintf(stderr, "adapter_capture: %s\n", err);
        return 1;
    }
    if (impl->lastStatus() != RIVE_CUDA_OK)
    {
        fprintf(stderr, "adapter_capture: backend status %d\n", impl->lastStatus());
        return 1;
    }
    return abi_recorder_write(argv[2]);
}
