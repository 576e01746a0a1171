/*
 * cmdbuf_capture -- TEST INFRASTRUCTURE (oracle). Never linked into the
 * product. The reference's deferred 2D command buffer
 * (renderer/include/rive/renderer/cmd/render_command_buffer.hpp), both ends:
 *
 *   cmdbuf_capture record <scene.bin> <out.rcb>
 *       Replays a rive_scene.h recording into the reference's DeferredFactory
 *       and DeferredRenderer (cmd/deferred_render_factory.hpp) and stores the
 *       command bytes and blob arena they recorded.
 *   cmdbuf_capture replay <in.rcb> <capture.bin>
 *       Replays a stored stream with the reference's own replayRenderCommands
 *       (cmd/render_replay.hpp, renderer/src/deferred_cmd.cpp) into
 *       RiveRenderer -> RenderContext with the recording RenderContextImpl and
 *       writes the capture (layout in ref_capture.cpp).
 *   cmdbuf_capture record-sriv <in.sriv> <out.rcs>
 *       Replays a recorded .sriv animation with the reference's own
 *       replaySerializedCommands (utils/serialized_replay.cpp) into the
 *       deferred recorder, one command stream per frame (resetFrame at every
 *       frame op), as a session that keeps its resources across frames.
 *   cmdbuf_capture replay-frame <in.rcs> <k> <capture.bin>
 *       Consumes frames 0..k-1 of a stored session for their resources and
 *       destroys (filtered replays, version aliases cleared per frame, as the
 *       deferred host does) and captures frame k.
 *
 * .rcb layout (little-endian): u32 magic 'RCB1', u32 width, u32 height,
 * u32 clear colour, u32 dither mode, u32 scene flags, u64 command bytes,
 * u64 blob bytes, the command bytes, the blob bytes.
 * .rcs layout: u32 magic 'RCS1', width, height, clear colour, dither mode,
 * scene flags, frame count, 0; per frame u64 command bytes, u64 blob bytes,
 * the command bytes, the blob bytes.
 */
#include "capture_impl.hpp"
#include "scene_replay.hpp"

#include "rive/renderer/cmd/deferred_render_factory.hpp"
#include "rive/renderer/cmd/render_replay.hpp"
#include "utils/serialized_replay.hpp"

#include <string>

using namespace capture;

namespace
{
constexpr uint32_t kRcbMagic = 0x31424352u; // "RCB1"
constexpr uint32_t kRcsMagic = 0x31534352u; // "RCS1"

struct RcbHeader
{
    uint32_t magic, width, height, clearColor, ditherMode, flags;
    uint64_t commandBytes, blobBytes;
};

int fail(const char* msg)
{
    fprintf(stderr, "cmdbuf_capture: %s\n", msg);
    return 1;
}

int record(const char* scenePath, const char* outPath)
{
    std::vector<uint8_t> scene = read_file(scenePath);
    SceneView v;
    if (const char* err = parse_scene(scene, &v))
        return fail(err);
    cmd::DeferredFactory df;
    std::unique_ptr<Renderer> dr = df.makeRenderer();
    SceneResources res;
    if (const char* err = make_scene_resources(&df, v, &res))
        return fail(err);
    if (const char* err = issue_scene_commands(dr.get(), v, res))
        return fail(err);
    dr.reset();
    const cmd::RenderCommandBuffer& buf = df.commandBuffer();
    Span<const uint8_t> cmds = buf.commandBytes(), blobs = buf.blobBytes();
    RcbHeader h{kRcbMagic,       v.hdr.width, v.hdr.height, v.hdr.clear_color, v.hdr.dither_mode,
                v.hdr.flags,     cmds.size(), blobs.size()};
    FILE* f = fopen(outPath, "wb");
    if (!f)
        return fail("cannot open output");
    fwrite(&h, sizeof(h), 1, f);
    if (cmds.size())
        fwrite(cmds.data(), 1, cmds.size(), f);
    if (blobs.size())
        fwrite(blobs.data(), 1, blobs.size(), f);
    fclose(f);
    return 0;
}

int replay(const char* rcbPath, const char* outPath)
{
    std::vector<uint8_t> data = read_file(rcbPath);
    RcbHeader h;
    if (data.size() < sizeof(h))
        return fail("cannot read stream");
    memcpy(&h, data.data(), sizeof(h));
    if (h.magic != kRcbMagic || sizeof(h) + h.commandBytes + h.blobBytes > data.size())
        return fail("bad stream");
    Span<const uint8_t> cmds(data.data() + sizeof(h), h.commandBytes);
    Span<const uint8_t> blobs(data.data() + sizeof(h) + h.commandBytes, h.blobBytes);
    CaptureImpl* impl = nullptr;
    std::unique_ptr<RenderContext> ctx = CaptureImpl::Make(&impl);
    impl->setAlwaysFeatherToAtlas((h.flags & RIVE_SCENE_FLAG_FEATHER_ATLAS) != 0);
    rcp<RenderTarget> target(impl->makeRenderTarget(h.width, h.height));
    ctx->beginFrame(scene_frame(h.width, h.height, h.clearColor, h.ditherMode, h.flags));
    {
        RiveRenderer renderer(ctx.get());
        cmd::ResourceTable table;
        cmd::replayRenderCommands(ctx.get(), &renderer, cmds, blobs, table);
    }
    ctx->flush({.renderTarget = target.get()});
    if (!write_capture(outPath, *impl, h.width, h.height))
        return fail("cannot open output");
    return 0;
}

struct Frame
{
    std::vector<uint8_t> commands, blobs;
};

int record_sriv(const char* srivPath, const char* outPath)
{
    std::vector<uint8_t> stream = read_file(srivPath);
    if (stream.empty())
        return fail("cannot read stream");
    cmd::DeferredFactory df;
    std::unique_ptr<Renderer> dr = df.makeRenderer();
    std::vector<Frame> frames;
    uint32_t width = 0, height = 0;
    auto take = [&]() {
        const cmd::RenderCommandBuffer& buf = df.commandBuffer();
        Frame f;
        f.commands.assign(buf.commandBytes().begin(), buf.commandBytes().end());
        f.blobs.assign(buf.blobBytes().begin(), buf.blobBytes().end());
        frames.push_back(std::move(f));
        df.resetFrame();
    };
    SerializedReplayHooks hooks;
    hooks.onFrame = take;
    hooks.onFrameSize = [&](uint32_t w, uint32_t h) {
        width = w;
        height = h;
    };
    if (!replaySerializedCommands(Span<const uint8_t>(stream.data(), stream.size()), &df, dr.get(),
                                  hooks))
        return fail("the .sriv stream did not replay");
    take(); // the last frame
    if (!width || !height)
        return fail("no frame size");
    FILE* f = fopen(outPath, "wb");
    if (!f)
        return fail("cannot open output");
    uint32_t head[8] = {kRcsMagic, width, height, 0u, 1u, 0u, (uint32_t)frames.size(), 0u};
    fwrite(head, sizeof(head), 1, f);
    for (const Frame& fr : frames)
    {
        uint64_t n[2] = {fr.commands.size(), fr.blobs.size()};
        fwrite(n, sizeof(n), 1, f);
        if (n[0])
            fwrite(fr.commands.data(), 1, n[0], f);
        if (n[1])
            fwrite(fr.blobs.data(), 1, n[1], f);
    }
    fclose(f);
    return 0;
}

int replay_frame(const char* rcsPath, const char* kArg, const char* outPath)
{
    std::vector<uint8_t> data = read_file(rcsPath);
    uint32_t head[8];
    if (data.size() < sizeof(head))
        return fail("cannot read session");
    memcpy(head, data.data(), sizeof(head));
    if (head[0] != kRcsMagic)
        return fail("bad session");
    const uint32_t k = (uint32_t)std::stoul(kArg);
    if (k >= head[6])
        return fail("frame out of range");
    std::vector<Span<const uint8_t>> cmds, blobs;
    size_t o = sizeof(head);
    for (uint32_t i = 0; i < head[6]; ++i)
    {
        uint64_t n[2];
        if (o + sizeof(n) > data.size())
            return fail("truncated session");
        memcpy(n, data.data() + o, sizeof(n));
        o += sizeof(n);
        if (o + n[0] + n[1] > data.size())
            return fail("truncated session");
        cmds.emplace_back(data.data() + o, n[0]);
        blobs.emplace_back(data.data() + o + n[0], n[1]);
        o += n[0] + n[1];
    }
    CaptureImpl* impl = nullptr;
    std::unique_ptr<RenderContext> ctx = CaptureImpl::Make(&impl);
    impl->setAlwaysFeatherToAtlas((head[5] & RIVE_SCENE_FLAG_FEATHER_ATLAS) != 0);
    rcp<RenderTarget> target(impl->makeRenderTarget(head[1], head[2]));
    cmd::ResourceTable table;
    ctx->beginFrame(scene_frame(head[1], head[2], head[3], head[4], head[5]));
    {
        RiveRenderer renderer(ctx.get());
        for (uint32_t i = 0; i < k; ++i)
        {
            cmd::ReplayHooks resources, destroys;
            resources.filter = cmd::ReplayFilter::resources;
            destroys.filter = cmd::ReplayFilter::destroys;
            cmd::replayRenderCommands(ctx.get(), &renderer, cmds[i], blobs[i], table, resources);
            cmd::replayRenderCommands(ctx.get(), &renderer, cmds[i], blobs[i], table, destroys);
            table.clearVersionAliases();
        }
        cmd::replayRenderCommands(ctx.get(), &renderer, cmds[k], blobs[k], table);
    }
    ctx->flush({.renderTarget = target.get()});
    if (!write_capture(outPath, *impl, head[1], head[2]))
        return fail("cannot open output");
    return 0;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc == 4 && !strcmp(argv[1], "record"))
        return record(argv[2], argv[3]);
    if (argc == 4 && !strcmp(argv[1], "replay"))
        return replay(argv[2], argv[3]);
    if (argc == 4 && !strcmp(argv[1], "record-sriv"))
        return record_sriv(argv[2], argv[3]);
    if (argc == 5 && !strcmp(argv[1], "replay-frame"))
        return replay_frame(argv[2], argv[3], argv[4]);
    return fail("usage: cmdbuf_capture record <scene.bin> <out.rcb> | replay <in.rcb> <capture.bin>"
                " | record-sriv <in.sriv> <out.rcs> | replay-frame <in.rcs> <k> <capture.bin>");
}
