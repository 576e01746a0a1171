"""Benchmark of the GB300 flush backend on the full-feature single scene.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload full_feature|full_feature_1024|plain_small|stroke_stress_1024] [--capture FILE]

A step is one frame: every logical flush of the frame (gradient ramps,
tessellation, patch set-up, tile binning + sort, raster resolve) over the
frame's record buffers. Workload (default): the full-feature scene, a
2048x2048 RGBA8 canvas with 5,000 paths (seeded synthetic, see
rive-runtime_gb300/scene.py), turned into flush records by the planner (or read
from --capture).

Printed JSON (one line, rank 0):
  value        frames/s with the records resident in HBM (rive_cuda_flush_device)
  e2e          frames/s through the C ABI with host buffers: map/write/unmap of
               every record buffer (H2D) + all flushes + read-back of the
               RGBA8 target (D2H), inside the timed region
  roofline     the dominant kernel's algorithmic bytes per launch over its
               CUDA-event duration, against the measured HBM copy peak
  cpu_baseline the oracle (CPU restatement of the passes) on the host cores
--impl reference times that CPU implementation alone, on the same workload.

Multi-GPU: the path shards by scene only (replicas). With N>1 each rank
renders its own copy of the workload; value = frames of all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "tests"))


# DRAM bytes per bin entry of the raster, from one ncu capture of each raster
# form on the 1024x1024 full-feature frame (9.766 M entries): the one-CTA-per-
# tile grid read and wrote 696.4 MB, the work queue 993.6 MB (profiles/).
RASTER_DRAM_BYTES_PER_ENTRY = {"grid": 696.4e6 / 9.766e6, "queue": 993.6e6 / 9.766e6}


def _package():
    from conftest import load_package
    return load_package()


def build_workload(args):
    """(capture, workload name, scene recording or None)."""
    _package()
    from rive_runtime_gb300 import capture, scene
    if args.capture:
        with open(args.capture, "rb") as f:
            return capture.parse(f.read()), f"capture:{os.path.basename(args.capture)}", None
    from inputgen import planner
    if args.workload == "full_feature":
        sc = scene.full_feature(seed=2)
    elif args.workload == "full_feature_1024":
        # The same distributions on a quarter of the area (profiling size).
        sc = scene.full_feature(seed=21, width=1024, height=1024, n_paths=1250)
    elif args.workload == "plain_small":
        sc = scene.plain_small(seed=1)
    elif args.workload == "stroke_stress_1024":
        # One 1024x1024 canvas of the tessellation-heavy stress: 5,000 strokes.
        sc = scene.stroke_stress(seed=4, width=1024, height=1024, n_strokes=5000)
    else:
        raise SystemExit(f"unknown workload {args.workload}")
    sb = sc.to_bytes()
    return planner.plan(sb), args.workload, sb


def max_over_ranks(value, device):
    """The largest `value` over all ranks (host-side timing only; the path has
    no data exchange)."""
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def workload_counts(cap):
    spans = paths = contours = grad_spans = grad_rows = verts = 0
    for f in cap.flushes:
        d = f.desc
        spans += d["tess_span_count"]
        paths += d["path_count"]
        contours += d["contour_count"]
        grad_spans += d["grad_span_count"]
        grad_rows += d["grad_data_height"]
        verts += int(f.batches[:, 1].sum()) * 8 if len(f.batches) else 0
    return dict(spans=spans, paths=paths, contours=contours, grad_spans=grad_spans,
                grad_rows=grad_rows, tess_vertices=verts, flushes=len(cap.flushes))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_baseline(cap, threads):
    """The oracle (CPU restatement of the passes) on one whole frame."""
    import oracle
    t0 = time.perf_counter()
    oracle.render(cap, threads=threads)
    dt = time.perf_counter() - t0
    return dt


def run_reference(args, cap, wname, rank, world):
    """The reference's CPU implementation of the path (the oracle port: the
    reference's pixel passes exist only as shaders) on all host cores. A step
    is one logical flush of the frame, in turn, so a step is a bounded sample;
    frames/s = frames' worth of flushes / time."""
    if rank != 0:
        return
    import numpy as np
    import oracle
    threads = os.cpu_count() or 1
    nflush = len(cap.flushes)
    fb = np.zeros((cap.height, cap.width, 4), np.uint8)

    def step(i):
        oracle.render_flush(cap, i % nflush, fb, threads=threads)

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        step(i)
    dt = time.perf_counter() - t0
    fps = (args.steps / nflush) / dt
    line = {
        "impl": "reference", "metric": "frames/s", "value": fps, "unit": "frames/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / max(args.steps, 1), "higher_is_better": True,
        "scaling": "weak", "dtype": "f32", "data": "synthetic",
        "config": workload_config(cap, wname),
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} logical flushes ({args.steps / nflush:.2f} "
                                   f"frames) of {wname} through the oracle, OpenMP on "
                                   f"{threads} threads"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "vs_baseline": None,
    }
    print(json.dumps(line))


def workload_config(cap, wname):
    return {"workload": wname, "width": cap.width, "height": cap.height,
            "flushes_per_frame": len(cap.flushes),
            "l2": "inputs per frame far larger than L2 (no flush needed)",
            **workload_counts(cap)}


def run_ours(args, cap, wname, rank, world, scene_bytes=None):
    import numpy as np
    import torch
    from rive_runtime_gb300 import rive_cuda
    from rive_runtime_gb300.capture import BUFFER_NAMES

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    # A stream of our own: the flushes and the timing events must share one
    # stream (the library's default stream does not order with torch's).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = rive_cuda.Context(dev)
    W, H = cap.width, cap.height

    # Device-resident records for the `value` measurement.
    dbufs = rive_cuda.DeviceBuffers()
    keep = []
    for name in BUFFER_NAMES:
        b = cap.buffers.get(name, b"")
        t = torch.from_numpy(np.frombuffer(b, np.uint8).copy()).cuda() if b else None
        keep.append(t)
        setattr(dbufs, name, t.data_ptr() if t is not None else None)
    target = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")

    def frame_device():
        for f in cap.flushes:
            ctx.flush_device(f, dbufs, target.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        frame_device()
    # Raster configuration: the autotuner times its candidates on this frame
    # (untimed) and leaves the fastest set, or a fixed "T,C" is used.
    raster = raster_setup(args, ctx, lambda s: frame_device(), stream)
    # One more untimed frame, flush by flush, for the per-frame bin entries
    # (the pair count is known on the host when a flush call returns).
    frame_entries = 0
    for f in cap.flushes:
        ctx.flush_device(f, dbufs, target.data_ptr(), stream.cuda_stream)
        frame_entries += ctx.stats()["bin_entries"]
    ctx.sync(stream.cuda_stream)
    torch.cuda.synchronize()

    # Timed region (device-resident). Inputs per frame (records, 4 tess
    # textures, triangle records, bins) are far larger than the 129 MB L2.
    sampler = ClockSampler(dev)
    sampler.start()
    ctx.set_profiling(True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        frame_device()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clocks = sampler.stop()
    prof = ctx.profile_collect()
    ctx.set_profiling(False)
    ctx.sync(stream.cuda_stream)
    stats = ctx.stats()
    if world > 1:
        ms = max_over_ranks(ms, "cuda")
    fps = world * args.steps / (ms / 1e3)

    # End to end through the C ABI with host buffers.
    frame_bytes = sum(len(cap.buffers.get(n, b"")) for n in BUFFER_NAMES)
    host_t = ctx.render_target(W, H)
    # Page-locked read-back buffers, two in turn: frames are pipelined as an
    # application drives the reference's 3-deep rings, so the host writes
    # frame k+1's records while frame k renders and reads back.
    outs = [torch.empty((H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(2)]
    step = [0]

    def frame_e2e():
        ctx.upload_frame(cap)
        for f in cap.flushes:
            ctx.flush(f, host_t)
        ctx.read_target_async(host_t, outs[step[0] & 1].data_ptr())
        step[0] += 1

    for _ in range(args.warmup):
        frame_e2e()
    ctx.sync()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        frame_e2e()
    ctx.sync()  # the last frame's read-back has landed
    e2e_s = time.perf_counter() - t0
    e2e_fps = args.steps / e2e_s

    # Roofline of the dominant stage.
    counts = workload_counts(cap)
    peak, peak_kind = measured_peak_gbs()
    dominant = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_launches = prof[dominant]
    per_launch_s = (dom_ms / max(dom_launches, 1)) / 1e3
    traffic = None
    if dominant == "raster":
        # Per launch: bin entries x (4 B slot index + 96 B triangle record)
        # + 4 B per pixel written (+ 4 B read when the flush preserves the
        # target), averaged over the frame's flushes.
        preserve = sum(1 for f in cap.flushes if f.desc["color_load_action"] != 0)
        frame_bytes_raster = frame_entries * 100 + 4 * W * H * (len(cap.flushes) + preserve)
        alg_bytes = frame_bytes_raster / len(cap.flushes)
        # DRAM bytes (read + write) per launch, scaled by bin entries from one
        # ncu capture of this raster form on the 1024x1024 full-feature frame;
        # the full frame is too large to capture.
        form = "queue" if raster.get("queue") and raster.get("tile") == 16 else "grid"
        traffic = RASTER_DRAM_BYTES_PER_ENTRY[form] * frame_entries / len(cap.flushes)
    elif dominant == "tessellate":
        alg_bytes = 64 * counts["spans"] / counts["flushes"] + 16 * counts["tess_vertices"] / counts["flushes"]
    else:
        alg_bytes = 0
    achieved = alg_bytes / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    line = {
        "metric": "frames/s", "value": fps, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": dict(workload_config(cap, wname), raster=raster),
        "gpx_per_s": fps * W * H / 1e9,
        "e2e": {"value": e2e_fps, "unit": "frames/s", "h2d_bytes_per_step": frame_bytes,
                "d2h_bytes_per_step": W * H * 4},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic},
        "stage_ms_per_frame": {k: v[0] / args.steps for k, v in prof.items()},
        # Tessellated vertices per second of the tessellation stage.
        "tess_vertices_per_s": (counts["tess_vertices"] * args.steps / (prof["tessellate"][0] / 1e3)
                                if prof["tessellate"][0] > 0 else None),
        "gpu_launches": int(sum(v[1] for v in prof.values())),
        "clocks": clocks,
    }
    ctx.close()
    del keep, target
    # The batched and serving measurements are single-GPU (rank 0 of N=1).
    if args.batch_scenes > 0 and world == 1:
        line["batched"] = run_batched(args, dev, raster)
        line["batched_recorded"] = run_batched(args, dev, raster, recorded=True)
    if args.serve_sessions > 0 and world == 1:
        line["serving"] = run_serving(args, dev, raster)
    if args.serve_curve and world == 1:
        line["serving_curve"] = run_serving_curve(args, dev, raster)
    if args.serve_rec_sessions > 0 and world == 1:
        line["serving_recorded"] = run_serving_recorded(args, dev, raster)
    if args.feather_steps > 0 and world == 1:
        line["feathered"] = run_feathered(args, dev)
        line["images"] = run_images(args, dev)
    if args.stress_canvases > 0 and world == 1:
        line["stroke_stress"] = run_stress(args, dev, raster)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        dt = cpu_baseline(cap, threads)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "frames/s", "cores": threads,
                                "kind": "port",
                                "sample": f"1 whole frame of {wname} through the oracle"}
        if scene_bytes is not None:
            # The CPU front end beside the passes: RiveRenderer -> RenderContext
            # turning the scene into flush records, single-threaded as the
            # reference's RenderContext is. On this machine it is the stand-in
            # (tests/inputgen), whose records equal the reference's byte for byte.
            from inputgen import planner
            t0 = time.perf_counter()
            planner.plan_bytes(scene_bytes)
            fe = time.perf_counter() - t0
            line["cpu_baseline"]["front_end"] = {
                "value": 1.0 / fe, "unit": "frames/s", "cores": 1,
                "kind": "stand-in for the reference front end (records byte-identical)",
                "ms_per_frame": fe * 1e3}
            line["cpu_baseline"]["front_end_plus_passes"] = {
                "value": 1.0 / (fe + dt), "unit": "frames/s",
                "ms_per_frame": (fe + dt) * 1e3}
    if rank == 0:
        print(json.dumps(line))


FEATHERED_CAPTURE = ("silver_police_files_f60",
                     "recorded frame 60 of game_menu_ad_police_files (1080x1080) with feathered "
                     "fills and strokes below the atlas threshold, planned by the reference front end")


def _recorded_frame_fps(args, dev, name):
    """(capture, frames/s, ms per frame) of golden capture `name` rendered
    args.feather_steps times, records resident in HBM, timed with CUDA events
    on the flush stream (textures and render buffers are made during the
    warm-up)."""
    import numpy as np
    import torch
    from rive_runtime_gb300 import capture, rive_cuda
    from rive_runtime_gb300.capture import BUFFER_NAMES
    with open(os.path.join(REPO, "tests", "golden", name + ".cap"), "rb") as f:
        cap = capture.parse(f.read())
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = rive_cuda.Context(dev)
    dbufs = rive_cuda.DeviceBuffers()
    keep = []
    for n in BUFFER_NAMES:
        b = cap.buffers.get(n, b"")
        t = torch.from_numpy(np.frombuffer(b, np.uint8).copy()).cuda() if b else None
        keep.append(t)
        setattr(dbufs, n, t.data_ptr() if t is not None else None)
    target = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda")

    def frame():
        for fl in cap.flushes:
            ctx.flush_device(fl, dbufs, target.data_ptr(), stream.cuda_stream)

    for _ in range(max(args.warmup, 3)):
        frame()
    ctx.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.feather_steps):
        frame()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    ctx.sync(stream.cuda_stream)
    ctx.close()
    return cap, args.feather_steps / (ms / 1e3), ms / args.feather_steps


def run_feathered(args, dev):
    """Frames/s of a recorded frame with feathered draws (the feather kernel
    variants and the center-AA fans)."""
    name, what = FEATHERED_CAPTURE
    cap, fps, ms = _recorded_frame_fps(args, dev, name)
    center = sum(int((fl.batches[:, 0] == 1).sum()) for fl in cap.flushes)
    return {"workload": name, "content": what, "width": cap.width, "height": cap.height,
            "center_aa_batches": center, "steps": args.feather_steps,
            "frames_per_s": fps, "ms_per_frame": ms,
            "raster": "16x16 tiles, full occupancy (not autotuned)"}


# Recorded frames with images: drawImage draws (image paints) and a
# drawImageMesh, with the images the recordings carry.
IMAGE_CAPTURES = (
    ("silver_superbowl_images_f5", "recorded frame 5 of superbowl (2914x296): 4 PNG images "
     "drawn with drawImage among 99 path draws"),
    ("silver_image_mesh_f10", "recorded frame 10 of image_fit_alignment_2 (500x500): drawImage "
     "draws and a drawImageMesh"),
)


def run_images(args, dev):
    """Frames/s of recorded frames with image paints and an image mesh."""
    out = []
    for name, what in IMAGE_CAPTURES:
        cap, fps, ms = _recorded_frame_fps(args, dev, name)
        out.append({"workload": name, "content": what, "width": cap.width,
                    "height": cap.height, "textures": len(cap.textures),
                    "image_meshes": sum(int((fl.batches[:, 0] == 6).sum()) for fl in cap.flushes),
                    "steps": args.feather_steps, "frames_per_s": fps, "ms_per_frame": ms})
    return out


def run_serving(args, dev, raster=None):
    """The serving loop (rive-runtime_gb300/serving.py): sessions with the
    full-feature distributions on a smaller canvas, Poisson arrivals at 50/s,
    each animated for a fixed number of frames at a fixed frame rate."""
    from inputgen import planner
    from rive_runtime_gb300 import rive_cuda, scene, serving
    scs = [scene.full_feature(seed=1000 + i, width=args.serve_size, height=args.serve_size,
                              n_paths=args.serve_paths) for i in range(args.serve_sessions)]
    sessions = serving.poisson_sessions(scs, 50.0, frames=args.serve_frames,
                                        fps=args.serve_fps, seed=7)
    ctx = rive_cuda.Context(dev)
    if raster:
        ctx.set_raster_config(raster["tile"], raster["ctas_per_sm"])
        ctx.set_winding_tiles(raster.get("winding", False))
        ctx.set_raster_queue(raster.get("queue", False))
    try:
        server = serving.FrameServer(ctx, planner.plan, device=dev, hbm_budget_bytes=120 << 30,
                                     planner_threads=min(16, os.cpu_count() or 1))
        st = server.run(sessions, timeout_s=600.0)
    finally:
        ctx.close()
    offered = args.serve_sessions * args.serve_fps
    return {"workload": f"serving_{args.serve_sessions}x{args.serve_frames}",
            "scene": f"full_feature distributions, {args.serve_size}x{args.serve_size}, "
                     f"{args.serve_paths} paths",
            "arrivals_per_s": 50.0, "fps_per_session": args.serve_fps,
            "offered_frames_per_s_at_full_concurrency": offered,
            "hbm_budget_gb": 120, **st}


def _serve(ctx, dev, raster, scenes, frames, fps, seed):
    """One serving-loop run over `scenes` (Poisson arrivals at 50/s)."""
    from inputgen import planner
    from rive_runtime_gb300 import serving
    sessions = serving.poisson_sessions(scenes, 50.0, frames=frames, fps=fps, seed=seed)
    server = serving.FrameServer(ctx, planner.plan, device=dev, hbm_budget_bytes=120 << 30,
                                 planner_threads=min(16, os.cpu_count() or 1))
    return server.run(sessions, timeout_s=600.0)


def run_serving_curve(args, dev, raster=None):
    """Frame latency against session count.

    (1) The serving scene (full-feature distributions at --serve-size with
    --serve-paths paths) at each count of --serve-curve, --serve-curve-frames
    frames per session at --serve-fps; the largest count whose p99 stays
    within 8 ms is the capacity at that bound. (2) Sessions of the
    full-feature single scene itself (2048x2048, 5,000 paths) at one and two
    sessions: one such frame alone occupies the whole GPU for longer than
    8 ms, so no session count of that scene holds p99 within 8 ms on one GPU
    (1,000 of them would need 1,000 x 60 frames/s)."""
    from rive_runtime_gb300 import rive_cuda, scene
    counts = [int(x) for x in args.serve_curve.split(",") if x.strip()]
    ctx = rive_cuda.Context(dev)
    if raster:
        ctx.set_raster_config(raster["tile"], raster["ctas_per_sm"])
        ctx.set_winding_tiles(raster.get("winding", False))
        ctx.set_raster_queue(raster.get("queue", False))
    keys = ("sessions", "frames", "frames_per_s", "p50_ms", "p99_ms", "mean_batch",
            "max_concurrent", "peak_reserved_gb", "wall_s")
    curve, full = [], []
    try:
        for n in counts:
            scs = [scene.full_feature(seed=3000 + i, width=args.serve_size,
                                      height=args.serve_size, n_paths=args.serve_paths)
                   for i in range(n)]
            st = _serve(ctx, dev, raster, scs, args.serve_curve_frames, args.serve_fps, seed=n)
            curve.append({"offered_frames_per_s": n * args.serve_fps,
                          **{k: st[k] for k in keys}})
        if args.serve_full_frames > 0:
            for n in (1, 2):
                scs = [scene.full_feature(seed=5000 + i) for i in range(n)]
                st = _serve(ctx, dev, raster, scs, args.serve_full_frames, 4.0, seed=50 + n)
                full.append({"offered_frames_per_s": n * 4.0, **{k: st[k] for k in keys}})
    finally:
        ctx.close()
    within = [c["sessions"] for c in curve if c["p99_ms"] is not None and c["p99_ms"] <= 8.0]
    return {
        "scene": f"full_feature distributions, {args.serve_size}x{args.serve_size}, "
                 f"{args.serve_paths} paths",
        "fps_per_session": args.serve_fps, "frames_per_session": args.serve_curve_frames,
        "arrivals_per_s": 50.0, "curve": curve,
        "max_sessions_p99_within_8ms": max(within) if within else 0,
        "full_scale": {"scene": "full_feature 2048x2048, 5,000 paths",
                       "fps_per_session": 4.0, "frames_per_session": args.serve_full_frames,
                       "runs": full,
                       "sessions_p99_within_8ms": 0 if full and all(
                           r["p99_ms"] > 8.0 for r in full) else None},
    }


def raster_setup(args, ctx, run, stream):
    """Applies --raster-config ("auto" or "tile,ctas_per_sm"); returns what was set."""
    if args.raster_config == "auto":
        from rive_runtime_gb300 import autotune
        best, trials = autotune.autotune(ctx, run, stream=stream, warmup=1, iters=3)
        return {"tile": best.tile_size, "ctas_per_sm": best.ctas_per_sm,
                "winding": best.winding, "queue": best.queue, "autotuned": True,
                "trial_ms": {f"{t.tile_size},{t.ctas_per_sm}{',w' if t.winding else ''}"
                             f"{',q' if t.queue else ''}": round(t.ms, 3) for t in trials}}
    parts = args.raster_config.split(",")
    t, c = int(parts[0]), int(parts[1])
    w, q = "w" in parts[2:], "q" in parts[2:]
    ctx.set_raster_config(t, c)
    ctx.set_winding_tiles(w)
    ctx.set_raster_queue(q)
    return {"tile": t, "ctas_per_sm": c, "winding": w, "queue": q, "autotuned": False}


def run_serving_recorded(args, dev, raster=None):
    """The serving loop on real content: sessions playing the reference's
    recorded .riv animations (tests/golden/anim, converted from its .sriv
    streams), each from a random start frame, Poisson arrivals at 50/s."""
    import glob
    from inputgen import planner
    from rive_runtime_gb300 import rive_cuda, serving, sriv
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "anim")
    anims, names = [], []
    for path in sorted(glob.glob(os.path.join(here, "*.rsa"))):
        with open(path, "rb") as f:
            anims.append(sriv.unpack_frames(f.read()))
        names.append(os.path.basename(path)[:-4])
    sessions = serving.recorded_sessions(anims, args.serve_rec_sessions, 50.0,
                                         frames=args.serve_rec_frames, fps=args.serve_rec_fps,
                                         seed=11)
    ctx = rive_cuda.Context(dev)
    if raster:
        ctx.set_raster_config(raster["tile"], raster["ctas_per_sm"])
        ctx.set_winding_tiles(raster.get("winding", False))
        ctx.set_raster_queue(raster.get("queue", False))
    try:
        server = serving.FrameServer(ctx, planner.plan, device=dev, hbm_budget_bytes=120 << 30,
                                     planner_threads=min(16, os.cpu_count() or 1))
        st = server.run(sessions, timeout_s=600.0)
    finally:
        ctx.close()
    return {"workload": f"serving_recorded_{args.serve_rec_sessions}x{args.serve_rec_frames}",
            "content": "recorded .riv animations: " + ", ".join(names),
            "arrivals_per_s": 50.0, "fps_per_session": args.serve_rec_fps,
            "offered_frames_per_s_at_full_concurrency":
                args.serve_rec_sessions * args.serve_rec_fps, **st}


def recorded_caps(count):
    """`count` frames of the recorded .riv animations (tests/golden/anim),
    taken in turn from each animation, planned."""
    import glob
    from inputgen import planner
    from rive_runtime_gb300 import sriv
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "anim")
    anims = []
    for path in sorted(glob.glob(os.path.join(here, "*.rsa"))):
        with open(path, "rb") as f:
            anims.append(sriv.unpack_frames(f.read()))
    caps = []
    for i in range(count):
        fr = anims[i % len(anims)]
        caps.append(planner.plan(fr[(i // len(anims)) % len(fr)]))
    return caps


def run_batched(args, dev, raster=None, recorded=False):
    """The batched form: N independent scenes of uneven canvas sizes and path
    counts (scene.batched_scenes; or, `recorded`, frames of the recorded .riv
    animations), rendered (a) one flush at a time, (b) as one
    rive_cuda_flush_batch per flush index, (c) as one CUDA graph launch per
    flush index. Frames/s counts scenes; each pass renders every scene once,
    with the records resident in HBM."""
    from inputgen import planner
    from rive_runtime_gb300 import scene

    if recorded:
        caps = recorded_caps(args.batch_scenes)
    else:
        caps = [planner.plan(sc.to_bytes())
                for sc in scene.batched_scenes(count=args.batch_scenes)]
    out = time_batch(caps, args, dev, raster)
    out["workload"] = f"batched_{'recorded_' if recorded else ''}{len(caps)}"
    return out


def _stress_scene_bytes(job):
    # One canvas of the tessellation-heavy stress (a worker of a spawned
    # process pool: scene generation is plain Python).
    seed, size, strokes = job
    from conftest import load_package
    load_package()
    from rive_runtime_gb300 import scene
    return scene.stroke_stress(seed=seed, width=size, height=size, n_strokes=strokes).to_bytes()


def run_stress(args, dev, raster=None):
    """The tessellation-heavy stress at its stated size: one 4096x4096 canvas
    of 100,000 strokes and 64 1024x1024 canvases of 5,000 strokes each (1-16
    cubics, 20% cusp or near-degenerate, width log-uniform in [0.5, 64] px,
    round joins and caps, alpha 0.8), rendered together as batches: wave i
    batches logical flush i of every canvas. A frame is all 65 canvases."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from inputgen import planner
    jobs = [(4000, 4096, args.stress_big)] + [(4001 + i, 1024, args.stress_small)
                                               for i in range(args.stress_canvases)]
    sys.path.insert(0, os.path.join(REPO, "tests"))
    # Spawned workers (never forked from a process that has used the GPU).
    with cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1),
                                mp_context=mp.get_context("spawn")) as ex:
        scenes = list(ex.map(_stress_scene_bytes, jobs))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        caps = list(ex.map(planner.plan, scenes))
    out = time_batch(caps, args, dev, raster, modes=("batch", "graph"))
    verts = sum(int(f.batches[:, 1].sum()) * 8 for c in caps for f in c.flushes
                if len(f.batches))
    out["workload"] = (f"stroke_stress: 1 x 4096^2 with {args.stress_big} strokes + "
                       f"{args.stress_canvases} x 1024^2 with {args.stress_small} strokes")
    out["tess_vertices_per_frame"] = verts
    out["graph_tess_vertices_per_s"] = verts * out["graph_frames_per_s"] / len(caps)
    return out


def time_batch(caps, args, dev, raster=None, modes=("plain", "batch", "graph")):
    """Times rendering every capture once, with the records resident in HBM:
    one flush at a time, as one rive_cuda_flush_batch per wave of logical
    flushes, and as one CUDA graph per wave; frames/s counts captures."""
    import numpy as np
    import torch
    from rive_runtime_gb300 import rive_cuda
    from rive_runtime_gb300.capture import BUFFER_NAMES

    stream = torch.cuda.current_stream()
    keep, bufs, targets = [], [], []
    for cap in caps:
        b = rive_cuda.DeviceBuffers()
        for name in BUFFER_NAMES:
            d = cap.buffers.get(name, b"")
            t = torch.from_numpy(np.frombuffer(d, np.uint8).copy()).cuda() if d else None
            keep.append(t)
            setattr(b, name, t.data_ptr() if t is not None else None)
        bufs.append(b)
        targets.append(torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda"))
    nflush = max(len(c.flushes) for c in caps)
    waves = [[(c.flushes[k], b, t.data_ptr()) for c, b, t in zip(caps, bufs, targets)
              if k < len(c.flushes)] for k in range(nflush)]
    steps = max(1, args.batch_steps)

    def timed(fn):
        fn()  # warm-up pass (also sizes every buffer)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    def configured():
        c = rive_cuda.Context(dev)
        if raster:
            c.set_raster_config(raster["tile"], raster["ctas_per_sm"])
            c.set_winding_tiles(raster.get("winding", False))
            c.set_raster_queue(raster.get("queue", False))
        return c

    n = len(caps)
    px = sum(c.width * c.height for c in caps)
    out = {"scenes": n, "mpx": px / 1e6,
           "paths": int(sum(f.desc["path_count"] for c in caps for f in c.flushes)),
           "flushes": int(sum(len(c.flushes) for c in caps)), "waves": len(waves),
           "steps": steps}
    ctx = configured()
    if "plain" in modes:
        ms_plain = timed(lambda: [ctx.flush_device(f, b, tp, stream.cuda_stream)
                                  for w in waves for (f, b, tp) in w])
        out["plain_frames_per_s"] = n * 1e3 / ms_plain
    if "batch" in modes:
        ms_batch = timed(lambda: [ctx.flush_batch(w, stream.cuda_stream) for w in waves])
        ctx.sync(stream.cuda_stream)
        out["bin_entries_last_wave"] = int(ctx.stats()["bin_entries"])
        out["batch_frames_per_s"] = n * 1e3 / ms_batch
    ctx.close()
    if "graph" in modes:
        ctx = configured()
        graphs = [ctx.graph(w) for w in waves]
        ms_graph = timed(lambda: [g.launch(stream.cuda_stream) for g in graphs])
        for g in graphs:
            g.check(stream.cuda_stream)
            g.close()
        ctx.close()
        out["graph_frames_per_s"] = n * 1e3 / ms_graph
        out["graph_gpx_per_s"] = px / (ms_graph * 1e6)
        if "plain" in modes:
            out["speedup_vs_plain"] = ms_plain / ms_graph
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="full_feature")
    ap.add_argument("--capture", default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched-form measurement (0 skips it)")
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--serve-sessions", type=int, default=64,
                    help="sessions of the serving-loop measurement (0 skips it)")
    ap.add_argument("--serve-size", type=int, default=512)
    ap.add_argument("--serve-paths", type=int, default=300)
    ap.add_argument("--serve-frames", type=int, default=60)
    ap.add_argument("--serve-fps", type=float, default=8.0)
    ap.add_argument("--serve-curve", default="4,16,64,128",
                    help="session counts of the latency-against-sessions curve (empty skips it)")
    ap.add_argument("--serve-curve-frames", type=int, default=40)
    ap.add_argument("--serve-full-frames", type=int, default=6,
                    help="frames per session of the full-scale serving runs (0 skips them)")
    ap.add_argument("--serve-rec-sessions", type=int, default=128,
                    help="sessions of the recorded-animation serving run (0 = skip)")
    ap.add_argument("--serve-rec-frames", type=int, default=120)
    ap.add_argument("--serve-rec-fps", type=float, default=30.0)
    ap.add_argument("--feather-steps", type=int, default=200,
                    help="frames of the recorded feathered-frame measurement (0 skips it)")
    ap.add_argument("--stress-canvases", type=int, default=64,
                    help="1024x1024 canvases of the stroke stress beside its 4096x4096 one "
                         "(0 skips the stress measurement)")
    ap.add_argument("--stress-small", type=int, default=5000)
    ap.add_argument("--stress-big", type=int, default=100000)
    ap.add_argument("--raster-config", default="auto",
                    help='"auto" (autotuned on the workload) or "tile,ctas_per_sm[,w][,q]", e.g. '
                         '"16,0" (",w": interior tiles as winding records; ",q": work-queue '
                         'raster)')
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group(backend)
    cap, wname, scene_bytes = build_workload(args)
    if args.impl == "reference":
        run_reference(args, cap, wname, rank, world)
    else:
        run_ours(args, cap, wname, rank, world, scene_bytes)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
