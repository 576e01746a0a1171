"""The serving loop (rive-runtime_gb300/serving.py): host-side animation on
CPU, and the continuous-batching server on the GPU, where every frame kept
from the mix must equal the same frame rendered alone."""
import math

import numpy as np
import pytest

from conftest import load_package

load_package()
from rive_runtime_gb300 import scene, serving  # noqa: E402
from inputgen import planner  # noqa: E402


def _anim(seed=5):
    sc = scene.full_feature(seed=seed, width=256, height=256, n_paths=40, max_cubics=8)
    return sc, serving.AnimatedScene(sc, np.random.default_rng(seed))


def test_animation_moves_points_and_turns_transforms():
    sc, a = _anim()
    f0, f1 = a.frame(0.0), a.frame(0.25)
    assert len(f0) == len(f1) == len(sc.to_bytes())
    assert f0 != f1 and a.frame(0.25) == f1  # deterministic in t
    p0 = np.frombuffer(f0, "<f4", 2 * a.npts, a.pts_off).reshape(-1, 2)
    p1 = np.frombuffer(f1, "<f4", 2 * a.npts, a.pts_off).reshape(-1, 2)
    shift = np.linalg.norm(p1 - p0, axis=1)
    assert shift.max() <= 2 * a.amplitude + 1e-3 and shift.max() > 0
    # Everything but points and transform matrices is unchanged.
    assert f0[:a.cmd_off] == f1[:a.cmd_off]


def test_animated_frames_plan_like_fresh_scenes():
    _, a = _anim(7)
    for t in (0.0, 0.5, 1.0):
        cap = planner.plan(a.frame(t))
        assert cap.width == 256 and len(cap.flushes) >= 1


def test_poisson_arrivals_are_ordered_and_seeded():
    scs = [scene.plain_canvas(np.random.default_rng(i), 64, 64, 5) for i in range(20)]
    s1 = serving.poisson_sessions(scs, 50.0, frames=3, seed=1)
    s2 = serving.poisson_sessions(scs, 50.0, frames=3, seed=1)
    t = [s.arrival for s in s1]
    assert t == sorted(t) and t == [s.arrival for s in s2]
    assert 0.1 < t[-1] < 1.5  # 20 arrivals at 50/s


@pytest.mark.gpu
def test_server_frames_match_frames_rendered_alone():
    from rive_runtime_gb300 import rive_cuda
    scs = [scene.full_feature(seed=40 + i, width=160 + 32 * i, height=200, n_paths=30,
                              max_cubics=8) for i in range(6)]
    sessions = serving.poisson_sessions(scs, 200.0, frames=5, fps=120.0, seed=3)
    keep = {(s.sid, k) for s in sessions for k in (0, 4)}
    ctx = rive_cuda.Context(0)
    try:
        server = serving.FrameServer(ctx, planner.plan, keep_frames=keep, planner_threads=4)
        stats = server.run(sessions, timeout_s=120.0)
        assert stats["frames"] == 6 * 5 and stats["sessions"] == 6
        assert stats["mean_batch"] > 1.0  # frames of several sessions shared batches
        alone_ctx = rive_cuda.Context(0)
        try:
            for (sid, k), img in server.kept.items():
                want = serving.render_alone(alone_ctx, planner.plan, sessions[sid], k)
                assert np.array_equal(img, want), (sid, k)
        finally:
            alone_ctx.close()
    finally:
        ctx.close()


def _recorded():
    import glob
    import os
    from rive_runtime_gb300 import sriv
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "anim")
    out = {}
    for path in sorted(glob.glob(os.path.join(here, "*.rsa"))):
        with open(path, "rb") as f:
            out[os.path.basename(path)[:-4]] = sriv.unpack_frames(f.read())
    return out


def test_recorded_animations_load_and_plan():
    anims = _recorded()
    assert len(anims) >= 5
    for name, frames in anims.items():
        a = serving.RecordedAnimation(frames, rate=60.0)
        assert a.frame(0.0) == frames[0] and a.frame(1.0 / 60.0) == frames[1 % len(frames)]
        assert a.frame(len(frames) / 60.0) == frames[0]  # loops
        cap = planner.plan(a.frame(0.5))
        assert (cap.width, cap.height) == (a.width, a.height) and cap.flushes, name


def test_recorded_sessions_cycle_through_animations():
    anims = list(_recorded().values())
    ss = serving.recorded_sessions(anims, 10, 50.0, frames=4, fps=30.0, seed=2)
    assert [s.anim.frames is anims[i % len(anims)] or s.anim.frames == anims[i % len(anims)]
            for i, s in enumerate(ss)] == [True] * 10
    assert [s.arrival for s in ss] == sorted(s.arrival for s in ss)


@pytest.mark.gpu
def test_server_recorded_frames_match_frames_rendered_alone():
    """Real content in the mix: recorded animations of different canvas sizes
    and clip/blend/clockwise content, each kept frame equal to itself alone."""
    from rive_runtime_gb300 import rive_cuda
    anims = list(_recorded().values())
    sessions = serving.recorded_sessions(anims, 8, 400.0, frames=4, fps=60.0, seed=5)
    keep = {(s.sid, k) for s in sessions for k in (0, 3)}
    ctx = rive_cuda.Context(0)
    try:
        server = serving.FrameServer(ctx, planner.plan, keep_frames=keep, planner_threads=4)
        stats = server.run(sessions, timeout_s=120.0)
        assert stats["frames"] == 8 * 4
        alone_ctx = rive_cuda.Context(0)
        try:
            for (sid, k), img in server.kept.items():
                want = serving.render_alone(alone_ctx, planner.plan, sessions[sid], k)
                assert np.array_equal(img, want), (sid, k)
        finally:
            alone_ctx.close()
    finally:
        ctx.close()
