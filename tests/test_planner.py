"""The planner (host front end) against the reference front end's own output.

Golden fixtures pin the reference's bytes; where the reference sources exist,
fresh seeded scenes are compared live as well.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, load_package
from planner_compare import diff_captures
import oracle

load_package()
from rive_runtime_gb300 import scene  # noqa: E402
from inputgen import planner  # noqa: E402


def _triangulated(scene_bytes):
    import struct
    return struct.unpack_from("<12I", scene_bytes, 0)[11] & scene.FLAG_TRIANGULATE


def _feathered(scene_bytes):
    import struct
    h = struct.unpack_from("<12I", scene_bytes, 0)
    off = 48 + 20 * h[4]
    return any(struct.unpack_from("<f", scene_bytes, off + 56 * i + 52)[0] != 0
               for i in range(h[5]))


@pytest.mark.parametrize("name", golden_names())
def test_planner_matches_golden_capture(name):
    cap, scene_bytes = load_golden(name)
    if _triangulated(scene_bytes):
        # Interior triangulation stays with the reference front end.
        with pytest.raises(RuntimeError, match="triangulation"):
            planner.plan(scene_bytes)
        return
    if _feathered(scene_bytes):
        # So do feathered paints.
        with pytest.raises(RuntimeError, match="feathered"):
            planner.plan(scene_bytes)
        return
    if cap.textures:
        # And image draws.
        with pytest.raises(RuntimeError, match="image"):
            planner.plan(scene_bytes)
        return
    got = planner.plan(scene_bytes)
    assert diff_captures(cap, got) == []


def test_planner_is_deterministic():
    sb = scene.full_feature(seed=5, width=300, height=300, n_paths=60, max_cubics=10).to_bytes()
    assert planner.plan_bytes(sb) == planner.plan_bytes(sb)


def test_planner_rejects_garbage():
    with pytest.raises(RuntimeError):
        planner.plan(b"not a scene")
    sb = bytearray(scene.plain_small(seed=1, n_paths=3).to_bytes())
    with pytest.raises(RuntimeError):
        planner.plan(bytes(sb[:60]))  # truncated


def test_planner_empty_scene():
    sc = scene.Scene(64, 64)
    cap = planner.plan(sc.to_bytes())
    assert len(cap.flushes) == 1
    d = cap.flushes[0].desc
    assert d["tess_span_count"] == 0 and d["path_count"] == 1 and len(cap.flushes[0].batches) == 0
    img = oracle.render(cap)
    assert (img == 255).all()  # cleared to opaque white


SEEDED = [
    ("full_feature", dict(seed=101, width=640, height=480, n_paths=250, max_cubics=24)),
    ("full_feature", dict(seed=102, width=333, height=777, n_paths=200, max_cubics=16,
                          p_clip=0.5, p_blend=0.4, p_gradient=0.6)),
    ("stroke_stress", dict(seed=103, width=800, height=800, n_strokes=1500)),
    ("plain_small", dict(seed=104)),
]


@pytest.mark.skipif(not oracle.reference_available(), reason="reference sources absent")
@pytest.mark.parametrize("kind,kw", SEEDED)
def test_planner_matches_reference_live(kind, kw):
    sb = getattr(scene, kind)(**kw).to_bytes()
    from rive_runtime_gb300 import capture
    ref = capture.parse(oracle.reference_capture(sb))
    assert diff_captures(ref, planner.plan(sb)) == []


@pytest.mark.skipif(not oracle.reference_available(), reason="reference sources absent")
def test_planner_matches_reference_multi_flush():
    """The full-size full-feature scene spans several logical flushes
    (tessellation texture overflow); every flush must match."""
    sb = scene.full_feature(seed=2).to_bytes()
    from rive_runtime_gb300 import capture
    ref = capture.parse(oracle.reference_capture(sb))
    assert len(ref.flushes) > 1
    assert diff_captures(ref, planner.plan(sb)) == []
