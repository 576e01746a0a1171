"""RenderContextCUDAImpl (rive-runtime_gb300/csrc/render_context_cuda_impl.*)
inside the reference's own, unmodified RiveRenderer and RenderContext.

The backend is linked against a recording stand-in of the C ABI
(oracle/capture/abi_recorder.c), so this runs without a GPU: every record
buffer, flush descriptor and draw batch that reaches the ABI must be
byte-identical to what the reference's RenderContext handed a
RenderContextImpl for the same scene. Needs the reference sources (skipped
where they are absent).
"""
import pytest

from conftest import golden_names, load_golden, load_package
import oracle

load_package()
from rive_runtime_gb300 import scene  # noqa: E402

pytestmark = pytest.mark.skipif(not oracle.reference_available(),
                                reason="reference sources absent")


@pytest.mark.parametrize("name", golden_names())
def test_backend_forwards_golden_frames_unchanged(name):
    _, scene_bytes = load_golden(name)
    with open(f"{oracle.REPO}/tests/golden/{name}.cap", "rb") as f:
        want = f.read()
    assert oracle.adapter_capture(scene_bytes) == want


def test_backend_forwards_every_logical_flush():
    """Full-size full-feature scene: several logical flushes, gradients,
    clips and blend modes, compared against a live reference capture."""
    sb = scene.full_feature(seed=2).to_bytes()
    ref = oracle.reference_capture(sb)
    got = oracle.adapter_capture(sb)
    from rive_runtime_gb300 import capture
    assert len(capture.parse(ref).flushes) > 1
    assert got == ref
