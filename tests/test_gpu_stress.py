"""The tessellation-heavy stress on the GPU: one 1024x1024 canvas of its
batch (5,000 strokes of 1-16 cubics, 20% cusp or near-degenerate, widths
0.5-64 px, round joins and caps), a sub-sample of the 4096^2 + 64 x 1024^2
batch the benchmark renders. Every tessellated vertex bit-exact against the
oracle and within 1e-4 px of the FP64 evaluation of its segment parameters
(or 1 ulp of its coordinate where fp32 spacing is coarser), and the image
within the parity tolerance."""
import numpy as np
import pytest

from conftest import load_package, tess_written
import oracle

load_package()


@pytest.fixture(scope="module")
def stress():
    from rive_runtime_gb300 import scene
    from inputgen import planner
    return planner.plan(scene.stroke_stress(seed=4001, width=1024, height=1024,
                                            n_strokes=5000).to_bytes())


@pytest.mark.gpu
def test_stress_canvas_tessellation_and_image(stress):
    from rive_runtime_gb300 import rive_cuda
    cap = stress
    ctx = rive_cuda.Context(0)
    try:
        t = ctx.render_target(cap.width, cap.height)
        ctx.upload_frame(cap)
        worst, vertices = 0.0, 0
        for i, f in enumerate(cap.flushes):
            ctx.flush(f, t)
            ctx.sync()
            written = tess_written(cap, i)
            got = ctx.read_tess(f.desc["tess_data_height"])[written]
            want = oracle.tessellate(cap, i)[written]
            assert np.array_equal(got, want), int((got != want).any(axis=1).sum())
            xy64, flags64 = oracle.tessellate_f64(cap, i)
            used = flags64[written] != 0
            xy = got[used, :2].view(np.float32).astype(np.float64)
            ref = xy64[written][used]
            err = np.abs(xy - ref)
            ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
            assert (err <= np.maximum(1e-4, ulp)).all(), float(err.max())
            worst = max(worst, float(err.max()))
            vertices += int(used.sum())
        img = ctx.read_target(t, cap.width, cap.height)
    finally:
        ctx.close()
    print(f"stroke stress 1024x1024: {vertices} vertices, worst error vs FP64 {worst:.3g} px")
    want = oracle.render(cap)
    d = np.abs(img.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    assert (d <= 2).mean() >= 0.999 and d.max() <= 8, (float((d <= 2).mean()), int(d.max()))
