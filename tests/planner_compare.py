"""Field-by-field comparison of two flush captures of the same scene (the
reference front end's and the planner's). Used by the planner tests."""
import numpy as np

# (buffer, element size, desc first-field, desc count-field, compared bytes)
RANGES = [
    ("paths", 64, "first_path", "path_count", 36),   # matrix, radii, zIndex
    ("paints", 8, "first_paint", "path_count", 8),
    ("paint_aux", 128, "first_paint_aux", "path_count", 64),  # paint + clip-rect parts
    ("contours", 16, "first_contour", "contour_count", 16),
    ("grad_spans", 16, "first_grad_span", "grad_span_count", 16),
    ("tess_spans", 64, "first_tess_span", "tess_span_count", 64),
]


def diff_captures(ref, got):
    """Returns a list of human-readable differences (empty when identical)."""
    out = []
    if (ref.width, ref.height) != (got.width, got.height):
        out.append("canvas size")
    if len(ref.flushes) != len(got.flushes):
        return out + [f"flush count {len(ref.flushes)} vs {len(got.flushes)}"]
    for fi, (a, b) in enumerate(zip(ref.flushes, got.flushes)):
        for k in a.desc:
            if a.desc[k] != b.desc[k]:
                out.append(f"flush {fi} desc.{k}: {a.desc[k]} vs {b.desc[k]}")
        if not np.array_equal(a.batches, b.batches):
            out.append(f"flush {fi} batches: {a.batches.tolist()} vs {b.batches.tolist()}")
        for name, elem, first, count, nbytes in RANGES:
            n = a.desc[count]
            fa, fb = a.desc[first], b.desc[first]
            ra = np.frombuffer(ref.buffers[name], np.uint8)[fa * elem:(fa + n) * elem]
            rb = np.frombuffer(got.buffers[name], np.uint8)[fb * elem:(fb + n) * elem]
            if len(ra) != len(rb):
                out.append(f"flush {fi} {name}: {len(ra)} vs {len(rb)} bytes")
                continue
            ra = ra.reshape(n, elem)[:, :nbytes]
            rb = rb.reshape(n, elem)[:, :nbytes]
            bad = np.nonzero((ra != rb).any(axis=1))[0]
            if len(bad):
                i = int(bad[0])
                out.append(f"flush {fi} {name}: {len(bad)} of {n} records differ, first #{i}: "
                           f"{ra[i].view(np.uint32).tolist()} vs {rb[i].view(np.uint32).tolist()}")
        ua = np.frombuffer(ref.buffers["flush_uniforms"], np.uint8)
        ub = np.frombuffer(got.buffers["flush_uniforms"], np.uint8)
        o = a.desc["flush_uniform_offset_bytes"]
        if not np.array_equal(ua[o:o + 104], ub[o:o + 104]):
            out.append(f"flush {fi} uniforms: {ua[o:o+104].view(np.uint32).tolist()} vs "
                       f"{ub[o:o+104].view(np.uint32).tolist()}")
    return out
