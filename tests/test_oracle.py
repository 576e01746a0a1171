"""CPU tests of the oracle (the CPU restatement of the reference's GPU passes)
against the reference's own known answers, plus the golden flush captures.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_names, load_golden
import oracle

# advanced_blend.glsl mode numbers (constants.glsl).
COLORDODGE, COLORBURN, HUE, SATURATION, COLOR, LUMINOSITY = 5, 6, 12, 13, 14, 15


def coeffs(src, dst_premul, mode):
    import ctypes
    lib = oracle.lib()
    s = (ctypes.c_float * 3)(*src)
    d = (ctypes.c_float * 4)(*dst_premul)
    o = (ctypes.c_float * 3)()
    lib.oracle_advanced_blend_coeffs(s, d, mode, o)
    return np.array(list(o), np.float32)


def coeffs_dst_alpha(src, dst, a, mode):
    return coeffs(src, [dst[0] * a, dst[1] * a, dst[2] * a, a], mode)


def test_f16_round_trip_matches_numpy():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.normal(0, 4, 4000), rng.uniform(-1, 1, 4000),
                         [0.0, -0.0, 1.0, 65504.0, 1e-8, 6.1e-5, 2049.0, 1e9]])
    for x in xs.astype(np.float32):
        h = oracle.f32_to_f16(float(x))
        assert h == int(np.float16(x).view(np.uint16)), x
        assert oracle.f16_to_f32(h) == float(np.float16(x))


# Known answers of tests/unit_tests/renderer/advanced_blend_test.cpp
# ("glsl_colordodge", "glsl_colorburn"), restated.
DST_ALPHAS = [0.0, 1 / 255, 0.25, 0.5, 254 / 255, 1.0, 256 / 255]


def test_colordodge_known_answers():
    inf = np.inf
    assert np.all(coeffs([0, 0, 0], [0, 0, 0, 0], COLORDODGE) == 0)
    assert np.all(coeffs([1, 1.001, inf], [0.0001, 1, inf, 0], COLORDODGE) == 0)
    rng = np.random.default_rng(1)
    for a in DST_ALPHAS:
        assert np.all(coeffs_dst_alpha([0, 0, 0], [0, -0.001, -1], a, COLORDODGE) == 0)
        assert np.all(coeffs_dst_alpha([1, 1, 1], [-10, -100, -inf], a, COLORDODGE) == 0)
        if a != 0:
            assert np.all(coeffs_dst_alpha([1, 1.00001, 2], [1e-10] * 3, a, COLORDODGE) == 1)
            assert np.all(coeffs_dst_alpha([10, 100, inf], [1] * 3, a, COLORDODGE) == 1)
        for _ in range(100):
            src = rng.uniform(0, 1, 3).astype(np.float32)
            dst = np.zeros(3, np.float32) if a == 0 else rng.uniform(0, 1, 3).astype(np.float32)
            c = coeffs_dst_alpha(src, dst, a, COLORDODGE)
            for i in range(3):
                if dst[i] <= 0:
                    assert c[i] == 0
                elif src[i] >= 1:
                    assert c[i] == 1
                else:
                    assert c[i] == pytest.approx(min(1.0, dst[i] / (1 - src[i])), rel=1e-4)


def test_colorburn_known_answers():
    inf = np.inf
    rng = np.random.default_rng(2)
    for a in DST_ALPHAS:
        if a != 0:
            assert np.all(coeffs_dst_alpha([0, 0, 0], [1, 1.001, 2], a, COLORBURN) == 1)
            assert np.all(coeffs_dst_alpha([1, 1, 1], [10, 100, inf], a, COLORBURN) == 1)
        assert np.all(coeffs_dst_alpha([0, -0.1, -1], [1 - 1e-6] * 3, a, COLORBURN) == 0)
        assert np.all(coeffs_dst_alpha([-10, -100, -inf], [0] * 3, a, COLORBURN) == 0)
        for _ in range(100):
            src = rng.uniform(0, 1, 3).astype(np.float32)
            dst = np.zeros(3, np.float32) if a == 0 else rng.uniform(0, 1, 3).astype(np.float32)
            c = coeffs_dst_alpha(src, dst, a, COLORBURN)
            for i in range(3):
                if dst[i] >= 1 and a != 0:
                    assert c[i] == 1
                elif src[i] <= 0:
                    assert c[i] == 0
                else:
                    assert c[i] == pytest.approx(1 - min(1.0, (1 - dst[i]) / src[i]), abs=1e-4)


# The NV_blend_equation_advanced reference functions the reference's
# "glsl_*_blend" tests compare against (published spec formulas).
def _lum(c):
    return float(np.dot(c, [0.30, 0.59, 0.11]))


def _clip_color(c):
    lum, mn, mx = _lum(c), c.min(), c.max()
    if mn < 0:
        c = lum + (c - lum) * lum / (lum - mn)
    if mx > 1:
        c = lum + (c - lum) * (1 - lum) / (mx - lum)
    return c


def _set_lum(cbase, clum):
    return _clip_color(cbase + (_lum(clum) - _lum(cbase)))


def _set_lum_sat(cbase, csat, clum):
    sbase = cbase.max() - cbase.min()
    ssat = csat.max() - csat.min()
    color = (cbase - cbase.min()) * ssat / sbase if sbase > 0 else np.zeros(3)
    return _set_lum(color, clum)


@pytest.mark.parametrize("mode,spec", [
    (COLOR, lambda a, b: _set_lum(a, b)),
    (LUMINOSITY, lambda a, b: _set_lum(b, a)),
    (SATURATION, lambda a, b: _set_lum_sat(b, a, b)),
    (HUE, lambda a, b: _set_lum_sat(a, b, b)),
])
def test_hsl_modes_match_spec(mode, spec):
    steps = np.arange(6) / 5.0
    grid = np.array(np.meshgrid(steps, steps, steps)).reshape(3, -1).T
    rng = np.random.default_rng(mode)
    for x in grid:
        y = grid[rng.integers(0, len(grid))]
        x8 = np.floor(x * 255) / 255
        y8 = np.floor(y * 255) / 255
        got = coeffs_dst_alpha(x8, y8, 1.0, mode)
        want = spec(x8.astype(np.float64), y8.astype(np.float64))
        assert np.max(np.abs(got - want)) <= 1e-4


@pytest.mark.parametrize("name", golden_names())
def test_oracle_renders_golden(name):
    cap, _ = load_golden(name)
    img = oracle.render(cap, threads=4)
    tris, frags = oracle.last_stats()
    assert tris > 0 and frags > 0
    again = oracle.render(cap, threads=1)
    assert np.array_equal(img, again), "oracle must not depend on its thread count"
    clear = np.array([255, 255, 255, 255], np.uint8)
    assert (img != clear).any(axis=2).mean() > 0.05


@pytest.mark.parametrize("name", golden_names())
def test_oracle_tessellation_within_fp64(name):
    """fp32 tessellated vertices vs the FP64 evaluation of the same segment
    parameters: every vertex within 1e-4 px, or within 1 ulp of its coordinate
    where fp32 spacing itself exceeds that (coordinates beyond 1024 px)."""
    cap, _ = load_golden(name)
    for fi in range(len(cap.flushes)):
        t32 = oracle.tessellate(cap, fi)
        xy64, flags64 = oracle.tessellate_f64(cap, fi)
        used = flags64 != 0
        assert np.array_equal(t32[used, 3], flags64[used])
        xy32 = t32[used, :2].view(np.float32).astype(np.float64)
        err = np.abs(xy32 - xy64[used])
        ulp = np.spacing(np.abs(xy64[used]).astype(np.float32)).astype(np.float64)
        ok = err <= np.maximum(1e-4, ulp)
        assert ok.all(), (name, float(ok.mean()), float(err.max()))


@pytest.mark.skipif(not oracle.reference_available(), reason="reference sources absent")
@pytest.mark.parametrize("name", golden_names())
def test_golden_captures_reproduce_from_reference(name):
    """The fixtures are exactly what the reference front end emits today."""
    cap_bytes = open(os.path.join(GOLDEN, name + ".cap"), "rb").read()
    scene_bytes = open(os.path.join(GOLDEN, name + ".scene"), "rb").read()
    assert oracle.reference_capture(scene_bytes) == cap_bytes


def _reference_f16_table(name):
    import os
    import re
    import pytest
    src = os.path.join(oracle.REFERENCE_SOURCES, "renderer", "src", "gpu.cpp")
    if not os.path.exists(src):
        pytest.skip("reference sources absent")
    text = open(src).read()
    body = text[text.index(f"const uint16_t {name}[GAUSSIAN_TABLE_SIZE] = {{"):]
    body = body[body.index("{") + 1:body.index("};")]
    return [int(v, 16) for v in re.findall(r"0x[0-9a-fA-F]+", body)]


def test_feather_table_matches_the_reference_table():
    """The oracle's Gaussian-integral table, built from the published
    generator, equals the fp16 table the reference ships."""
    want = _reference_f16_table("g_gaussianIntegralTableF16")
    got = oracle.feather_table().tolist()
    assert len(want) == 512
    diff = [i for i in range(512) if got[i] != want[i]]
    assert diff == [], (diff[:8], [(got[i], want[i]) for i in diff[:8]])


def test_inverse_feather_table_matches_the_reference_table():
    """The inverse table feathered-fill tessellation softens curves with
    equals the reference's shipped fp16 inverse table."""
    want = _reference_f16_table("g_inverseGaussianIntegralTableF16")
    got = oracle.inverse_feather_table().tolist()
    assert len(want) == 512
    diff = [i for i in range(512) if got[i] != want[i]]
    assert diff == [], (diff[:8], [(got[i], want[i]) for i in diff[:8]])
