"""The oracle's tessellation building blocks held to the reference's own unit
tests of the same functions, and (on the GPU) the kernel's device functions
held to the oracle's, bit for bit.

Restated from the reference (rive-runtime, tests/unit_tests):
  * renderer/eval_cubic_test.cpp:33-54 and runtime/bezier_utils_test.cpp:603-614:
    a point on the cubic at t (here: the tessellator's De Casteljau chain,
    tessellate.glsl:535-540) within 1e-3 of the Bernstein form, for t in
    steps of 1/100 and t + 3e-3;
  * runtime/bezier_utils_test.cpp:670-688: the known answers of
    clamped_divide, infinities and NaNs included;
  * runtime/bezier_utils_test.cpp:690-744: find_cubic_max_height returns a
    height h >= 0 at a T in [0, 1] where the curve's height above its chord is
    h within 1e-4, and no sampled point of the curve is higher than
    h + max(h, 1) * 1e-3;
  * runtime/bezier_utils_test.cpp:989-1072: measure_cubic_local_curvature
    within 1e-2 rad of the turn found by a binary search for the same spread,
    on curves without an inflection that turn at most 90 degrees;
  * runtime/wangs_formula_test.cpp:400-460: Wang's segment count is enough
    (the n-segment chords stay within the tolerance, 1/4 px) and a matrix
    applied inside the formula gives the count of the transformed points.
Inputs: the reference tests' own cubics (read from the reference sources when
they are present), every cubic on the corners of a 100 px square (the
reference tests' enumeration), and seeded random cubics.
"""
import math
import os
import re

import numpy as np
import pytest

import oracle
from conftest import load_package

load_package()

REF_TESTS = os.path.join(oracle.REFERENCE_SOURCES, "tests", "unit_tests")
LAYOUT = {0: (2, 1), 1: (8, 2), 2: (10, 1), 3: (9, 2), 4: (12, 1), 5: (8, 4)}


def cubic_eval(fn, items):
    import ctypes
    k_in, k_out = LAYOUT[fn]
    x = np.ascontiguousarray(items, np.float32).reshape(-1, k_in)
    out = np.zeros((len(x), k_out), np.float32)
    lib = oracle.lib()
    lib.oracle_cubic_eval.restype = ctypes.c_int
    rc = lib.oracle_cubic_eval(ctypes.c_int(fn), x.ctypes.data_as(ctypes.c_void_p),
                               out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(len(x)))
    assert rc == 0
    return out


def _parse_cubic_array(path, name):
    """The Vec2D[][4] array `name` of a reference test file, as (n, 8)."""
    text = open(path).read()
    text = re.sub(r"//[^\n]*", "", text)
    start = text.index(name)
    body = text[text.index("{", start) + 1:]
    depth, i = 1, 0
    while depth:
        depth += {"{": 1, "}": -1}.get(body[i], 0)
        i += 1
    body = body[:i - 1]
    pairs = re.findall(r"\{([^{}]*)\}", body)

    def num(expr):
        expr = re.sub(r"(\d)\.?f\b", r"\1", expr.strip())
        assert re.fullmatch(r"[0-9.+\-*/ ()]+", expr), expr
        return float(eval(expr))  # arithmetic on literals only

    vals = [[num(c) for c in p.split(",")] for p in pairs]
    assert len(vals) % 4 == 0
    return np.array(vals, np.float32).reshape(-1, 8)


def reference_cubics():
    out = []
    for rel, name in (("renderer/eval_cubic_test.cpp", "cubics[][4]"),
                      ("runtime/bezier_utils_test.cpp", "TEST_CUBICS[][4]")):
        p = os.path.join(REF_TESTS, rel)
        if os.path.exists(p):
            out.append(_parse_cubic_array(p, name))
    return np.concatenate(out) if out else np.zeros((0, 8), np.float32)


def corner_cubics():
    # Every cubic whose four points are corners of [0, 100]^2.
    i = np.arange(256)
    bits = (i[:, None] >> np.arange(8)[None, :]) & 1
    return (bits * 100).astype(np.float32)


def random_cubics(n=100, seed=0, lo=-100.0, hi=100.0):
    return np.random.default_rng(seed).uniform(lo, hi, (n, 8)).astype(np.float32)


def all_cubics():
    return np.concatenate([reference_cubics(), corner_cubics(), random_cubics()])


def bernstein(c, t):
    c = c.astype(np.float64).reshape(4, 2)
    t = np.asarray(t, np.float64)[:, None]
    u = 1 - t
    return u ** 3 * c[0] + 3 * u * u * t * c[1] + 3 * u * t * t * c[2] + t ** 3 * c[3]


def test_de_casteljau_point_matches_the_bernstein_form():
    ts = np.arange(0, 101, dtype=np.float32) / np.float32(100)
    ts = np.concatenate([ts, ts + np.float32(3e-3), np.float32([0, 1])])
    for c in all_cubics():
        got = cubic_eval(3, np.concatenate([np.tile(c, (len(ts), 1)), ts[:, None]], 1))
        want = bernstein(c, ts.astype(np.float64))
        assert np.abs(got - want).max() <= 1e-3, (c, float(np.abs(got - want).max()))


def _reference_clamped_divide_answers():
    p = os.path.join(REF_TESTS, "runtime", "bezier_utils_test.cpp")
    if not os.path.exists(p):
        pytest.skip("reference sources absent")
    text = open(p).read()
    env = {"INF": math.inf, "NAN": math.nan}
    out = []
    for a, b, want in re.findall(r"clamped_divide\(([^,()]+),\s*([^()]+)\)\s*==\s*([^)]+)\)", text):
        def val(s):
            s = re.sub(r"(\d)\.?f\b", r"\1", s.strip())
            return float(eval(s, {"__builtins__": {}}, env))
        out.append((val(a), val(b), val(want)))
    assert len(out) >= 10
    return out


def test_clamped_divide_known_answers():
    cases = _reference_clamped_divide_answers()
    got = cubic_eval(0, np.array([[a, b] for a, b, _ in cases], np.float32))[:, 0]
    for (a, b, want), g in zip(cases, got):
        assert g == np.float32(want), (a, b, want, g)


def _height_at(c, t):
    c64 = c.astype(np.float64).reshape(4, 2)
    base = c64[3] - c64[0]
    n = np.array([-base[1], base[0]]) / np.hypot(*base)
    return np.abs((bernstein(c, t) - c64[0]) @ n)


def test_cubic_max_height_is_the_highest_point():
    cubics = all_cubics()
    out = cubic_eval(1, cubics)
    t2 = np.arange(0, 1.0000001, .005137)
    for c, (h, t) in zip(cubics, out):
        assert h >= 0 and 0 <= t <= 1, (c, h, t)
        if np.hypot(*(c[6:8].astype(np.float64) - c[0:2])) == 0:
            continue  # no chord: height 0 by definition
        assert abs(_height_at(c, [t])[0] - h) <= 1e-4 * max(1.0, h), (c, h, t)
        eps = max(h, 1.0) * 1e-3
        assert (h + eps > _height_at(c, np.concatenate([[0, 1], t2]))).all(), (c, h)


def _derivative(c, t):
    c = c.astype(np.float64).reshape(4, 2)
    t = np.asarray(t, np.float64)[:, None]
    u = 1 - t
    return 3 * (u * u * (c[1] - c[0]) + 2 * u * t * (c[2] - c[1]) + t * t * (c[3] - c[2]))


def _turn(d0, d1):
    cosv = np.sum(d0 * d1, -1) / (np.linalg.norm(d0, axis=-1) * np.linalg.norm(d1, axis=-1))
    return np.arccos(np.clip(cosv, -1, 1))


def _guess_local_curvature(c, t, spread):
    # Binary search for the half-width dt whose chord, projected on the unit
    # tangent at t, spans `spread`; then the turn between the tangents at
    # t - dt and t + dt (the rotation of the chopped, non-inflecting section).
    tan = _derivative(c, [t])[0]
    tan /= np.linalg.norm(tan)
    lo, hi = 0.0, min(t, 1 - t) * .9999
    for _ in range(40):
        mid = (lo + hi) / 2
        p = bernstein(c, [t - mid, t + mid])
        if abs(np.dot(p[1] - p[0], tan)) <= spread:
            lo = mid
        else:
            hi = mid
    d = _derivative(c, [t - lo, t + lo])
    return float(_turn(d[0:1], d[1:2])[0])


def _convex_within_90(c):
    ts = np.linspace(0, 1, 513)
    d = _derivative(c, ts)
    if (np.linalg.norm(d, axis=1) < 1e-3).any():
        return False
    cross = d[:-1, 0] * d[1:, 1] - d[:-1, 1] * d[1:, 0]
    if not ((cross >= 0).all() or (cross <= 0).all()):
        return False  # an inflection
    return _turn(d[0:1], d[-1:])[0] <= math.pi / 2 and np.sum(_turn(d[:-1], d[1:])) <= math.pi / 2


def _chop(c, t0, t1):
    # The section [t0, t1] of cubic c (blossoming), as a cubic.
    q = c.astype(np.float64).reshape(4, 2)

    def blossom(a, b, d):
        p = [q[0], q[1], q[2], q[3]]
        for u in (a, b, d):
            p = [p[i] + (p[i + 1] - p[i]) * u for i in range(len(p) - 1)]
        return p[0]

    return np.concatenate([blossom(t0, t0, t0), blossom(t0, t0, t1), blossom(t0, t1, t1),
                           blossom(t1, t1, t1)]).astype(np.float32)


def _sections():
    # Sections of random cubics short enough to be convex and turn <= 90
    # degrees, as the reference test obtains them by chopping at inflections
    # and every 90 degrees of turn.
    rng = np.random.default_rng(11)
    out = []
    for c in random_cubics(400, seed=12):
        t0 = rng.uniform(0, .8)
        out.append(_chop(c, t0, t0 + rng.uniform(.05, .2)))
    return np.array(out)


def test_local_curvature_matches_a_binary_search():
    cubics = [c for c in np.concatenate([all_cubics(), _sections()]) if _convex_within_90(c)]
    assert len(cubics) >= 100
    checked = 0
    for c in cubics:
        _, tmax = cubic_eval(1, c[None])[0]
        for spread in (1.0, 10.0, 100.0):
            for t in (float(tmax), .5):
                if not (1e-3 < t < 1 - 1e-3):
                    continue
                theta = cubic_eval(2, np.concatenate([c, [t, spread]])[None])[0, 0]
                assert 0 <= theta <= math.pi + 1e-6
                guess = _guess_local_curvature(c, t, spread)
                assert abs(theta - guess) <= 1e-2, (c, t, spread, theta, guess)
                checked += 1
    assert checked >= 100


def _random_beziers(seed=0, exps=range(-10, 21)):
    # Points (1 + u) * 2^i for a range of magnitudes i, as the reference's
    # Wang's-formula tests draw them.
    rng = np.random.default_rng(seed)
    return np.array([(1 + rng.uniform(0, 1, 8)) * 2.0 ** i for i in exps], np.float32)


def _max_chord_deviation(c, n):
    worst = 0.0
    for k in range(int(n)):
        t = np.linspace(k / n, (k + 1) / n, 33)
        p = bernstein(c, t)
        a, b = p[0], p[-1]
        ab = b - a
        L = np.hypot(*ab)
        if L == 0:
            dist = np.hypot(*(p - a).T)
        else:
            dist = np.abs((p - a) @ np.array([-ab[1], ab[0]]) / L)
        worst = max(worst, float(dist.max()))
    return worst


def test_wang_segment_count_meets_the_tolerance():
    ident = np.float32([1, 0, 0, 1])
    cubics = np.concatenate([reference_cubics(), corner_cubics(), random_cubics(200, seed=2),
                             _random_beziers()])
    n = cubic_eval(4, np.concatenate([cubics, np.tile(ident, (len(cubics), 1))], 1))[:, 0]
    for c, k in zip(cubics, n):
        assert k >= 1 and k == int(k)
        scale = float(np.abs(c).max())
        assert _max_chord_deviation(c, k) <= .25 + 1e-6 * max(scale, 1.0), (c, k)


def test_wang_matrix_inside_equals_transformed_points():
    rng = np.random.default_rng(3)
    cubics = np.concatenate([random_cubics(300, seed=4), _random_beziers(seed=5, exps=range(-4, 12))])
    same = 0
    for c in cubics:
        m = rng.uniform(-2, 2, 4).astype(np.float32)
        pts = c.reshape(4, 2).astype(np.float32)
        moved = np.stack([m[0] * pts[:, 0] + m[2] * pts[:, 1],
                          m[1] * pts[:, 0] + m[3] * pts[:, 1]], 1).astype(np.float32).reshape(8)
        a = cubic_eval(4, np.concatenate([c, m])[None])[0, 0]
        b = cubic_eval(4, np.concatenate([moved, np.float32([1, 0, 0, 1])])[None])[0, 0]
        assert abs(a - b) <= 1, (c, m, a, b)
        same += a == b
    assert same >= .98 * len(cubics)


def test_end_tangents_skip_repeated_points():
    cubics = np.concatenate([corner_cubics(), reference_cubics()])
    out = cubic_eval(5, cubics)
    for c, t in zip(cubics, out):
        p = c.reshape(4, 2)
        t0 = next((q - p[0] for q in p[1:] if (q != p[0]).any()), p[3] - p[0])
        t1 = next((p[3] - q for q in p[2::-1] if (q != p[3]).any()), p[3] - p[0])
        assert np.array_equal(t[:2], t0) and np.array_equal(t[2:], t1), (c, t)


@pytest.mark.gpu
@pytest.mark.parametrize("fn", [0, 1, 2, 3, 4, 5])
def test_kernel_device_functions_equal_the_oracle(fn):
    """The tessellation kernel's own device functions (through a small test
    kernel) give the oracle's bits on every input above."""
    from rive_runtime_gb300 import rive_cuda
    cubics = np.concatenate([all_cubics(), _random_beziers(), random_cubics(500, seed=6)])
    rng = np.random.default_rng(7)
    if fn == 0:
        items = rng.uniform(-10, 10, (2000, 2)).astype(np.float32)
        items = np.concatenate([items, np.float32([[np.inf, 1], [1, np.nan], [np.nan, np.nan],
                                                   [0, 0], [-2, 0], [1, 0]])])
    elif fn == 2:
        items = np.concatenate([cubics, rng.uniform(0, 1, (len(cubics), 1)),
                                rng.choice([1.0, 10.0, 100.0], (len(cubics), 1))], 1)
    elif fn == 3:
        items = np.concatenate([cubics, rng.uniform(0, 1, (len(cubics), 1))], 1)
    elif fn == 4:
        items = np.concatenate([cubics, rng.uniform(-3, 3, (len(cubics), 4))], 1)
    else:
        items = cubics
    items = np.ascontiguousarray(items, np.float32)
    got = rive_cuda.eval_tessellation_math(fn, items)
    want = cubic_eval(fn, items)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (
        fn, int((got.view(np.uint32) != want.view(np.uint32)).any(axis=1).sum()))


@pytest.mark.gpu
@pytest.mark.parametrize("fn", [10, 11, 12, 13])
def test_kernel_elementary_functions_equal_the_oracle(fn):
    import test_fp32_math as m
    from rive_runtime_gb300 import rive_cuda
    rng = np.random.default_rng(fn)
    if fn in (10, 11):
        x = np.concatenate([np.linspace(-64, 64, 200001), rng.uniform(-7, 7, 50000)])
    elif fn == 12:
        x = np.concatenate([np.linspace(-1, 1, 200001), 1 - np.arange(2000) * 2.0 ** -24])
    else:
        x = rng.integers(1, 0x7f7fffff, 200000, dtype=np.uint32).view(np.float32)
    x = x.astype(np.float32)
    got = rive_cuda.eval_tessellation_math(fn, x)[:, 0]
    want = m._eval(fn - 10, x)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), int(
        (got.view(np.uint32) != want.view(np.uint32)).sum())
