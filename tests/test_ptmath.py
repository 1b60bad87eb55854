"""Accuracy of the shared elementary functions (optix-path-tracer_gb300/
csrc/ptmath.h), evaluated through the CPU oracle's build of the header,
against double-precision references."""
import ctypes
import math

import numpy as np
import pytest


def run(L, fn, x, y=None):
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros_like(x)
    yp = None if y is None else np.ascontiguousarray(y, dtype=np.float32)
    L.or_math(fn, x.ctypes.data_as(ctypes.c_void_p),
              None if yp is None else yp.ctypes.data_as(ctypes.c_void_p),
              out.ctypes.data_as(ctypes.c_void_p), len(x))
    return out


def ulps(got, ref):
    ref32 = np.abs(np.float32(ref))
    sp = np.spacing(np.maximum(ref32, np.float32(1e-37)))
    return np.abs(got.astype(np.float64) - ref) / sp


@pytest.mark.parametrize("fn,f,lo,hi,tol", [
    (0, math.sin, -40.0, 40.0, 3.0),
    (1, math.cos, -40.0, 40.0, 3.0),
    (3, math.atan, -50.0, 50.0, 3.0),
    (5, math.asin, -1.0, 1.0, 4.0),
    (6, math.acos, -1.0, 1.0, 4.0),
])
def test_unary_ulp(oracle_mod, fn, f, lo, hi, tol):
    L = oracle_mod.load()
    x = np.random.default_rng(fn).uniform(lo, hi, 100000).astype(np.float32)
    got = run(L, fn, x)
    ref = np.array([f(float(v)) for v in x])
    assert ulps(got, ref).max() <= tol


def test_tan_ulp(oracle_mod):
    L = oracle_mod.load()
    x = np.random.default_rng(7).uniform(-6.3, 6.3, 100000).astype(np.float32)
    got = run(L, 2, x)
    ref = np.array([math.tan(float(v)) for v in x])
    m = np.abs(ref) < 1e3
    assert ulps(got[m], ref[m]).max() <= 4.0


def test_atan2_quadrants(oracle_mod):
    L = oracle_mod.load()
    rng = np.random.default_rng(3)
    x = rng.uniform(-5, 5, 100000).astype(np.float32)
    y = rng.uniform(-5, 5, 100000).astype(np.float32)
    got = run(L, 4, x, y)
    ref = np.array([math.atan2(float(b), float(a)) for a, b in zip(x, y)])
    assert ulps(got, ref).max() <= 3.0
    # axes and signed zeros
    xs = np.array([1, -1, 0, 0, 0, -0.0], dtype=np.float32)
    ys = np.array([0, 0, 1, -1, 0, 0], dtype=np.float32)
    got = run(L, 4, xs, ys)
    ref = [math.atan2(float(b), float(a)) for a, b in zip(xs, ys)]
    assert np.allclose(got, ref, atol=1e-7)


def test_pow(oracle_mod):
    L = oracle_mod.load()
    rng = np.random.default_rng(5)
    x = rng.uniform(0, 1, 100000).astype(np.float32)
    y = rng.uniform(0, 40, 100000).astype(np.float32)
    got = run(L, 7, x, y)
    ref = np.array([float(a) ** float(b) for a, b in zip(x, y)])
    m = ref > 1e-30
    rel = np.abs(got[m] - ref[m]) / ref[m]
    assert rel.max() < 2e-5
    # special cases used by the BRDFs: exponent 5 of [0,1], cube roots
    assert run(L, 7, [0.0], [5.0])[0] == 0.0
    assert run(L, 7, [1.0], [123.0])[0] == 1.0
    assert run(L, 7, [0.5], [0.0])[0] == 1.0
    assert abs(run(L, 7, [0.125], [1.0 / 3.0])[0] - 0.5) < 1e-6
    assert run(L, 7, [-2.0], [3.0])[0] == pytest.approx(-8.0, rel=1e-6)
    assert math.isnan(run(L, 7, [-2.0], [0.5])[0])
