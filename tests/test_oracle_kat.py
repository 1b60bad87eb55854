"""Known-answer tests that pin the oracle (the reference publishes no golden
vectors for this path): the integer RNG of programs/random.cuh against an
independent Python statement of TEA and the Numerical Recipes LCG, and
analytic ray/primitive answers for the shapes of programs/hitables/."""
import ctypes
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
M32 = 0xFFFFFFFF


def tea64_py(v0, v1):
    """TEA, Wheeler & Needham 1994, 64 rounds as programs/random.cuh:33-47."""
    s0 = 0
    for _ in range(64):
        s0 = (s0 + 0x9E3779B9) & M32
        v0 = (v0 + ((((v1 << 4) + 0xA341316C) & M32) ^ ((v1 + s0) & M32)
                    ^ (((v1 >> 5) + 0xC8013EA4) & M32))) & M32
        v1 = (v1 + ((((v0 << 4) + 0xAD90777D) & M32) ^ ((v0 + s0) & M32)
                    ^ (((v0 >> 5) + 0x7E95761E) & M32))) & M32
    return v0


def rnd_stream_py(seed, n):
    out = []
    for _ in range(n):
        seed = (1664525 * seed + 1013904223) & M32
        out.append(np.float32(seed & 0xFFFFFF) / np.float32(16777216.0))
    return np.array(out, dtype=np.float32)


def test_tea_matches_python(oracle_mod):
    L = oracle_mod.load()
    rng = np.random.default_rng(0)
    for a, b in rng.integers(0, 2**32, size=(200, 2), dtype=np.uint64):
        assert L.or_tea64(int(a), int(b)) == tea64_py(int(a), int(b))


def test_rng_golden_vectors(oracle_mod):
    """Fixture generated by tests/golden/make_golden.py (pure Python)."""
    L = oracle_mod.load()
    with open(os.path.join(GOLDEN, "rng.json")) as f:
        g = json.load(f)
    for (a, b), v in zip(g["tea_inputs"], g["tea64"]):
        assert L.or_tea64(a, b) == v
    for seed, stream in zip(g["lcg_seeds"], g["rnd_streams"]):
        out = np.zeros(len(stream), dtype=np.float32)
        L.or_rnd_stream(seed, len(stream), out.ctypes.data_as(ctypes.c_void_p))
        assert out.tolist() == stream
        assert np.array_equal(out, rnd_stream_py(seed, len(stream)))


def _single(oracle_mod, ptgb_like):
    return oracle_mod.Oracle(ptgb_like)


def make_scene(kind):
    import ptgb
    s = ptgb.Scene()
    m = s.lambertian((0.5, 0.5, 0.5))
    if kind == "sphere":
        s.sphere((0.0, 0.0, 10.0), 2.0, m)
    elif kind == "rect":
        s.rect(-1, 1, -1, 1, 5.0, False, ptgb.PT_Z_AXIS, m)
    elif kind == "box":
        s.box((-1, -1, 4), (1, 1, 6), m)
    elif kind == "tri":
        s.mesh(np.array([[-1, -1, 3], [1, -1, 3], [0, 1, 3]], dtype=np.float32),
               np.array([[0, 1, 2]], dtype=np.uint32), m)
    elif kind == "box_rot":
        s.box((-1, -1, -1), (1, 1, 1), m,
              ptgb.compose([ptgb.mat_translate((0, 0, 5)), ptgb.mat_rotate(90.0, 1)]))
    s.set_camera((0, 0, 0), (0, 0, 1), (0, 1, 0), 40.0, 1.0, 0.0, 1.0)
    return s


def trace(o, org, d, tmin=1e-6):
    L = o.L
    org = np.array(org, dtype=np.float32)
    d = np.array(d, dtype=np.float32)
    t = ctypes.c_float()
    uv = np.zeros(2, dtype=np.float32)
    pid = L.or_trace_ray(o.h, org.ctypes.data_as(ctypes.c_void_p),
                         d.ctypes.data_as(ctypes.c_void_p), tmin, ctypes.byref(t),
                         uv.ctypes.data_as(ctypes.c_void_p))
    return pid, t.value, uv


def hitrec(o, org, d):
    org = np.array(org, dtype=np.float32)
    d = np.array(d, dtype=np.float32)
    out = np.zeros(8, dtype=np.float32)
    pid = o.L.or_hit_record(o.h, org.ctypes.data_as(ctypes.c_void_p),
                            d.ctypes.data_as(ctypes.c_void_p),
                            out.ctypes.data_as(ctypes.c_void_p))
    return pid, out


def test_sphere_axis_hit(oracle_mod):
    o = oracle_mod.Oracle(make_scene("sphere"))
    pid, t, _ = trace(o, (0, 0, 0), (0, 0, 1))
    assert pid == 0 and t == 8.0  # centre 10 - radius 2
    # from inside: near root behind tmin, far root reported
    pid, t, _ = trace(o, (0, 0, 10), (0, 0, 1))
    assert pid == 0 and t == 2.0
    # unnormalised direction: t scales inversely
    pid, t, _ = trace(o, (0, 0, 0), (0, 0, 2))
    assert pid == 0 and t == 4.0
    pid, _, _ = trace(o, (0, 3, 0), (0, 0, 1))
    assert pid == -1
    _, rec = hitrec(o, (0, 0, 0), (0, 0, 1))
    assert np.allclose(rec[:3], [0, 0, 8]) and np.allclose(rec[3:6], [0, 0, -1])


def test_rect_hit_and_edges(oracle_mod):
    o = oracle_mod.Oracle(make_scene("rect"))
    pid, t, _ = trace(o, (0.5, 0.25, 0), (0, 0, 1))
    assert pid == 0 and t == 5.0
    pid, _, _ = trace(o, (1.0, 1.0, 0), (0, 0, 1))  # closed bounds: corner hits
    assert pid == 0
    pid, _, _ = trace(o, (1.0001, 0, 0), (0, 0, 1))
    assert pid == -1
    _, rec = hitrec(o, (0.5, 0.5, 0), (0, 0, 1))
    assert np.allclose(rec[6:8], [0.75, 0.75])  # u=(x-a0)/(a1-a0)


def test_box_slab_normals(oracle_mod):
    o = oracle_mod.Oracle(make_scene("box"))
    pid, t, _ = trace(o, (0, 0, 0), (0, 0, 1))
    assert pid == 0 and t == 4.0
    _, rec = hitrec(o, (0, 0, 0), (0, 0, 1))
    assert np.allclose(rec[3:6], [0, 0, -1])
    _, rec = hitrec(o, (-5, 0, 5), (1, 0, 0))
    assert np.allclose(rec[3:6], [-1, 0, 0])


def test_rotated_box_instance(oracle_mod):
    o = oracle_mod.Oracle(make_scene("box_rot"))
    pid, t, _ = trace(o, (0, 0, 0), (0, 0, 1))
    assert pid == 0 and abs(t - 4.0) < 1e-5
    _, rec = hitrec(o, (0, 0, 0), (0, 0, 1))
    assert np.allclose(rec[:3], [0, 0, 4], atol=1e-5)
    assert np.allclose(rec[3:6], [0, 0, -1], atol=1e-5)


def test_triangle_barycentrics(oracle_mod):
    o = oracle_mod.Oracle(make_scene("tri"))
    pid, t, uv = trace(o, (0, 0, 0), (0, 0, 1))
    assert pid == 0 and t == 3.0
    # hit point = a*(1-u-v) + b*u + c*v  (programs/hitables/triangle.cu:106-110)
    a, b, c = np.array([-1, -1, 3.]), np.array([1, -1, 3.]), np.array([0, 1, 3.])
    p = a * (1 - uv[0] - uv[1]) + b * uv[0] + c * uv[1]
    assert np.allclose(p, [0, 0, 3], atol=1e-6)
    # watertight: a ray through the shared edge of two triangles hits one
    import ptgb
    s = ptgb.Scene()
    m = s.lambertian((1, 1, 1))
    v = np.array([[-1, -1, 3], [1, -1, 3], [1, 1, 3], [-1, 1, 3]], dtype=np.float32)
    s.mesh(v, np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32), m)
    s.set_camera((0, 0, 0), (0, 0, 1), (0, 1, 0), 40.0, 1.0, 0.0, 1.0)
    o2 = oracle_mod.Oracle(s)
    for x in np.linspace(-0.9, 0.9, 37):
        pid, t, _ = trace(o2, (x, x, 0), (0, 0, 1))
        assert pid in (0, 1) and abs(t - 3.0) < 1e-6
