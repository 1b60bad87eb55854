"""ctypes harness of the CPU oracle (liboracle.so, built from oracle.cpp).

TEST INFRASTRUCTURE ONLY: the parity checker of the CUDA path tracer.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module.  It replays a ptgb.Scene into the oracle and exposes its
first-hit, per-path and progressive render entry points.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_P = ctypes.c_void_p
_lib = None


def build():
    """Compiles liboracle.so with the committed Makefile."""
    r = subprocess.run(["make", "-C", HERE, "-s"], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = ctypes.CDLL(LIB_PATH)
    L.or_create.restype = _P
    L.or_destroy.argtypes = [_P]
    L.or_add_material.argtypes = [_P, ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_float]
    L.or_add_prim.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
    L.or_add_mesh.argtypes = [_P, _P, ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_int, _P, _P,
                              _P]
    L.or_add_light.argtypes = [_P, ctypes.c_int, _P, ctypes.c_int, _P]
    L.or_set_miss.argtypes = [_P, ctypes.c_int, _P, _P, _P, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int]
    L.or_set_camera.argtypes = [_P, _P, _P, _P] + [ctypes.c_float] * 6
    L.or_commit.argtypes = [_P]
    L.or_add_texture.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P]
    L.or_material_set_texture.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.or_mesh_set_texture_index.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P]
    L.or_first_hits.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P,
                                ctypes.c_int]
    L.or_render_paths.argtypes = [_P, _P, ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_int]
    L.or_render.argtypes = [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
    L.or_render.restype = ctypes.c_double
    L.or_tea64.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    L.or_tea64.restype = ctypes.c_uint32
    L.or_rnd_stream.argtypes = [ctypes.c_uint32, ctypes.c_int, _P]
    L.or_math.argtypes = [ctypes.c_int, _P, _P, _P, ctypes.c_int]
    L.or_trace_ray.argtypes = [_P, _P, _P, ctypes.c_float, _P, _P]
    L.or_hit_record.argtypes = [_P, _P, _P, _P]
    L.or_bsdf_c.argtypes = [ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P, _P, _P]
    L.or_bsdf_sample_c.argtypes = [ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_float, _P,
                                   ctypes.c_uint32, ctypes.c_int, _P]
    L.or_env_sample.argtypes = [_P, _P, ctypes.c_int, _P, _P]
    L.or_bsdf_c_batch.argtypes = [ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_float, _P,
                                  ctypes.c_int, _P, _P, _P]
    L.or_lcg_stream.argtypes = [ctypes.c_uint32, ctypes.c_int, _P]
    L.or_sampling.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_int, _P]
    L.or_brdf_sample.argtypes = [ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_int, _P, _P, _P, _P]
    L.or_brdf_eval.argtypes = [ctypes.c_int, _P, _P, ctypes.c_float, ctypes.c_float,
                               ctypes.c_int, _P, _P, _P, _P, _P]
    L.or_helper.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P]
    L.or_light.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P]
    L.or_probe.argtypes = [_P, _P, _P, ctypes.c_float, _P, _P]
    L.or_camera_rays.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P]
    L.or_trace64.argtypes = [_P, ctypes.c_int, _P, _P, ctypes.c_float, _P, _P, ctypes.c_int]
    L.or_prim64.argtypes = [_P, ctypes.c_int, _P, _P, ctypes.c_float, _P]
    L.or_msphere.argtypes = [_P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P,
                             ctypes.c_float, ctypes.c_float, _P]
    _lib = L
    return L


def _f(v):
    return np.ascontiguousarray(v, dtype=np.float32)


def _p(a):
    return None if a is None else a.ctypes.data_as(_P)


def replay(L, prefix, h, s):
    """Replays a ptgb.Scene (materials, primitives, meshes, lights, miss
    program, camera, in call order) into a scene of the CPU oracle
    (prefix "or_") or of the reference-program harness (prefix "rh_"): both
    libraries take the same calls."""
    fn = lambda name: getattr(L, prefix + name)
    for kind, a, b, cc, data, perm, ids in getattr(s, "textures", []):
        fn("add_texture")(h, kind, a, b, _p(_f(cc)), _p(data), _p(perm), _p(ids))
    for kind, c0, c1, p0, p1 in s.materials:
        c0a = _f(c0)
        c1a = _f(c1) if c1 is not None else None
        fn("add_material")(h, kind, _p(c0a), _p(c1a), p0, p1)
    for m, slot, t in getattr(s, "mat_textures", []):
        fn("material_set_texture")(h, m, slot, t)
    tex_index = getattr(s, "tex_index", {})
    for k, it in enumerate(s.items):
        if it[0] == "sphere":
            _, cen, r, m, xf = it
            fn("add_prim")(h, 1, _p(_f(list(cen) + [r])), 0, 0, m, _p(xf))
        elif it[0] == "msphere":
            if prefix != "or_":
                raise NotImplementedError("the reference harness has no moving sphere scene path")
            _, c0, c1, r, t0, t1, m, xf = it
            fn("add_prim")(h, 4, _p(_f(list(c0) + [r, t0, t1] + list(c1))), 0, 0, m, _p(xf))
        elif it[0] == "rect":
            _, v5, flip, axis, m, xf = it
            fn("add_prim")(h, 2, _p(_f(v5)), axis, flip, m, _p(xf))
        elif it[0] == "box":
            _, p0, p1, m, xf = it
            fn("add_prim")(h, 3, _p(_f(list(p0) + list(p1))), 0, 0, m, _p(xf))
        else:
            _, v, idx, m, mpt, nrm, uv, xf = it
            mpt_i = None if mpt is None else np.ascontiguousarray(mpt, dtype=np.int32)
            first = fn("add_mesh")(h, _p(v), len(v), _p(idx), len(idx), _p(mpt_i),
                                   m if m is not None else 0, _p(nrm), _p(uv), _p(xf))
            if k in tex_index:
                ti = tex_index[k]
                fn("mesh_set_texture_index")(h, first, len(ti), _p(ti))
    for lt in s.lights:
        if lt[0] == "rect":
            _, v5, axis, e = lt
            fn("add_light")(h, 0, _p(_f(v5)), axis, _p(_f(e)))
        else:
            _, cen, r, e = lt
            fn("add_light")(h, 1, _p(_f(list(cen) + [r])), 0, _p(_f(e)))
    ms = s.miss
    if ms[0] == "gradient":
        fn("set_miss")(h, 0, _p(_f(ms[1])), _p(_f(ms[2])), None, 0, 0, 1)
    elif ms[0] == "constant":
        fn("set_miss")(h, 1, _p(_f(ms[1])), None, None, 0, 0, 1)
    else:
        rgba = ms[1]
        fn("set_miss")(h, ms[3], None, None, _p(rgba), rgba.shape[1], rgba.shape[0], ms[2])
    cf, ca, cu, vfov, aspect, ap, fd, t0, t1 = s.camera
    fn("set_camera")(h, _p(_f(cf)), _p(_f(ca)), _p(_f(cu)), vfov, aspect, ap, fd, t0, t1)
    fn("commit")(h)


class Oracle:
    """A scene loaded into the CPU oracle."""

    def __init__(self, scene):
        self.L = load()
        self.h = self.L.or_create()
        self._keep = []
        self.load(scene)

    def __del__(self):
        try:
            self.L.or_destroy(self.h)
        except Exception:
            pass

    def load(self, s):
        replay(self.L, "or_", self.h, s)

    def env_sample(self, u):
        u = np.ascontiguousarray(u, dtype=np.float32)
        n = len(u)
        dirs = np.zeros((n, 3), dtype=np.float32)
        pdf = np.zeros(n, dtype=np.float32)
        ok = self.L.or_env_sample(self.h, _p(u), n, _p(dirs), _p(pdf))
        return (dirs, pdf) if ok else (None, None)

    def camera_rays(self, width, height, frame):
        """Camera rays of `frame` as the float path generates them."""
        o = np.zeros((width * height, 3), np.float32)
        d = np.zeros((width * height, 3), np.float32)
        self.L.or_camera_rays(self.h, width, height, frame, _p(o), _p(d))
        return o, d

    def trace64(self, o, d, tmin=1e-6, threads=0):
        """Closest hits in double precision: primitive (-1) and, per ray, t,
        margin, mslack, tslack (the FP32 error scales; see or_trace64)."""
        o, d = _f(o), _f(d)
        n = len(o)
        prim = np.zeros(n, np.int32)
        out = np.zeros((n, 4), np.float64)
        self.L.or_trace64(self.h, n, _p(o), _p(d), tmin, _p(prim), _p(out),
                          threads or os.cpu_count())
        return prim, out

    def prim64(self, prim, o, d, tmin=1e-6):
        """(hit, [t, margin, mslack, tslack]) of one primitive in double."""
        out = np.zeros(4, np.float64)
        hit = self.L.or_prim64(self.h, int(prim), _p(_f(o)), _p(_f(d)), tmin, _p(out))
        return bool(hit), out

    def first_hits(self, width, height, frame, threads=0):
        prim = np.zeros(width * height, dtype=np.int32)
        mat = np.zeros(width * height, dtype=np.int32)
        t = np.zeros(width * height, dtype=np.float32)
        self.L.or_first_hits(self.h, width, height, frame, _p(prim), _p(mat), _p(t),
                             threads or os.cpu_count())
        return prim.view(np.uint32), mat.view(np.uint32), t

    @staticmethod
    def _params(width, height, spp, frame0, max_depth, rr_enable, rr_depth, mode=0, guide=0):
        return np.array([width, height, spp, frame0, max_depth, rr_enable, rr_depth, mode, guide],
                        dtype=np.int32)

    def render_paths(self, width, height, frame, pixels, max_depth=50, rr_enable=1, rr_depth=10,
                     threads=0, mode=0):
        pix = np.ascontiguousarray(pixels, dtype=np.uint32)
        out = np.zeros((len(pix), 3), dtype=np.float32)
        prm = self._params(width, height, 1, frame, max_depth, rr_enable, rr_depth, mode)
        self.L.or_render_paths(self.h, _p(prm), frame, _p(pix), len(pix), _p(out),
                               threads or os.cpu_count())
        return out

    def render(self, width, height, spp, frame0=0, max_depth=50, rr_enable=1, rr_depth=10,
               acc=None, pixel_stride=1, pixel_offset=0, threads=0, mode=0):
        if acc is None:
            acc = np.zeros((height, width, 4), dtype=np.float32)
        prm = self._params(width, height, spp, frame0, max_depth, rr_enable, rr_depth, mode)
        stats = np.zeros(3, dtype=np.uint64)
        secs = self.L.or_render(self.h, _p(prm), _p(acc), pixel_stride, pixel_offset,
                                threads or os.cpu_count(), _p(stats))
        return acc, {"seconds": secs, "ext_rays": int(stats[0]), "shadow_rays": int(stats[1]),
                     "paths": int(stats[2])}


def bsdf_c(mtype, c0, c1, p0, p1, wo, wi):
    """Consistent-mode f (rgb) and pdf for local y-up directions."""
    L = load()
    f = np.zeros(3, dtype=np.float32)
    pdf = np.zeros(1, dtype=np.float32)
    c1a = None if c1 is None else _f(c1)
    L.or_bsdf_c(mtype, _p(_f(c0)), _p(c1a), p0, p1, _p(_f(wo)), _p(_f(wi)), _p(f), _p(pdf))
    return f, float(pdf[0])


def bsdf_sample_c(mtype, c0, c1, p0, p1, wo, seed, n):
    L = load()
    out = np.zeros((n, 3), dtype=np.float32)
    c1a = None if c1 is None else _f(c1)
    L.or_bsdf_sample_c(mtype, _p(_f(c0)), _p(c1a), p0, p1, _p(_f(wo)), seed, n, _p(out))
    return out


def bsdf_c_batch(mtype, c0, c1, p0, p1, wo, wi):
    L = load()
    wi = np.ascontiguousarray(wi, dtype=np.float32)
    n = len(wi)
    f = np.zeros((n, 3), dtype=np.float32)
    pdf = np.zeros(n, dtype=np.float32)
    c1a = None if c1 is None else _f(c1)
    L.or_bsdf_c_batch(mtype, _p(_f(c0)), _p(c1a), p0, p1, _p(_f(wo)), n, _p(wi), _p(f), _p(pdf))
    return f, pdf


def msphere(f9, o, d, tmin, tmax, time, cam_t0=0.0, cam_t1=1.0):
    """The oracle's moving sphere (f9 = centre at time0, radius, time0,
    time1, centre at time1) against one ray at `time`: (hit, [t, P, shading
    normal, u, v, Wo] as 12 floats, box6 for the camera times)."""
    L = load()
    out = np.zeros(12, np.float32)
    box = np.zeros(6, np.float32)
    hit = L.or_msphere(_p(_f(f9)), _p(_f(o)), _p(_f(d)), tmin, tmax, time, _p(out), cam_t0, cam_t1,
                       _p(box))
    return bool(hit), out, box
