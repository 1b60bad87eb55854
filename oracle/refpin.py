"""ctypes harness of oracle/_ref/libref.so: the reference's own device
programs (programs/ of joaovbs96/OptiX-Path-Tracer), compiled unmodified on
the host over the OptiX stand-in in oracle/refhost and run by its emulated
runtime.

TEST INFRASTRUCTURE ONLY: it pins the CPU oracle (oracle.cpp), which the
CUDA kernels are checked against, to the reference's code.  Only tests/ use
it.  The library is built from the reference's source tree (the Makefile's
REF path, overridable by the environment variable PT_REFERENCE); where that
tree is absent, `available()` is False and the pin tests skip.
"""
import ctypes
import os
import subprocess

import numpy as np

import oracle as _oracle

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref.so")
DEFAULT_REF = "/root/reference/OptiX-Path-Tracer"

_P = ctypes.c_void_p
_lib = None
_f, _p = _oracle._f, _oracle._p


def reference_tree():
    return os.environ.get("PT_REFERENCE", DEFAULT_REF)


def build():
    """Builds _ref/libref.so with the committed Makefile; None if the
    reference's tree is not present here."""
    ref = reference_tree()
    if not os.path.isdir(os.path.join(ref, "programs")):
        return None
    r = subprocess.run(["make", "-C", HERE, "-s", "ref", f"REF={ref}"], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError("reference harness build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


def available():
    try:
        return load() is not None
    except OSError:
        return False


def load():
    global _lib
    if _lib is not None:
        return _lib
    if build() is None and not os.path.exists(LIB_PATH):
        return None
    L = ctypes.CDLL(LIB_PATH)
    i, u, fl = ctypes.c_int, ctypes.c_uint32, ctypes.c_float
    L.rh_create.restype = _P
    L.rh_destroy.argtypes = [_P]
    L.rh_add_material.argtypes = [_P, i, _P, _P, fl, fl]
    L.rh_add_prim.argtypes = [_P, i, _P, i, i, i, _P]
    L.rh_add_mesh.argtypes = [_P, _P, i, _P, i, _P, i, _P, _P, _P]
    L.rh_add_light.argtypes = [_P, i, _P, i, _P]
    L.rh_set_miss.argtypes = [_P, i, _P, _P, _P, i, i, i]
    L.rh_set_camera.argtypes = [_P, _P, _P, _P] + [fl] * 6
    L.rh_commit.argtypes = [_P]
    L.rh_add_texture.argtypes = [_P, i, i, i, _P, _P, _P, _P]
    L.rh_material_set_texture.argtypes = [_P, i, i, i]
    L.rh_mesh_set_texture_index.argtypes = [_P, i, i, _P]
    L.rh_render_paths.argtypes = [_P, _P, i, _P, i, _P]
    L.rh_first_hits.argtypes = [_P, i, i, i, _P, _P, _P]
    L.rh_probe.argtypes = [_P, _P, _P, fl, _P, _P]
    L.rh_triangle_sw.argtypes = [_P, i, _P, _P, fl, _P]
    L.rh_light.argtypes = [_P, i, i, _P, _P, _P, _P]
    L.rh_stats.argtypes = [_P, _P]
    L.rh_msphere.argtypes = [_P, _P, _P, ctypes.c_float, ctypes.c_float, ctypes.c_float, _P, _P]
    L.ref_tea64.argtypes = [u, u]
    L.ref_tea64.restype = u
    L.ref_lcg_stream.argtypes = [u, i, _P]
    L.ref_rnd_stream.argtypes = [u, i, _P]
    L.ref_sampling.argtypes = [i, u, i, _P]
    L.ref_brdf_sample.argtypes = [i, _P, _P, fl, fl, i, _P, _P, _P, _P]
    L.ref_brdf_eval.argtypes = [i, _P, _P, fl, fl, i, _P, _P, _P, _P, _P]
    L.ref_helper.argtypes = [i, i, _P, _P]
    _lib = L
    return L


class RefPrograms:
    """A ptgb.Scene loaded into the emulated OptiX runtime that runs the
    reference's programs."""

    def __init__(self, scene):
        self.L = load()
        if self.L is None:
            raise RuntimeError("the reference's source tree is not available here")
        self.h = self.L.rh_create()
        _oracle.replay(self.L, "rh_", self.h, scene)

    def __del__(self):
        try:
            self.L.rh_destroy(self.h)
        except Exception:
            pass

    def render_paths(self, width, height, frame, pixels, max_depth=50, rr_enable=1):
        """Per-path radiance of renderPixel (raygen.cu:148-167) for the listed
        pixels (index y*W+x) of frame `frame`.  Russian roulette starts after
        depth 10 as in raygen.cu:112."""
        pix = np.ascontiguousarray(pixels, dtype=np.uint32)
        out = np.zeros((len(pix), 3), dtype=np.float32)
        prm = np.array([width, height, 1, frame, max_depth, rr_enable, 10, 0, 0], np.int32)
        rc = self.L.rh_render_paths(self.h, _p(prm), frame, _p(pix), len(pix), _p(out))
        if rc:
            raise RuntimeError("rh_render_paths failed")
        return out

    def first_hits(self, width, height, frame):
        prim = np.zeros(width * height, dtype=np.int32)
        mat = np.zeros(width * height, dtype=np.int32)
        t = np.zeros(width * height, dtype=np.float32)
        self.L.rh_first_hits(self.h, width, height, frame, _p(prim), _p(mat), _p(t))
        return prim.view(np.uint32), mat.view(np.uint32), t

    def probe(self, o, d, tmin=1e-6):
        t = np.zeros(1, np.float32)
        rec = np.zeros(17, np.float32)
        pid = self.L.rh_probe(self.h, _p(_f(o)), _p(_f(d)), tmin, _p(t), _p(rec))
        return pid, float(t[0]), rec

    def triangle_sw(self, prim, o, d, tmin=1e-6):
        out = np.zeros(3, np.float32)
        ok = self.L.rh_triangle_sw(self.h, prim, _p(_f(o)), _p(_f(d)), tmin, _p(out))
        return (float(out[0]), float(out[1]), float(out[2])) if ok == 1 else None

    def light(self, k, P, seeds):
        P = _f(P)
        seeds = np.ascontiguousarray(seeds, dtype=np.uint32).copy()
        wi = np.zeros((len(P), 3), np.float32)
        pdf = np.zeros(len(P), np.float32)
        self.L.rh_light(self.h, k, len(P), _p(P), _p(seeds), _p(wi), _p(pdf))
        return wi, pdf, seeds

    def stats(self):
        s = np.zeros(2, np.uint64)
        self.L.rh_stats(self.h, _p(s))
        return {"ext_rays": int(s[0]), "shadow_rays": int(s[1])}


def _side(prefix):
    """(library, prefix) of the reference harness ("ref_") or the oracle ("or_")."""
    return (load(), "ref_") if prefix == "ref" else (_oracle.load(), "or_")


def lcg_stream(side, seed, n):
    L, p = _side(side)
    out = np.zeros(n, np.uint32)
    getattr(L, p + "lcg_stream")(seed, n, _p(out))
    return out


def rnd_stream(side, seed, n):
    L, p = _side(side)
    out = np.zeros(n, np.float32)
    getattr(L, p + "rnd_stream")(seed, n, _p(out))
    return out


def tea64(side, a, b):
    L, p = _side(side)
    return getattr(L, p + "tea64")(a, b)


def sampling(side, kind, seed, n):
    L, p = _side(side)
    out = np.zeros((n, 3), np.float32)
    getattr(L, p + "sampling")(kind, seed, n, _p(out))
    return out


def brdf_sample(side, mtype, c0, c1, p0, p1, wo, n, seeds):
    L, p = _side(side)
    wo = _f(wo)
    n_ = _f(n)
    s = np.ascontiguousarray(seeds, np.uint32).copy()
    wi = np.zeros_like(wo)
    c1a = None if c1 is None else _f(c1)
    getattr(L, p + "brdf_sample")(mtype, _p(_f(c0)), _p(c1a), p0, p1, len(wo), _p(wo), _p(n_),
                                  _p(s), _p(wi))
    return wi, s


def brdf_eval(side, mtype, c0, c1, p0, p1, wo, wi, n):
    L, p = _side(side)
    wo, wi, n_ = _f(wo), _f(wi), _f(n)
    f = np.zeros_like(wo)
    pdf = np.zeros(len(wo), np.float32)
    c1a = None if c1 is None else _f(c1)
    getattr(L, p + "brdf_eval")(mtype, _p(_f(c0)), _p(c1a), p0, p1, len(wo), _p(wo), _p(wi),
                                _p(n_), _p(f), _p(pdf))
    return f, pdf


def helper(side, fn, inputs):
    """inputs: (n, 8) float32; returns (n, 4)."""
    L, p = _side(side)
    a = _f(inputs)
    out = np.zeros((len(a), 4), np.float32)
    getattr(L, p + "helper")(fn, len(a), _p(a), _p(out))
    return out


def oracle_light(orc, k, P, seeds):
    L = _oracle.load()
    P = _f(P)
    seeds = np.ascontiguousarray(seeds, dtype=np.uint32).copy()
    wi = np.zeros((len(P), 3), np.float32)
    pdf = np.zeros(len(P), np.float32)
    L.or_light(orc.h, k, len(P), _p(P), _p(seeds), _p(wi), _p(pdf))
    return wi, pdf, seeds


def oracle_probe(orc, o, d, tmin=1e-6):
    L = _oracle.load()
    t = np.zeros(1, np.float32)
    rec = np.zeros(17, np.float32)
    pid = L.or_probe(orc.h, _p(_f(o)), _p(_f(d)), tmin, _p(t), _p(rec))
    return pid, float(t[0]), rec


def msphere(f9, o, d, tmin, tmax, time):
    """programs/hitables/moving_sphere.cu on one ray at `time`: (hit, [t, P,
    shading normal, u, v, Wo] as 12 floats, get_bounds box6)."""
    L = load()
    out = np.zeros(12, np.float32)
    box = np.zeros(6, np.float32)
    hit = L.rh_msphere(_p(_f(f9)), _p(_f(o)), _p(_f(d)), tmin, tmax, time, _p(out), _p(box))
    return bool(hit), out, box
