"""Builds libpt.so (the CUDA path tracer) in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process in parallel, then
linked into optix-path-tracer_gb300/libpt.so.  Numerics flags: -fmad=false
and IEEE division/sqrt on the device, -ffp-contract=off on the host, so the
kernels round exactly like the CPU oracle.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpt.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-I", CSRC,
]
SOURCES = ["pt_kernels.cu", "pt_trace.cu", "pt_api.cu", "pt_batch.cu", "pt_guide.cu", "pt_guide_host.cu", "bvh_host.cpp",
           "bvh_gpu.cu", "pt_io.cpp", "pt_image.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "pt.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append([nvcc] + NVCC_FLAGS + lang + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("nvcc failed for " + cmd[-3])
        return r

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB) or _stale(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    # the C++ facade example (host_includes-style scene code over the C ABI)
    ex_src = os.path.join(HERE, "examples", "cornell.cpp")
    ex_bin = os.path.join(HERE, "examples", "cornell")
    inc = os.path.join(HERE, "..", "include")
    if _stale(ex_bin, [ex_src, LIB, os.path.join(inc, "pt_scene.hpp")]):
        run([os.environ.get("CXX", "g++"), "-O2", "-std=c++14", "-I", inc, ex_src, "-o", ex_bin,
             "-L", HERE, "-lpt", "-Wl,-rpath,$ORIGIN/.."])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
