"""Malformed files against the host readers (PNG, PPM, Radiance HDR, OBJ/MTL):
seed files of every form the readers accept, each mutated a few hundred
times (bytes flipped or replaced, cut short, spans duplicated or dropped,
32-bit sizes overwritten) by tests/io_fuzz_driver.cpp, built here with the
address and undefined-behaviour sanitizers.  A reader must return an error
or a consistent result; an out-of-bounds access, an uncaught exception or a
write past the caller's w*h*4 floats fails the test."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from test_io import hdr_header, png_bytes

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.join(HERE, "..")
CSRC = os.path.join(REPO, "optix-path-tracer_gb300", "csrc")
MUTATIONS = 400


def seeds(d):
    rng = np.random.default_rng(11)
    out = []
    for ctype, ch in ((0, 1), (2, 3), (4, 2), (6, 4)):
        for level in (0, 9):
            px = rng.integers(0, 256, (7, 9, ch), dtype=np.uint8)
            px[:3] //= 32
            p = d / f"s_{ctype}_{level}.png"
            p.write_bytes(png_bytes([px[y].tobytes() for y in range(7)], ctype, level=level))
            out.append(p)
    pal = rng.integers(0, 256, 3 * 8, dtype=np.uint8)
    idx = rng.integers(0, 8, (5, 6), dtype=np.uint8)
    p = d / "s_pal.png"
    p.write_bytes(png_bytes([idx[y].tobytes() for y in range(5)], 3, palette=pal, trns=[9, 99]))
    out.append(p)
    v16 = rng.integers(0, 65536, (4, 5, 3), dtype=np.uint16)
    p = d / "s_16.png"
    p.write_bytes(png_bytes([v16[y].astype(">u2").tobytes() for y in range(4)], 2, depth=16))
    out.append(p)
    q = rng.integers(0, 256, (4, 12, 4), dtype=np.uint8)
    p = d / "s_flat.hdr"
    p.write_bytes(hdr_header(12, 4) + q.tobytes())
    out.append(p)
    body = bytearray()
    for y in range(4):
        body += bytes([2, 2, 0, 12])
        for c in range(4):
            body += bytes([128 + 5, q[y, 0, c]]) + bytes([7]) + q[y, 5:12, c].tobytes()
    p = d / "s_rle.hdr"
    p.write_bytes(hdr_header(12, 4) + bytes(body))
    out.append(p)
    p = d / "s_old.hdr"
    p.write_bytes(hdr_header(6, 1) + bytes([10, 20, 30, 130, 1, 1, 1, 3, 200, 100, 50, 127,
                                            1, 1, 1, 1, 1, 1, 1, 0]))
    out.append(p)
    px = rng.integers(0, 256, (3, 4, 3), dtype=np.uint8)
    p = d / "s6.ppm"
    p.write_bytes(b"P6\n# c\n4 3\n255\n" + px.tobytes())
    out.append(p)
    p = d / "s3.ppm"
    p.write_text("P3 4 3 255\n" + " ".join(str(x) for x in px.reshape(-1)) + "\n")
    out.append(p)
    (d / "fz.mtl").write_text("newmtl red\nKa 0.8 0.1 0.1\nKd 0.5 0 0\nmap_Kd red.png\n"
                              "newmtl blue\nKa 0.1 0.1 0.9\n# note\nnewmtl green\nKa 0 1 0\n")
    out.append(d / "fz.mtl")
    p = d / "s.obj"
    p.write_text("mtllib fz.mtl\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0.5 0.2 0\n"
                 "vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nvn 0 0 1\n"
                 "f 1 2 3\nusemtl red\nf 1/1/1 2/2/1 3/3/1 4/4/1\nusemtl blue\n"
                 "f -5//1 -4//1 -2//1\nf 1 2 5 3 4\nusemtl nosuch\nf 2 3 4\n")
    out.append(p)
    return out


def test_readers_survive_malformed_files(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "io_fuzz")
    build = subprocess.run(
        [cxx, "-std=c++17", "-g", "-O1", "-fsanitize=address,undefined",
         "-fno-sanitize-recover=undefined", "-I", os.path.join(REPO, "include"),
         os.path.join(HERE, "io_fuzz_driver.cpp"), os.path.join(CSRC, "pt_image.cpp"),
         os.path.join(CSRC, "pt_io.cpp"), "-o", exe], capture_output=True, text=True)
    if build.returncode != 0 and "sanitize" in build.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert build.returncode == 0, build.stderr[-2000:]
    work = tmp_path / "work"
    work.mkdir()
    files = seeds(tmp_path)
    (work / "mtlref.obj").write_text("mtllib fz.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nusemtl red\n"
                                     "f 1 2 3\nusemtl green\nf 3 2 1\n")
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0",
               UBSAN_OPTIONS="print_stacktrace=1")
    run = subprocess.run([exe, str(work), str(MUTATIONS)] + [str(f) for f in files],
                         capture_output=True, text=True, env=env, timeout=600)
    tail = (run.stdout[-3000:] + run.stderr[-3000:])
    assert run.returncode == 0, tail
    assert run.stdout.strip().splitlines()[-1] == f"ALL PASS {MUTATIONS * len(files)} files", tail


def test_readers_refuse_sizes_their_data_cannot_hold(ptgb_mod, tmp_path):
    """Headers that claim far more pixels than their files can carry fail at
    the size query, before a caller sizes a buffer by them."""
    big = tmp_path / "big.png"
    big.write_bytes(png_bytes([bytes(4 * 32)] * 2, 6)[:33]        # signature + IHDR of 32x2
                    .replace(b"\x00\x00\x00\x20\x00\x00\x00\x02", b"\x00\x00\x80\x00\x00\x00\x80\x00")
                    + png_bytes([bytes(4)], 6)[33:])               # a one-pixel IDAT, IEND
    with pytest.raises(ptgb_mod.PtError, match="too short"):
        ptgb_mod.image_load(big)
    ppm = tmp_path / "big.ppm"
    ppm.write_bytes(b"P6 32768 32768 255\n" + bytes(300))
    with pytest.raises(ptgb_mod.PtError, match="truncated"):
        ptgb_mod.image_load(ppm)
    txt = tmp_path / "big3.ppm"
    txt.write_text("P3 1000 1000 255\n1 2 3\n")
    with pytest.raises(ptgb_mod.PtError, match="truncated"):
        ptgb_mod.image_load(txt)
    hdr = tmp_path / "big.hdr"
    hdr.write_bytes(hdr_header(65536, 65536) + bytes(64))
    with pytest.raises(ptgb_mod.PtError, match="too large"):
        ptgb_mod.hdr_load(hdr)
    hdr2 = tmp_path / "tall.hdr"
    hdr2.write_bytes(hdr_header(8, 4096) + bytes(64))
    with pytest.raises(ptgb_mod.PtError, match="truncated"):
        ptgb_mod.hdr_load(hdr2)
