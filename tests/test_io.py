"""File formats on either side of the path, through the C ABI, without a
GPU: OBJ/MTL meshes (the reference's Mesh over tinyobjloader), Radiance
HDR in and out (lib/HDRloader.cpp, Save_HDR) and PNG out (Save_PNG)."""
import struct
import zlib

import numpy as np
import pytest


def write(path, text):
    path.write_text(text)
    return path


def tri_area(t):
    return 0.5 * np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0]))


def test_obj_faces_indices_and_materials(ptgb_mod, tmp_path):
    write(tmp_path / "m.mtl", "newmtl red\nKa 0.8 0.1 0.1\nKd 0.5 0 0\nmap_Kd red.png\n"
                              "newmtl blue\nKa 0.1 0.1 0.9\n")
    obj = write(tmp_path / "m.obj", """# test mesh
mtllib m.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
f 1 2 3
usemtl red
f 1/1/1 2/2/1 3/3/1 4/4/1
usemtl blue
f -4//1 -3//1 -1//1
""")
    m = ptgb_mod.ObjMesh(obj)
    assert m.n_tris == 4 and m.n_materials == 2
    # not every corner has a normal / uv: both dropped (geometric normals)
    assert m.normals is None and m.uvs is None
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    assert np.array_equal(m.verts[0], v[[0, 1, 2]])
    # a convex quad: ears (0,1,2) then (0,2,3), as the reference's loader
    assert np.array_equal(m.verts[1], v[[0, 1, 2]])
    assert np.array_equal(m.verts[2], v[[0, 2, 3]])
    # negative indices count back from the end
    assert np.array_equal(m.verts[3], v[[0, 1, 3]])
    assert list(m.mat) == [ptgb_mod.PT_OBJ_NO_MATERIAL, 0, 0, 1]
    red = m.material(0)
    assert red["name"] == "red" and red["map_Kd"] == "red.png"
    assert np.allclose(red["Ka"], [0.8, 0.1, 0.1]) and np.allclose(red["Kd"], [0.5, 0, 0])
    assert m.material(1)["name"] == "blue"
    m.close()


def test_obj_normals_uvs_kept_when_complete(ptgb_mod, tmp_path):
    obj = write(tmp_path / "t.obj", "v 0 0 0\nv 2 0 0\nv 0 2 0\nvt 0 0\nvt 1 0\nvt 0 1\n"
                                    "vn 0 0 1\nvn 0 1 0\nvn 1 0 0\nf 1/1/1 2/2/2 3/3/3\n")
    m = ptgb_mod.ObjMesh(obj)
    assert m.n_tris == 1 and m.n_materials == 0
    assert np.array_equal(m.normals[0], np.eye(3, dtype=np.float32)[[2, 1, 0]])
    assert np.array_equal(m.uvs[0], np.array([[0, 0], [1, 0], [0, 1]], np.float32))
    m.close()


def test_obj_concave_polygon_ear_clipping(ptgb_mod, tmp_path):
    # an L-shaped hexagon in the xz plane: n - 2 triangles covering its area
    pts = [(0, 0), (2, 0), (2, 1), (1, 1), (1, 2), (0, 2)]
    text = "".join(f"v {x} 0 {z}\n" for x, z in pts) + "f 1 2 3 4 5 6\n"
    m = ptgb_mod.ObjMesh(write(tmp_path / "l.obj", text))
    assert m.n_tris == 4
    total = sum(tri_area(t.astype(np.float64)) for t in m.verts)
    assert abs(total - 3.0) < 1e-6
    # every triangle lies inside the polygon: its centroid is not in the notch
    for t in m.verts:
        c = t.mean(axis=0)
        assert not (c[0] > 1 and c[2] > 1)
    m.close()


def test_obj_errors(ptgb_mod, tmp_path):
    with pytest.raises(ptgb_mod.PtError, match="cannot read"):
        ptgb_mod.ObjMesh(tmp_path / "missing.obj")
    with pytest.raises(ptgb_mod.PtError, match="face index"):
        ptgb_mod.ObjMesh(write(tmp_path / "b.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 7\n"))
    with pytest.raises(ptgb_mod.PtError, match="material library"):
        ptgb_mod.ObjMesh(write(tmp_path / "c.obj", "mtllib nope.mtl\n"))


def rgbe_decode(q):
    q = q.astype(np.float64)
    return q[..., :3] / 256.0 * np.exp2(q[..., 3:4] - 128)


def hdr_header(w, h):
    return f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {h} +X {w}\n".encode()


def test_hdr_load_flat_and_rle(ptgb_mod, tmp_path):
    rng = np.random.default_rng(4)
    w, h = 19, 5
    q = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    q[..., 3] = rng.integers(100, 150, size=(h, w))
    q[1, 3] = q[1, 2]  # some repeats for the run-length rows
    (tmp_path / "flat.hdr").write_bytes(hdr_header(w, h) + q.tobytes())
    # the same pixels with run-length scanlines (2 2 hi lo, then per channel)
    body = bytearray()
    for y in range(h):
        body += bytes([2, 2, w >> 8, w & 0xFF])
        for c in range(4):
            ch = q[y, :, c]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and ch[x + run] == ch[x]:
                    run += 1
                if run >= 3:
                    body += bytes([128 + run, ch[x]])
                    x += run
                else:
                    n = min(w - x, 128)
                    body += bytes([n]) + ch[x:x + n].tobytes()
                    x += n
    (tmp_path / "rle.hdr").write_bytes(hdr_header(w, h) + bytes(body))
    want = rgbe_decode(q)
    for name in ("flat.hdr", "rle.hdr"):
        img = ptgb_mod.hdr_load(tmp_path / name)
        assert img.shape == (h, w, 4)
        assert np.array_equal(img[..., :3], want.astype(np.float32)), name
        assert np.all(img[..., 3] == 1)


def test_hdr_save_reinhard_round_trip(ptgb_mod, tmp_path):
    rng = np.random.default_rng(5)
    acc = (rng.random((7, 11, 4)) * 40).astype(np.float32)
    acc[0, 0, :3] = 0
    ptgb_mod.hdr_save(tmp_path / "o.hdr", acc, 8)
    back = ptgb_mod.hdr_load(tmp_path / "o.hdr")
    c = acc[..., :3].astype(np.float64) / 8
    want = c / (1 + c)
    # RGBE keeps 8 bits of the largest channel's mantissa
    err = np.abs(back[..., :3] - want)
    assert np.all(err <= want.max(axis=2, keepdims=True) / 128 + 1e-12)
    assert np.all(back[0, 0, :3] == 0)


def png_pixels(data):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert zlib.crc32(kind + body) & 0xFFFFFFFF == crc
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 2
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 1 + 3 * w)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def test_png_save_gamma_clamp(ptgb_mod, tmp_path):
    rng = np.random.default_rng(6)
    acc = (rng.random((9, 130, 4)) * 6 - 1).astype(np.float32)  # some negative, some over 1
    spp = 3
    ptgb_mod.png_save(tmp_path / "o.png", acc, spp)
    px = png_pixels((tmp_path / "o.png").read_bytes())
    v = np.sqrt(np.maximum(acc[..., :3] / np.float32(spp), 0).astype(np.float32))
    want = (np.float32(255.99) * np.clip(v, 0, 1)).astype(np.int32).astype(np.uint8)
    assert np.array_equal(px, want)


def test_png_large_image_spans_blocks(ptgb_mod, tmp_path):
    # more than one 65535-byte stored block
    acc = np.full((200, 150, 4), 0.25, np.float32)
    ptgb_mod.png_save(tmp_path / "big.png", acc, 1)
    px = png_pixels((tmp_path / "big.png").read_bytes())
    assert px.shape == (200, 150, 3) and np.all(px == int(255.99 * 0.5))


def test_hdr_old_style_repeats(ptgb_mod, tmp_path):
    # flat pixels with (1, 1, 1, n) markers repeating the previous pixel
    # (consecutive markers shift the count by 8 bits)
    a = [10, 20, 30, 130]
    b = [200, 100, 50, 127]
    body = bytes(a) + bytes([1, 1, 1, 3]) + bytes(b) + bytes([1, 1, 1, 1]) + bytes([1, 1, 1, 0])
    # row of 1 + 3 + 1 + (1 + (0 << 8)) = 6 pixels
    (tmp_path / "o.hdr").write_bytes(hdr_header(6, 1) + body)
    img = ptgb_mod.hdr_load(tmp_path / "o.hdr")
    q = np.array([a, a, a, a, b, b], np.uint8)[None]
    assert np.array_equal(img[..., :3], rgbe_decode(q).astype(np.float32))


def test_obj_crlf_and_convex_fan(ptgb_mod, tmp_path):
    # CRLF line ends, a convex pentagon: ear clipping gives the fan from vertex 0
    ang = np.linspace(0, 2 * np.pi, 6)[:5]
    text = "".join(f"v {np.cos(t):.6f} {np.sin(t):.6f} 0\r\n" for t in ang) + "f 1 2 3 4 5\r\n"
    m = ptgb_mod.ObjMesh(write(tmp_path / "p.obj", text))
    assert m.n_tris == 3
    v = m.verts
    first = v[:, 0, :]
    assert np.allclose(first, first[0])  # every triangle starts at vertex 0
    assert np.allclose(v[0, 1:], [[np.cos(ang[1]), np.sin(ang[1]), 0], [np.cos(ang[2]), np.sin(ang[2]), 0]],
                       atol=1e-6)
    m.close()


# ------------------------------------------------------------------ images
def png_bytes(rows, ctype, depth=8, palette=None, trns=None, level=6, filters=None):
    """A PNG file of the given raw rows (bytes per row), compressed by zlib
    at `level` (0: stored blocks; 1..9: fixed / dynamic Huffman blocks),
    each row filtered with filters[y] (0 none, 1 sub, 2 up, 3 average,
    4 Paeth)."""
    h = len(rows)
    bpp = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype] * depth // 8
    raw = b""
    prev = bytes(len(rows[0]))
    for y, r in enumerate(rows):
        ft = filters[y] if filters else y % 5
        out = bytearray()
        for i, x in enumerate(r):
            a = out_raw_a = r[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ft == 0:
                p = 0
            elif ft == 1:
                p = a
            elif ft == 2:
                p = b
            elif ft == 3:
                p = (a + b) >> 1
            else:
                pp = a + b - c
                pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - c)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            out.append((x - p) & 0xFF)
        raw += bytes([ft]) + bytes(out)
        prev = r

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d))

    w = len(rows[0]) // bpp
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        data += chunk(b"PLTE", bytes(palette))
    if trns is not None:
        data += chunk(b"tRNS", bytes(trns))
    data += chunk(b"IDAT", zlib.compress(raw, level)) + chunk(b"IEND", b"")
    return data


@pytest.mark.parametrize("level", [0, 1, 9])
@pytest.mark.parametrize("ctype", [0, 2, 4, 6])
def test_png_load_colour_types_filters_and_compression(ptgb_mod, tmp_path, level, ctype):
    rng = np.random.default_rng(ctype * 10 + level)
    w, h, ch = 37, 23, {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    px = rng.integers(0, 256, (h, w, ch), dtype=np.uint8)
    px[: h // 2] //= 16                       # runs and repeats for the Huffman coders
    f = tmp_path / "t.png"
    f.write_bytes(png_bytes([px[y].tobytes() for y in range(h)], ctype, level=level))
    img = ptgb_mod.image_load(f)
    assert img.shape == (h, w, 4)
    ref = np.ones((h, w, 4), np.float32)
    v = px.astype(np.float32) / np.float32(255)
    if ch <= 2:
        ref[..., :3] = v[..., :1]
        if ch == 2:
            ref[..., 3] = v[..., 1]
    else:
        ref[..., :ch] = v
    assert np.array_equal(img, ref)


def test_png_load_palette_and_16_bit(ptgb_mod, tmp_path):
    rng = np.random.default_rng(5)
    pal = rng.integers(0, 256, 3 * 16, dtype=np.uint8)
    idx = rng.integers(0, 16, (9, 11), dtype=np.uint8)
    f = tmp_path / "p.png"
    f.write_bytes(png_bytes([idx[y].tobytes() for y in range(9)], 3, palette=pal,
                            trns=[128] * 4))
    img = ptgb_mod.image_load(f)
    assert np.array_equal(img[..., :3], pal.reshape(16, 3)[idx].astype(np.float32) / np.float32(255))
    assert np.array_equal(img[..., 3], np.where(idx < 4, np.float32(128) / np.float32(255), 1.0))
    v16 = rng.integers(0, 65536, (5, 6, 3), dtype=np.uint16)
    f16 = tmp_path / "p16.png"
    f16.write_bytes(png_bytes([v16[y].astype(">u2").tobytes() for y in range(5)], 2, depth=16))
    img16 = ptgb_mod.image_load(f16)
    assert np.array_equal(img16[..., :3], v16.astype(np.float32) / np.float32(65535))


def test_ppm_load_and_unsupported_formats(ptgb_mod, tmp_path):
    px = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3) * 7
    f = tmp_path / "a.ppm"
    f.write_bytes(b"P6\n# comment\n3 2\n255\n" + px.tobytes())
    img = ptgb_mod.image_load(f)
    assert np.array_equal(img[..., :3], px.astype(np.float32) / np.float32(255))
    g = tmp_path / "b.ppm"
    g.write_text("P3 3 2 255\n" + " ".join(str(x) for x in px.reshape(-1)) + "\n")
    assert np.array_equal(ptgb_mod.image_load(g), img)
    j = tmp_path / "c.jpg"
    j.write_bytes(b"\xff\xd8\xff\xe0" + bytes(16))
    with pytest.raises(ptgb_mod.PtError, match="JPEG"):
        ptgb_mod.image_load(j)
    bad = tmp_path / "d.png"
    bad.write_bytes(png_bytes([bytes(12)] * 2, 2)[:-30])   # truncated
    with pytest.raises(ptgb_mod.PtError):
        ptgb_mod.image_load(bad)
