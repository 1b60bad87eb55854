"""An OBJ/MTL mesh through the renderer: the loaded triangles render exactly
as the oracle renders the same arrays, and pt_add_obj (materials from the
MTL file) gives the same image as the arrays through pt_add_mesh."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def obj_grid(tmp_path, n=8, seed=3):
    rng = np.random.default_rng(seed)
    (tmp_path / "g.mtl").write_text("newmtl warm\nKa 0.8 0.5 0.3\nnewmtl cool\nKa 0.3 0.5 0.8\n")
    lines = ["mtllib g.mtl"]
    for j in range(n + 1):
        for i in range(n + 1):
            lines.append(f"v {i / n * 2 - 1:.6f} {rng.random() * 0.2:.6f} {j / n * 2 - 1:.6f}")
    lines.append("vn 0 1 0")
    for j in range(n):
        lines.append("usemtl " + ("warm" if j % 2 == 0 else "cool"))
        for i in range(n):
            a = j * (n + 1) + i + 1
            b, c, d = a + 1, a + n + 2, a + n + 1
            lines.append(f"f {a}//1 {b}//1 {c}//1 {d}//1")  # quads, ear-clipped
    path = tmp_path / "g.obj"
    path.write_text("\n".join(lines) + "\n")
    return path


def scene_with(ptgb, mesh, via_add_obj):
    s = ptgb.Scene()
    s.obj(mesh, via_add_obj=via_add_obj)
    s.sphere((0.0, 0.5, 0.0), 0.3, s.metal((0.9, 0.9, 0.9), 0.1))
    s.miss_gradient((1.0, 1.0, 1.0), (0.5, 0.7, 1.0))
    s.set_camera((0.0, 1.5, 2.5), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, 1.0, 0.0, 1.0)
    return s


def test_obj_mesh_matches_oracle(ptgb_mod, oracle_mod, tmp_path):
    m = ptgb_mod.ObjMesh(obj_grid(tmp_path))
    assert m.n_tris == 128 and m.normals is not None
    s = scene_with(ptgb_mod, m, False)
    g, o = ptgb_mod.GpuRenderer(s), oracle_mod.Oracle(s)
    w = h = 48
    gp, gm, gt = g.first_hits(w, h, 0)
    op, om, ot = o.first_hits(w, h, 0)
    assert np.array_equal(gp, op) and np.array_equal(gm, om)
    assert (op < 128).sum() > 0.3 * w * h  # the mesh is in view
    prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=2)
    gpu = g.render_paths(prm).reshape(-1, 3)
    ref = o.render_paths(w, h, 2, np.arange(w * h))
    err = np.abs(gpu - ref) / np.maximum(np.maximum(np.abs(gpu), np.abs(ref)), 1e-3)
    assert err.max() <= 1e-4
    g.close()
    m.close()


def test_add_obj_equals_add_mesh(ptgb_mod, tmp_path):
    m = ptgb_mod.ObjMesh(obj_grid(tmp_path))
    imgs = []
    for via in (False, True):
        g = ptgb_mod.GpuRenderer(scene_with(ptgb_mod, m, via))
        imgs.append(g.render(ptgb_mod.GpuRenderer.params(40, 40, 4)))
        g.close()
    assert np.array_equal(imgs[0], imgs[1])
    assert imgs[0][..., :3].mean() > 0
    ptgb_mod.png_save(tmp_path / "obj.png", imgs[1], 4)
    assert (tmp_path / "obj.png").stat().st_size > 40 * 40 * 3
    m.close()


def test_obj_map_kd_image_texture(ptgb_mod, oracle_mod, tmp_path):
    """The reference's Mesh with an MTL file (mesh.hpp:78-98): a map_Kd PNG
    becomes an image texture (rows flipped as Image_Texture stores them),
    the other material a constant Ka, inside one vector texture indexed per
    face.  pt_add_obj builds it from the files; it renders as the oracle
    renders the same structure, and bright and dark texels of the image
    show in the image."""
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    from test_io import png_bytes
    n = 8
    img = np.zeros((16, 16, 3), np.uint8)
    img[:8] = (230, 40, 40)          # top half of the file: red
    img[8:] = (40, 40, 230)          # bottom half: blue
    (tmp_path / "tex.png").write_bytes(png_bytes([img[y].tobytes() for y in range(16)], 2, level=9))
    (tmp_path / "t.mtl").write_text("newmtl pic\nKa 0.1 0.1 0.1\nmap_Kd tex.png\n"
                                    "newmtl plain\nKa 0.2 0.7 0.2\n")
    lines = ["mtllib t.mtl"]
    for j in range(n + 1):
        for i in range(n + 1):
            lines.append(f"v {i / n * 2 - 1:.6f} 0 {j / n * 2 - 1:.6f}")
            lines.append(f"vt {i / n:.6f} {j / n:.6f}")
    lines.append("vn 0 1 0")
    for j in range(n):
        lines.append("usemtl " + ("pic" if j < n - 2 else "plain"))
        for i in range(n):
            a = j * (n + 1) + i + 1
            b, c, d = a + 1, a + n + 2, a + n + 1
            lines.append(f"f {a}/{a}/1 {b}/{b}/1 {c}/{c}/1 {d}/{d}/1")
    (tmp_path / "t.obj").write_text("\n".join(lines) + "\n")
    m = ptgb_mod.ObjMesh(tmp_path / "t.obj")
    assert m.uvs is not None and m.material(0)["map_Kd"] == "tex.png"
    w = h = 48
    imgs = []
    for via in (False, True):
        s = scene_with(ptgb_mod, m, via)
        g = ptgb_mod.GpuRenderer(s)
        imgs.append(g.render(ptgb_mod.GpuRenderer.params(w, h, 3)))
        if not via:
            o = oracle_mod.Oracle(s)
            prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=1)
            gpu = g.render_paths(prm).reshape(-1, 3)
            ref = o.render_paths(w, h, 1, np.arange(w * h))
            err = np.abs(gpu - ref) / np.maximum(np.maximum(np.abs(gpu), np.abs(ref)), 1e-3)
            assert err.max() <= 1e-4
        g.close()
    assert np.array_equal(imgs[0], imgs[1])
    mean = imgs[0][..., :3].reshape(-1, 3).mean(0)
    assert mean[0] > 0.05 and mean[2] > 0.05        # red and blue texels both seen
    m.close()
