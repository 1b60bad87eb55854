"""GPU path tracer vs the CPU oracle (same scenes, same per-pixel random
streams).  Contract: first-hit primitive and material ids bit-exact, per-path
radiance within 1e-4 relative (the arithmetic is shared bit for bit, so the
kernels in fact reproduce the oracle exactly)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4


def scenes(ptgb):
    return {
        "cornell_ref": (ptgb.cornell_reference(64, 64), 64, 64, dict(rr_depth=10)),
        "cornell_c1": (ptgb.cornell_c1(64, 64), 64, 64, dict(rr_depth=3)),
        "spheres_c2": (ptgb.random_spheres(96, 54), 96, 54, dict(rr_depth=10)),
        "zoo": (ptgb.material_zoo(80, 60), 80, 60, dict(rr_depth=10)),
        "heightfield_c3": (ptgb.heightfield_scene(96, 54, cells=48, env_w=256, env_h=128), 96, 54,
                           dict(rr_depth=10)),
        "moving": (ptgb.moving_spheres(96, 54), 96, 54, dict(rr_depth=10)),
    }


@pytest.fixture(scope="module")
def cases(ptgb_mod, oracle_mod):
    out = {}
    for name, (s, w, h, kw) in scenes(ptgb_mod).items():
        out[name] = (ptgb_mod.GpuRenderer(s), oracle_mod.Oracle(s), w, h, kw)
    yield out
    for g, *_ in out.values():
        g.close()


NAMES = ["cornell_ref", "cornell_c1", "spheres_c2", "zoo", "heightfield_c3", "moving"]


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("frame", [0, 5])
def test_first_hits_exact(cases, name, frame):
    g, o, w, h, _ = cases[name]
    gp, gm, gt = g.first_hits(w, h, frame)
    op, om, ot = o.first_hits(w, h, frame)
    assert np.array_equal(gp, op), f"{(gp != op).sum()} prim ids differ"
    assert np.array_equal(gm, om)
    hit = op != 0xFFFFFFFF
    assert np.array_equal(gt[hit], ot[hit])


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-3)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("frame", [0, 3])
def test_path_radiance(cases, ptgb_mod, name, frame):
    g, o, w, h, kw = cases[name]
    prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=frame, **kw)
    gpu = g.render_paths(prm).reshape(-1, 3)
    ref = o.render_paths(w, h, frame, np.arange(w * h), **kw)
    err = rel_err(gpu, ref)
    assert err.max() <= REL_TOL, f"max rel err {err.max()}, {np.sum(err > REL_TOL)} paths"
    exact = np.mean(np.all(gpu == ref, axis=1))
    assert exact > 0.999


@pytest.mark.parametrize("name", ["cornell_c1", "spheres_c2", "zoo"])
def test_accumulation_matches(cases, ptgb_mod, name):
    g, o, w, h, kw = cases[name]
    prm = ptgb_mod.GpuRenderer.params(w, h, 6, frame0=0, **kw)
    acc = g.render(prm)
    ref, _ = o.render(w, h, 6, frame0=0, **kw)
    assert np.array_equal(acc[..., 3], ref[..., 3])
    assert rel_err(acc[..., :3], ref[..., :3]).max() <= REL_TOL
    # progressive continuation: frames 6..9 on top
    prm2 = ptgb_mod.GpuRenderer.params(w, h, 4, frame0=6, **kw)
    acc2 = g.render(prm2, acc.copy())
    ref2, _ = o.render(w, h, 4, frame0=6, acc=ref.copy(), **kw)
    assert rel_err(acc2[..., :3], ref2[..., :3]).max() <= REL_TOL
    assert np.all(acc2[..., 3] == 10)


def test_chunked_render_equals_single(ptgb_mod):
    """Regeneration with few path slots must not change any path."""
    s = ptgb_mod.material_zoo(40, 30)
    a = ptgb_mod.GpuRenderer(s, path_slots=1000)
    b = ptgb_mod.GpuRenderer(s)
    prm = ptgb_mod.GpuRenderer.params(40, 30, 5)
    ra, rb = a.render(prm), b.render(prm)
    assert np.array_equal(ra, rb)
    st = a.stats()
    assert st["paths"] == 40 * 30 * 5 and st["ext_rays"] > st["paths"]


def test_resolve_display(cases, ptgb_mod):
    g, o, w, h, kw = cases["cornell_c1"]
    acc = g.render(ptgb_mod.GpuRenderer.params(w, h, 2, **kw))
    disp = g.resolve(acc, 1)
    ref = np.clip(np.sqrt(acc[..., :3] / 2), 0, 1)
    assert np.abs(disp[..., :3].astype(np.int32) - (255.99 * ref).astype(np.int32)).max() <= 1
    assert np.all(disp[..., 3] == 255)


def test_errors(ptgb_mod):
    import ctypes
    L = ptgb_mod.load_library()
    ctx = ctypes.c_void_p()
    assert L.pt_context_create(None, ctypes.byref(ctx)) == 0
    prm = ptgb_mod.GpuRenderer.params(8, 8, 1)
    acc = np.zeros((8, 8, 4), dtype=np.float32)
    rc = L.pt_render(ctx, ctypes.byref(prm), acc.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == -6  # PT_ESTATE: not committed
    mid = ctypes.c_uint32()
    assert L.pt_material_lambertian(ctx, ptgb_mod.f3((1, 1, 1)), ctypes.byref(mid)) == 0
    assert L.pt_add_sphere(ctx, ptgb_mod.f3((0, 0, 0)), -1.0, 0, None, None) == -1
    assert L.pt_add_sphere(ctx, ptgb_mod.f3((0, 0, 0)), 1.0, 7, None, None) == -1
    assert L.pt_add_rect(ctx, 0, 1, 0, 1, 0, 0, 5, 0, None, None) == -1
    assert L.pt_commit(ctx) == 0
    bad = ptgb_mod.GpuRenderer.params(0, 8, 1)
    assert L.pt_render(ctx, ctypes.byref(bad), acc.ctypes.data_as(ctypes.c_void_p), None) == -1
    assert b"invalid" in L.pt_last_error(ctx)
    # empty scene renders the miss colour
    assert L.pt_render(ctx, ctypes.byref(prm), acc.ctypes.data_as(ctypes.c_void_p), None) == 0
    assert L.pt_context_destroy(ctx) == 0


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("name", ["zoo", "heightfield", "spheres", "moving"])
def test_builders_match_oracle(ptgb_mod, oracle_mod, builder, name):
    """The host (binned SAH) and GPU (LBVH + treelets) BVH8 builders give the
    same first hits and paths as the oracle (moving spheres: boxes over the
    camera's shutter)."""
    if name == "zoo":
        s, w, h = ptgb_mod.material_zoo(64, 48), 64, 48
    elif name == "moving":
        s, w, h = ptgb_mod.moving_spheres(64, 36, grid=8), 64, 36
    elif name == "spheres":
        s, w, h = ptgb_mod.random_spheres(64, 36), 64, 36
    else:
        s, w, h = ptgb_mod.heightfield_scene(64, 36, cells=80, env_w=128, env_h=64), 64, 36
    g = ptgb_mod.GpuRenderer(s, builder=builder)
    o = oracle_mod.Oracle(s)
    gp, gm, gt = g.first_hits(w, h, 1)
    op, om, ot = o.first_hits(w, h, 1)
    assert np.array_equal(gp, op) and np.array_equal(gm, om)
    prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=2)
    gpu = g.render_paths(prm).reshape(-1, 3)
    ref = o.render_paths(w, h, 2, np.arange(w * h))
    assert rel_err(gpu, ref).max() <= REL_TOL
    st = g.stats()
    assert st["bvh_nodes"] > 0 and st["bvh_depth"] >= 1
    g.close()


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("width", [2, 4, 6])
def test_node_width_keeps_results(ptgb_mod, builder, width):
    """Narrower BVH nodes (2..8 children) change traversal, never results:
    first hits and paths equal the 8-wide tree's bit for bit."""
    s, w, h = ptgb_mod.heightfield_scene(64, 36, cells=80, env_w=128, env_h=64), 64, 36
    ref = ptgb_mod.GpuRenderer(s, builder=builder)
    g = ptgb_mod.GpuRenderer(s, builder=builder, bvh_width=width)
    for a, b in zip(g.first_hits(w, h, 3), ref.first_hits(w, h, 3)):
        assert np.array_equal(a, b)
    prm = ptgb_mod.GpuRenderer.params(w, h, 2, mode=1)
    assert np.array_equal(g.render(prm), ref.render(prm))
    assert g.stats()["bvh_depth"] >= ref.stats()["bvh_depth"]
    g.close()
    ref.close()


def test_gpu_builder_large_mesh(ptgb_mod):
    """GPU builder on 2M triangles: valid tree (checked at commit), sane
    depth and node count, and a render that completes."""
    s = ptgb_mod.heightfield_scene(64, 36, cells=1024, env_w=64, env_h=32)
    g = ptgb_mod.GpuRenderer(s, builder=2)
    st = g.stats()
    assert st["bvh_depth"] <= 24
    assert 2 * 1024 * 1024 // 24 < st["bvh_nodes"] < 2 * 1024 * 1024
    # host-to-device bytes of the commit: 48-byte records and 16-byte
    # attributes per triangle, per-vertex normals and uvs, the environment
    n, nv = 2 * 1024 * 1024, 1025 * 1025
    least = 64 * n + 20 * nv + 64 * 32 * 16
    assert least <= st["upload_bytes"] < least + (1 << 20)
    acc = g.render(ptgb_mod.GpuRenderer.params(64, 36, 2))
    assert np.isfinite(acc).all() and np.all(acc[..., 3] == 2)
    g.close()


CONSISTENT = ["cornell_c1", "zoo", "heightfield_c3", "spheres_c2", "moving"]


@pytest.mark.parametrize("name", CONSISTENT)
@pytest.mark.parametrize("frame", [0, 2])
def test_consistent_mode_paths(cases, ptgb_mod, name, frame):
    """Consistent mode (NEE + MIS, environment importance sampling) on the GPU
    reproduces the oracle's consistent mode path for path."""
    g, o, w, h, kw = cases[name]
    prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=frame, mode=1, **kw)
    gpu = g.render_paths(prm).reshape(-1, 3)
    ref = o.render_paths(w, h, frame, np.arange(w * h), mode=1, **kw)
    err = rel_err(gpu, ref)
    assert err.max() <= REL_TOL, f"max rel err {err.max()}, {np.sum(err > REL_TOL)} paths"
    assert np.mean(np.all(gpu == ref, axis=1)) > 0.999


def test_consistent_accumulation_and_env_sampling(cases, ptgb_mod):
    g, o, w, h, kw = cases["heightfield_c3"]
    prm = ptgb_mod.GpuRenderer.params(w, h, 4, mode=1, **kw)
    acc = g.render(prm)
    ref, st = o.render(w, h, 4, mode=1, **kw)
    assert rel_err(acc[..., :3], ref[..., :3]).max() <= REL_TOL
    gs = g.stats()
    assert gs["shadow_rays"] == st["shadow_rays"] > 0   # environment NEE ran


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", ["zoo", "heightfield_c3", "spheres_c2"])
def test_material_sorted_shading_keeps_results(cases, ptgb_mod, name, mode):
    """Shading in material-sorted tiles (the default) and in path order give
    the same image bit for bit: the order changes which warp runs a path,
    never its arithmetic."""
    g, _, w, h, kw = cases[name]
    srt = ptgb_mod.GpuRenderer(g.scene, shade_order=1)
    unsorted = ptgb_mod.GpuRenderer(g.scene, shade_order=2)
    prm = ptgb_mod.GpuRenderer.params(w, h, 3, frame0=1, mode=mode, **kw)
    ref = g.render(prm)
    assert np.array_equal(srt.render(prm), ref)
    assert np.array_equal(unsorted.render(prm), ref)
    srt.close()
    unsorted.close()


def test_double_accumulation(cases, ptgb_mod):
    """pt_render_accum64: per-pixel sums in double, frame order.  Equals the
    host's double sum of the per-frame path colours exactly, carries the same
    counts as the float accumulator, and continues progressively."""
    g, _, w, h, kw = cases["zoo"]
    frames = [g.render_paths(ptgb_mod.GpuRenderer.params(w, h, 1, frame0=f, **kw))
              for f in range(5)]
    ref = np.zeros((h, w, 3), np.float64)
    for fr in frames:
        ref += fr.astype(np.float64)
    ref = ref[::-1]                           # accumulator rows are y-flipped
    acc = g.render64(ptgb_mod.GpuRenderer.params(w, h, 3, **kw))
    acc = g.render64(ptgb_mod.GpuRenderer.params(w, h, 2, frame0=3, **kw), acc)
    assert np.array_equal(acc[..., :3], ref)
    assert np.all(acc[..., 3] == 5.0)
    f32 = g.render(ptgb_mod.GpuRenderer.params(w, h, 5, **kw))
    assert np.abs(f32[..., :3] - acc[..., :3]).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_double_accumulation_many_frames(ptgb_mod):
    """6000 frames (beyond where float sums drop low bits): the double sums
    of one call equal those of three progressive calls bit for bit (the same
    additions in the same frame order), the counts are exact, and the mean
    agrees with the float accumulator's to float accuracy."""
    g = ptgb_mod.GpuRenderer(ptgb_mod.cornell_c1(8, 8))
    P = ptgb_mod.GpuRenderer.params
    n = 6000
    one = g.render64(P(8, 8, n, rr_depth=3))
    acc = g.render64(P(8, 8, 2000, rr_depth=3))
    acc = g.render64(P(8, 8, 2000, frame0=2000, rr_depth=3), acc)
    acc = g.render64(P(8, 8, 2000, frame0=4000, rr_depth=3), acc)
    assert np.array_equal(one, acc)
    assert np.all(one[..., 3] == n)
    a32 = g.render(P(8, 8, n, rr_depth=3))
    m64, m32 = one[..., :3] / n, a32[..., :3].astype(np.float64) / n
    assert np.abs(m64 - m32).max() <= 1e-3 * max(1.0, m64.max())
    g.close()


def env_variant(ptgb, variant, w=48, h=36):
    s = ptgb.material_zoo(w, h)
    env = ptgb.sky_env(128, 64)
    if variant == "cylindrical":
        s.miss_env(env, spherical=False)     # programs/miss.cu:79-91
    else:
        s.miss_env(env, kind=ptgb.MISS_IMG)  # programs/miss.cu:51-59
    return s


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("variant", ["cylindrical", "image"])
def test_env_mapping_variants(ptgb_mod, oracle_mod, variant, mode):
    """The cylindrical HDR mapping and the image-background miss program
    (no importance sampling: only the spherical HDR map has sampling
    tables) match the oracle path for path in both integrator modes."""
    w, h = 48, 36
    s = env_variant(ptgb_mod, variant, w, h)
    g, o = ptgb_mod.GpuRenderer(s), oracle_mod.Oracle(s)
    gp, gm, gt = g.first_hits(w, h, 1)
    op, om, ot = o.first_hits(w, h, 1)
    assert np.array_equal(gp, op) and np.array_equal(gm, om)
    prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=4, mode=mode)
    gpu = g.render_paths(prm).reshape(-1, 3)
    ref = o.render_paths(w, h, 4, np.arange(w * h), mode=mode)
    err = rel_err(gpu, ref)
    assert err.max() <= REL_TOL, f"max rel err {err.max()}, {np.sum(err > REL_TOL)} paths"
    assert np.mean(np.all(gpu == ref, axis=1)) > 0.999
    assert (op == 0xFFFFFFFF).any(), "the camera must see the background"
    g.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_textures_match_oracle(ptgb_mod, oracle_mod, mode):
    """Every texture callable (checker of a checker, Perlin noise, image,
    gradient, a vector texture indexed per mesh face) on every material it
    can colour, including both Ashikhmin-Shirley colours and an emitter: the
    oracle's paths, whose textures are in turn pinned to the reference's own
    texture programs (tests/test_ref_pin.py)."""
    w, h = 96, 72
    s = ptgb_mod.texture_zoo(w, h)
    g, o = ptgb_mod.GpuRenderer(s), oracle_mod.Oracle(s)
    gp, gm, gt = g.first_hits(w, h, 0)
    op, om, ot = o.first_hits(w, h, 0)
    assert np.array_equal(gp, op) and np.array_equal(gm, om)
    for frame in (0, 2):
        prm = ptgb_mod.GpuRenderer.params(w, h, 1, frame0=frame, mode=mode)
        gpu = g.render_paths(prm).reshape(-1, 3)
        ref = o.render_paths(w, h, frame, np.arange(w * h), mode=mode)
        err = rel_err(gpu, ref)
        assert err.max() <= REL_TOL, f"max rel err {err.max()}, {np.sum(err > REL_TOL)} paths"
        assert np.mean(np.all(gpu == ref, axis=1)) > 0.999
    # progressive accumulation through the texture-colour hand-over of k_finish
    acc = g.render(ptgb_mod.GpuRenderer.params(w, h, 3, mode=mode))
    ref, _ = o.render(w, h, 3, mode=mode)
    assert rel_err(acc[..., :3], ref[..., :3]).max() <= REL_TOL
    g.close()


def test_textured_scene_in_a_batch(ptgb_mod):
    """A textured scene rendered in a batch beside untextured ones equals its
    own render (each item reads its own texture tables)."""
    P = ptgb_mod
    rs = [P.GpuRenderer(P.texture_zoo(48, 36)), P.GpuRenderer(P.material_zoo(40, 30)),
          P.GpuRenderer(P.texture_zoo(32, 24))]
    prms = [P.GpuRenderer.params(48, 36, 3), P.GpuRenderer.params(40, 30, 2),
            P.GpuRenderer.params(32, 24, 4, frame0=5)]
    accs = [np.zeros((p.height, p.width, 4), np.float32) for p in prms]
    b = P.Batch()
    b.render([(r, p, a) for r, p, a in zip(rs, prms, accs)])
    b.close()
    for r, p, a in zip(rs, prms, accs):
        assert np.array_equal(a, r.render(p))
        r.close()
