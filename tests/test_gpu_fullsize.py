"""Parity at the benchmark's full scene size: the 2,097,152-triangle
heightfield (1024x1024 cells, fBm terrain, 256 TS/AS/ON tile materials) with
its 2048x1024 HDR sky, built by both BVH builders (host binned SAH and GPU
LBVH + SAH treelets), against the CPU oracle on the same per-pixel random
streams; and a batch of large meshes (1e5..1e6 triangles) against each
item's own render.

A tree of two million triangles with 8-bit quantised child boxes is where a
conservative-rounding or tie-break error in the builders or the traversal
would show, so the checks are the same as on the small scenes: first-hit
primitive and material ids and hit distances bit-exact, per-path radiance
within 1e-4 relative with at least 99.9 % of paths bit-identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4
CELLS = 1024            # 2 * 1024^2 = 2,097,152 triangles
FH_W, FH_H = 192, 108   # first-hit image
PA_W, PA_H = 96, 54     # per-path image (same 16:9 camera)


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-3)


@pytest.fixture(scope="module")
def fullsize(ptgb_mod, oracle_mod):
    scene = ptgb_mod.heightfield_scene(FH_W, FH_H, cells=CELLS)
    assert len(scene.items[0][2]) == 2 * CELLS * CELLS
    o = oracle_mod.Oracle(scene)
    rends = {b: ptgb_mod.GpuRenderer(scene, builder=b) for b in (1, 2)}
    yield scene, o, rends
    for r in rends.values():
        r.close()


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("frame", [0, 7])
def test_fullsize_first_hits_exact(fullsize, builder, frame):
    _, o, rends = fullsize
    g = rends[builder]
    gp, gm, gt = g.first_hits(FH_W, FH_H, frame)
    op, om, ot = o.first_hits(FH_W, FH_H, frame)
    hit = op != 0xFFFFFFFF
    assert hit.mean() > 0.3, "the camera must see the terrain"
    assert np.array_equal(gp, op), f"{(gp != op).sum()} primitive ids differ"
    assert np.array_equal(gm, om)
    assert np.array_equal(gt[hit], ot[hit])


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("mode", [0, 1])
def test_fullsize_path_radiance(fullsize, ptgb_mod, builder, mode):
    _, o, rends = fullsize
    g = rends[builder]
    prm = ptgb_mod.GpuRenderer.params(PA_W, PA_H, 1, frame0=3, mode=mode)
    gpu = g.render_paths(prm).reshape(-1, 3)
    ref = o.render_paths(PA_W, PA_H, 3, np.arange(PA_W * PA_H), mode=mode)
    err = rel_err(gpu, ref)
    assert err.max() <= REL_TOL, f"max rel err {err.max()}, {np.sum(err > REL_TOL)} paths"
    assert np.mean(np.all(gpu == ref, axis=1)) > 0.999
    assert np.abs(ref).sum() > 0


def test_fullsize_builders_agree_on_accumulation(fullsize, ptgb_mod):
    """Two frames accumulated through either tree give the same image."""
    _, _, rends = fullsize
    prm = ptgb_mod.GpuRenderer.params(PA_W, PA_H, 2, mode=1)
    a = rends[1].render(prm)
    b = rends[2].render(prm)
    assert np.array_equal(a, b)
    assert np.all(a[..., 3] == 2)


def test_large_mesh_batch_items_equal_plain_renders(ptgb_mod):
    """Four heightfields of 1.3e5..1.0e6 triangles in one batch: every item's
    accumulator equals its own pt_render bit for bit."""
    P = ptgb_mod
    env = P.sky_env(512, 256)
    cells = [256, 400, 560, 707]
    rends = [P.GpuRenderer(P.heightfield_scene(64, 48, cells=c, seed=20 + k, env=env))
             for k, c in enumerate(cells)]
    prms = [P.GpuRenderer.params(64, 48, 3 + k, frame0=k, mode=1) for k in range(4)]
    accs = [np.zeros((48, 64, 4), np.float32) for _ in rends]
    b = P.Batch()
    b.render([(r, p, a) for r, p, a in zip(rends, prms, accs)])
    st = b.stats()
    b.close()
    assert st["graph_launches"] == 1
    for k, (r, p, a) in enumerate(zip(rends, prms, accs)):
        ref = r.render(p)
        assert np.array_equal(a, ref), f"item {k} ({2 * cells[k] ** 2} triangles) differs"
    for r in rends:
        r.close()


def test_fullsize_gpu_hit_distances_against_fp64(fullsize, oracle_mod):
    """The GPU's FP32 first-hit distances on the 2.1M-triangle scene, stated
    against the double-precision ray-primitive oracle with the bounds of
    tests/test_fp64_hits.py (|t32 - t64| |d| <= 16 eps tslack; ids differ
    only within 4 eps of an outline)."""
    from test_fp64_hits import check_against_fp64
    scene, _, rends = fullsize
    for builder in (1, 2):
        gp, _, gt = rends[builder].first_hits(FH_W, FH_H, 2)
        kmax, ndis = check_against_fp64(oracle_mod, scene, FH_W, FH_H, 2, gp, gt)
        assert ndis <= 5
