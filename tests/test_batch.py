"""Batched multi-scene rendering (pt_batch_*): every item's accumulator must
equal, bit for bit, what pt_render gives for the same scene and parameters
(the batch runs the same kernels on the same per-path random streams and
accumulates each pixel's frames in the same order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def empty_scene(ptgb, w, h):
    s = ptgb.Scene()
    s.miss_gradient((1.0, 1.0, 1.0), (0.5, 0.7, 1.0))
    s.set_camera((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), 40.0, w / h, 0.0, 1.0)
    return s


@pytest.fixture(scope="module")
def renderers(ptgb_mod):
    P = ptgb_mod
    out = {
        "cornell_c1": P.GpuRenderer(P.cornell_c1(40, 32)),
        "cornell_ref": P.GpuRenderer(P.cornell_reference(24, 24)),
        "spheres": P.GpuRenderer(P.random_spheres(48, 27)),
        "zoo": P.GpuRenderer(P.material_zoo(32, 24)),
        "heightfield": P.GpuRenderer(P.heightfield_scene(48, 27, cells=40, env_w=128, env_h=64)),
        "empty": P.GpuRenderer(empty_scene(P, 16, 12)),
        "moving": P.GpuRenderer(P.moving_spheres(40, 24, grid=3)),
    }
    yield out
    for r in out.values():
        r.close()


def jobs_ref_mode(P, R):
    prm = P.GpuRenderer.params
    return [
        (R["cornell_c1"], prm(40, 32, 3, rr_depth=3)),
        (R["spheres"], prm(48, 27, 2)),
        (R["zoo"], prm(32, 24, 4, max_depth=7)),
        (R["heightfield"], prm(48, 27, 2)),
        (R["empty"], prm(16, 12, 3)),
        (R["cornell_ref"], prm(24, 24, 5, rr_enable=0, max_depth=12)),
        (R["spheres"], prm(48, 27, 3, frame0=0, rr_depth=2)),  # same scene, other params
        (R["moving"], prm(40, 24, 3)),  # moving spheres: the paths' times in a batch
    ]


def plain(job):
    r, p = job
    return r.render(p)


def run_batch(P, jobs, **tune):
    b = P.Batch()
    if tune:
        t = b.tune()
        t.update(tune)
        b.set_tune(t["path_slots"], t["trace_block"], t["shade_block"], t["bvh_width"],
                   t["chunk_paths"])
    accs = [np.zeros((p.height, p.width, 4), np.float32) for _, p in jobs]
    b.render([(r, p, a) for (r, p), a in zip(jobs, accs)])
    st = b.stats()
    b.close()
    return accs, st


def assert_same(jobs, accs):
    for k, ((r, p), a) in enumerate(zip(jobs, accs)):
        ref = plain((r, p))
        assert np.array_equal(a, ref), (
            f"item {k}: {(a != ref).any(axis=2).sum()} pixels differ, max "
            f"{np.abs(a - ref).max()}")


def test_batch_matches_plain_renders(ptgb_mod, renderers):
    jobs = jobs_ref_mode(ptgb_mod, renderers)
    accs, st = run_batch(ptgb_mod, jobs)
    assert_same(jobs, accs)
    assert st["paths"] == sum(p.width * p.height * p.spp for _, p in jobs)
    assert st["graph_launches"] == 1, "the batch runs as one graph launch"
    assert st["iterations"] > 0


def test_batch_many_chunks(ptgb_mod, renderers):
    # chunks of at most 3000 paths split frames of several items across
    # chunk boundaries; few slots force many iterations per chunk
    jobs = jobs_ref_mode(ptgb_mod, renderers)
    accs, _ = run_batch(ptgb_mod, jobs, chunk_paths=3000, path_slots=1024)
    assert_same(jobs, accs)


@pytest.mark.parametrize("trace_block,shade_block,width", [(64, 128, 8), (256, 96, 4), (128, 256, 2)])
def test_batch_launch_shapes_and_widths(ptgb_mod, renderers, trace_block, shade_block, width):
    jobs = jobs_ref_mode(ptgb_mod, renderers)[:5]
    accs, _ = run_batch(ptgb_mod, jobs, trace_block=trace_block, shade_block=shade_block,
                        bvh_width=width)
    assert_same(jobs, accs)


def test_batch_consistent_mode(ptgb_mod, renderers):
    P, R = ptgb_mod, renderers
    prm = P.GpuRenderer.params
    jobs = [(R["heightfield"], prm(48, 27, 3, mode=1)),
            (R["cornell_c1"], prm(40, 32, 2, mode=1, rr_depth=3)),
            (R["zoo"], prm(32, 24, 2, mode=1, frame0=0))]
    accs, _ = run_batch(P, jobs)
    assert_same(jobs, accs)


def test_batch_progressive_and_device_accumulators(ptgb_mod, renderers):
    torch = pytest.importorskip("torch")
    P, R = ptgb_mod, renderers
    prm = P.GpuRenderer.params
    r1, r2 = R["cornell_c1"], R["zoo"]
    # plain: frames 0..1 then 2..4 accumulated onto the same buffer
    ref1 = r1.render(prm(40, 32, 2))
    ref1 = r1.render(prm(40, 32, 3, frame0=2), acc=ref1)
    ref2 = r2.render(prm(32, 24, 5))
    b = P.Batch()
    host = np.zeros((32, 40, 4), np.float32)
    dev = torch.zeros((24, 32, 4), dtype=torch.float32, device="cuda")
    b.render([(r1, prm(40, 32, 2), host), (r2, prm(32, 24, 5), dev.data_ptr())])
    b.render([(r1, prm(40, 32, 3, frame0=2), host)])
    torch.cuda.synchronize()
    assert np.array_equal(host, ref1)
    assert np.array_equal(dev.cpu().numpy(), ref2)
    b.close()


def test_batch_host_loop_with_stage_timing(ptgb_mod, renderers):
    jobs = jobs_ref_mode(ptgb_mod, renderers)[:4]
    b = ptgb_mod.Batch(timing=True)
    accs = [np.zeros((p.height, p.width, 4), np.float32) for _, p in jobs]
    b.render([(r, p, a) for (r, p), a in zip(jobs, accs)])
    st = b.stats()
    b.close()
    assert_same(jobs, accs)
    assert sum(st["stage_ms"]) > 0.0
    assert st["graph_launches"] >= 1


def test_batch_autotune(ptgb_mod, renderers):
    jobs = jobs_ref_mode(ptgb_mod, renderers)
    b = ptgb_mod.Batch()
    accs = [np.full((p.height, p.width, 4), 7.0, np.float32) for _, p in jobs]
    t = b.autotune([(r, p, a) for (r, p), a in zip(jobs, accs)])
    assert t["sample_paths_per_s"] > 0
    assert t["trace_block"] in (64, 128, 256) and 2 <= t["bvh_width"] <= 8
    assert all((a == 7.0).all() for a in accs), "autotune must not touch the accumulators"
    b.render([(r, p, a) for (r, p), a in zip(jobs, accs)])
    b.close()
    assert_same(jobs, accs)


def test_batch_rejects_bad_input(ptgb_mod, renderers):
    P, R = ptgb_mod, renderers
    prm = P.GpuRenderer.params
    b = P.Batch()
    a = np.zeros((32, 40, 4), np.float32)
    z = np.zeros((24, 32, 4), np.float32)
    with pytest.raises(P.PtError) as e:  # one integrator mode per batch
        b.render([(R["cornell_c1"], prm(40, 32, 1), a), (R["zoo"], prm(32, 24, 1, mode=1), z)])
    assert e.value.code == -1
    with pytest.raises(P.PtError):
        b.render([])
    with pytest.raises(P.PtError):
        b.render([(R["cornell_c1"], prm(40, 32, 0), a)])
    with pytest.raises(P.PtError):
        b.set_tune(100, 128, 256, 8)
    with pytest.raises(P.PtError):
        b.set_tune(1 << 20, 96, 256, 8)
    b.close()
