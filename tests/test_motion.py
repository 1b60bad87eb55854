"""Moving spheres (the reference's Moving_Sphere, host_includes/hitables.hpp:
130-181, programs/hitables/moving_sphere.cu) in the CPU oracle: every ray of a
path carries the path's time (color()'s prd.time, programs/raygen.cu:69) and
meets each moving sphere at its centre for that time."""
import numpy as np
import pytest


def static_at(ptgb, scene, time):
    """The same scene with every moving sphere replaced by a static sphere at
    its centre for `time` (float32 arithmetic of moving_sphere.cu:47-49)."""
    s = ptgb.Scene()
    s.__dict__.update({k: (list(v) if isinstance(v, list) else v) for k, v in scene.__dict__.items()})
    items = []
    for it in scene.items:
        if it[0] == "msphere":
            _, c0, c1, r, t0, t1, m, xf = it
            c0, c1 = np.float32(c0), np.float32(c1)
            k = (np.float32(time) - np.float32(t0)) / (np.float32(t1) - np.float32(t0))
            c = c0 + np.float32(k) * (c1 - c0)
            items.append(("sphere", tuple(float(x) for x in c), r, m, xf))
        else:
            items.append(it)
    s.items = items
    return s


def with_shutter(scene, t0, t1):
    cam = list(scene.camera)
    cam[7], cam[8] = float(t0), float(t1)
    scene.camera = tuple(cam)
    return scene


def test_shutter_closed_equals_static_scene(ptgb_mod, oracle_mod):
    """With the shutter at one instant every path's time is that instant: the
    moving scene renders exactly as the static scene at those centres."""
    W, H = 48, 27
    for t in (0.0, 0.6):
        mov = with_shutter(ptgb_mod.moving_spheres(W, H), t, t)
        sta = static_at(ptgb_mod, mov, t)
        om, os_ = oracle_mod.Oracle(mov), oracle_mod.Oracle(sta)
        pm, mm, tm = om.first_hits(W, H, 0, threads=2)
        ps, ms, ts = os_.first_hits(W, H, 0, threads=2)
        assert np.array_equal(pm, ps) and np.array_equal(mm, ms) and np.array_equal(tm, ts)
        for mode in (0, 1):
            a = om.render_paths(W, H, 1, np.arange(W * H), rr_depth=10, mode=mode, threads=2)
            b = os_.render_paths(W, H, 1, np.arange(W * H), rr_depth=10, mode=mode, threads=2)
            assert np.array_equal(a, b), mode


def test_open_shutter_differs_from_an_instant(ptgb_mod, oracle_mod):
    """With the shutter open the spheres are met at the paths' own times: the
    first hits differ from those of the scene frozen at time 0."""
    W, H = 48, 27
    o = oracle_mod.Oracle(ptgb_mod.moving_spheres(W, H))
    sta = oracle_mod.Oracle(static_at(ptgb_mod, ptgb_mod.moving_spheres(W, H), 0.0))
    p0, _, t0 = o.first_hits(W, H, 0, threads=2)
    q0, _, u0 = sta.first_hits(W, H, 0, threads=2)
    assert (p0 != q0).sum() + (t0 != u0).sum() > 0


@pytest.mark.gpu
def test_moving_sphere_checks(ptgb_mod):
    """pt_add_moving_sphere refuses a non-positive radius, non-finite centres
    and time1 <= time0."""
    import ctypes
    L = ptgb_mod.load_library()
    ctx = ctypes.c_void_p()
    assert L.pt_context_create(None, ctypes.byref(ctx)) == 0
    try:
        mid = ctypes.c_uint32()
        assert L.pt_material_lambertian(ctx, ptgb_mod.f3((1, 1, 1)), ctypes.byref(mid)) == 0
        f3 = ptgb_mod.f3
        ok = L.pt_add_moving_sphere(ctx, f3((0, 0, 0)), f3((0, 1, 0)), 1.0, 0.0, 1.0, 0, None, None)
        assert ok == 0
        assert L.pt_add_moving_sphere(ctx, f3((0, 0, 0)), f3((0, 1, 0)), 0.0, 0.0, 1.0, 0, None,
                                      None) == -1
        assert L.pt_add_moving_sphere(ctx, f3((0, 0, 0)), f3((0, 1, 0)), 1.0, 1.0, 1.0, 0, None,
                                      None) == -1
        assert L.pt_add_moving_sphere(ctx, f3((0, float("nan"), 0)), f3((0, 1, 0)), 1.0, 0.0, 1.0,
                                      0, None, None) == -1
        assert b"time1 > time0" in L.pt_last_error(ctx) or b"finite" in L.pt_last_error(ctx)
    finally:
        L.pt_context_destroy(ctx)
