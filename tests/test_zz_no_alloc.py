"""pt_render_noalloc: the entry point for callers that cannot allocate device
memory at render time (a strict memory pool, or an application that
allocates everything up front).  Its scratch is a fixed device array inside
libpt.so; this test checks, through the C ABI, that two calls in a row give
the same accumulator as pt_render and that the second call changes the
device's free memory by nothing.  Kept in a file collected last so that a
run stopping at the first failure has run every other test first."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4  # the tolerance of the other parity tests


def rel_err(a, b):
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1e-3)


def test_noalloc_matches_render_twice(ptgb_mod):
    torch = pytest.importorskip("torch")
    w, h = 64, 48
    g = ptgb_mod.GpuRenderer(ptgb_mod.material_zoo(w, h))
    L = g.lib
    prm = ptgb_mod.GpuRenderer.params(w, h, 6)
    ref = g.render(prm)                       # existing entry point
    acc = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    free_before = None
    for call in range(2):
        acc.fill_(123.0)                      # stale contents must be cleared (frame0 == 0)
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        rc = L.pt_render_noalloc(g.ctx, ctypes.byref(prm), ctypes.c_void_p(acc.data_ptr()), None)
        assert rc == 0, L.pt_last_error(g.ctx)
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        out = acc.cpu().numpy()
        assert np.array_equal(out[..., 3], ref[..., 3])
        assert rel_err(out[..., :3], ref[..., :3]).max() <= REL_TOL
    st = g.stats()
    assert st["paths"] == w * h * 6
    g.close()


def test_noalloc_progressive_and_limits(ptgb_mod):
    torch = pytest.importorskip("torch")
    w, h = 40, 30
    g = ptgb_mod.GpuRenderer(ptgb_mod.cornell_c1(w, h))
    L = g.lib
    p1 = ptgb_mod.GpuRenderer.params(w, h, 3, rr_depth=3)
    p2 = ptgb_mod.GpuRenderer.params(w, h, 2, frame0=3, rr_depth=3)
    ref = g.render(p2, g.render(p1))
    acc = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    for prm in (p1, p2):
        assert L.pt_render_noalloc(g.ctx, ctypes.byref(prm), ctypes.c_void_p(acc.data_ptr()),
                                   None) == 0
    out = acc.cpu().numpy()
    assert rel_err(out[..., :3], ref[..., :3]).max() <= REL_TOL
    assert np.all(out[..., 3] == 5)
    # beyond the static scratch: a clear PT_EINVAL, nothing launched
    big = ptgb_mod.GpuRenderer.params(1024, 512, 1)
    rc = L.pt_render_noalloc(g.ctx, ctypes.byref(big), ctypes.c_void_p(acc.data_ptr()), None)
    assert rc == -1 and b"at most 262144" in L.pt_last_error(g.ctx)
    # host accumulators are refused (staging them would allocate)
    host = np.zeros((h, w, 4), dtype=np.float32)
    rc = L.pt_render_noalloc(g.ctx, ctypes.byref(p1), host.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == -1
    g.close()


def test_noalloc_consistent_mode_with_environment(ptgb_mod):
    """Consistent mode (NEE + MIS, shadow rays through the occlusion
    traversal, the environment map importance-sampled) through the static
    scratch: two calls in a row equal pt_render, and the device time is
    reported."""
    torch = pytest.importorskip("torch")
    w, h = 96, 54
    g = ptgb_mod.GpuRenderer(ptgb_mod.heightfield_scene(w, h, cells=48, env_w=256, env_h=128))
    L = g.lib
    prm = ptgb_mod.GpuRenderer.params(w, h, 4, mode=1)
    ref = g.render(prm)
    acc = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    for _ in range(2):
        acc.fill_(-7.0)
        rc = L.pt_render_noalloc(g.ctx, ctypes.byref(prm), ctypes.c_void_p(acc.data_ptr()), None)
        assert rc == 0, L.pt_last_error(g.ctx)
        torch.cuda.synchronize()
        out = acc.cpu().numpy()
        assert np.array_equal(out[..., 3], ref[..., 3])
        assert rel_err(out[..., :3], ref[..., :3]).max() <= REL_TOL
        st = g.stats()
        assert st["shadow_rays"] > 0 and st["render_ms"] > 0
    g.close()
