"""Host-side scene construction: transform composition order of the
reference (host_includes/hitables.hpp:61-70,518-523), scene generators."""
import numpy as np


def test_compose_order(ptgb_mod):
    ptgb = ptgb_mod
    T = ptgb.mat_translate((265.0, 0.0, 295.0))
    R = ptgb.mat_rotate(15.0, ptgb.PT_Y_AXIS)
    # Hitable_List::addElementsTo: translate then rotate -> world = T*R*p
    m = ptgb.compose([T, R]).reshape(3, 4)
    p = np.array([165.0, 0.0, 0.0, 1.0])
    assert np.allclose(m @ p, (T @ R @ p)[:3], atol=1e-3)
    # Hitable::addTo reverses: world = R*T*p
    m2 = ptgb.compose([T, R], reverse=True).reshape(3, 4)
    assert np.allclose(m2 @ p, (R @ T @ p)[:3], atol=1e-3)


def test_rotation_right_handed(ptgb_mod):
    R = ptgb_mod.mat_rotate(90.0, 1)
    assert np.allclose(R[:3, :3] @ [1, 0, 0], [0, 0, -1], atol=1e-12)
    R = ptgb_mod.mat_rotate(90.0, 2)
    assert np.allclose(R[:3, :3] @ [1, 0, 0], [0, 1, 0], atol=1e-12)


def test_random_spheres_counts(ptgb_mod):
    s = ptgb_mod.random_spheres()
    assert s.n_prims == 488
    kinds = [m[0] for m in s.materials]
    assert kinds.count(ptgb_mod.MAT_LAMBERTIAN) > 300
    # deterministic
    s2 = ptgb_mod.random_spheres()
    assert s.items == s2.items


def test_heightfield_sizes(ptgb_mod):
    v, idx, n, uv, tile = ptgb_mod.heightfield_mesh(64)
    assert v.shape == (65 * 65, 3) and idx.shape == (2 * 64 * 64, 3)
    assert idx.max() < len(v)
    assert np.allclose(np.linalg.norm(n, axis=1), 1, atol=1e-5)
    assert abs(v[:, 1]).max() <= 0.1 + 1e-6
    env = ptgb_mod.sky_env(64, 32)
    assert env.shape == (32, 64, 4) and env.max() > 1e3
