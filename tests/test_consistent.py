"""Consistent mode (the unbiased integrator used for environment importance
sampling and the learned guide): pdf normalisation of every BSDF sampler,
agreement of samplers with their pdfs, environment-CDF sampling, and
white-furnace integrals in the CPU oracle."""
import math

import numpy as np
import pytest


def uniform_sphere(n, rng):
    z = rng.uniform(-1, 1, n)
    phi = rng.uniform(0, 2 * math.pi, n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(phi), z, r * np.sin(phi)], axis=1).astype(np.float32)


MATERIALS = [
    (0, (0.8, 0.8, 0.8), None, 0.0, 0.0),                # Lambertian
    (4, (0.8, 0.8, 0.8), None, 0.3, 0.0),                # Oren-Nayar
    (5, (0.9, 0.9, 0.9), None, 0.3, 0.3),                # Torrance-Sparrow (GGX)
    (5, (0.9, 0.9, 0.9), None, 0.15, 0.15),
    (6, (0.5, 0.5, 0.5), (0.2, 0.2, 0.2), 50.0, 400.0),  # Ashikhmin-Shirley, anisotropic
    (6, (0.5, 0.5, 0.5), (0.2, 0.2, 0.2), 80.0, 80.0),
]


def hemisphere_grid(nt=1024, nphi=2048):
    """Midpoint quadrature nodes and weights of the upper (y > 0) hemisphere."""
    th = (np.arange(nt) + 0.5) * (math.pi / 2) / nt
    ph = (np.arange(nphi) + 0.5) * (2 * math.pi) / nphi
    T, P = np.meshgrid(th, ph, indexing="ij")
    d = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1).reshape(-1, 3)
    w = (np.sin(T) * (math.pi / 2 / nt) * (2 * math.pi / nphi)).reshape(-1)
    return d.astype(np.float32), w


@pytest.mark.parametrize("mat", MATERIALS)
def test_pdf_normalised(oracle_mod, mat):
    """The pdf of every sampler integrates to 1 over the hemisphere (the
    Ashikhmin-Shirley specular half may lose the part reflected below)."""
    wo = np.array([0.3, 0.8, -0.2], dtype=np.float32)
    wo /= np.linalg.norm(wo)
    d, w = hemisphere_grid()
    _, pdf = oracle_mod.bsdf_c_batch(mat[0], mat[1], mat[2], mat[3], mat[4], wo, d)
    integral = float(np.sum(pdf * w))
    lo = 0.9 if mat[0] == 6 else 0.98
    assert lo < integral < 1.02, integral


@pytest.mark.parametrize("mat", MATERIALS)
def test_sampler_matches_pdf(oracle_mod, mat):
    """E_sampler[g(w)] equals the quadrature of g * pdf."""
    wo = np.array([0.3, 0.8, -0.2], dtype=np.float32)
    wo /= np.linalg.norm(wo)
    s = oracle_mod.bsdf_sample_c(mat[0], mat[1], mat[2], mat[3], mat[4], wo, 12345, 200000)
    s = s / np.linalg.norm(s, axis=1, keepdims=True)
    g = lambda v: (v[:, 1] > 0) * (v[:, 0] + 2.0 * v[:, 1] ** 2)
    lhs = float(np.mean(g(s)))
    d, w = hemisphere_grid()
    _, pdf = oracle_mod.bsdf_c_batch(mat[0], mat[1], mat[2], mat[3], mat[4], wo, d)
    rhs = float(np.sum(g(d) * pdf * w))
    assert abs(lhs - rhs) < 0.02, (lhs, rhs)


def test_env_cdf_sampling(oracle_mod, ptgb_mod):
    """Environment sampling: unit directions, pdf > 0, sample mean of g
    equals the quadrature of g * pdf over the sphere."""
    s = ptgb_mod.Scene()
    m = s.lambertian((0.5, 0.5, 0.5))
    s.sphere((0, 0, 0), 1.0, m)
    s.miss_env(ptgb_mod.sky_env(128, 64, sun_peak=200.0, sigma=0.1))
    s.set_camera((0, 0, 5), (0, 0, 0), (0, 1, 0), 40.0, 1.0, 0.0, 1.0)
    o = oracle_mod.Oracle(s)
    rng = np.random.default_rng(3)
    dirs, pdf = o.env_sample(rng.uniform(0, 1, (100000, 2)))
    assert dirs is not None and np.all(pdf > 0)
    assert np.allclose(np.linalg.norm(dirs, axis=1), 1, atol=1e-5)
    g = lambda v: v[:, 1] ** 2 + 0.5 * v[:, 0]
    lhs = float(np.mean(g(dirs)))
    # pdf on a sphere grid through the same sampler: invert via many samples
    hist, xe, ye = np.histogram2d(np.arctan2(dirs[:, 2], dirs[:, 0]), dirs[:, 1], bins=(64, 32),
                                  range=((-math.pi, math.pi), (-1, 1)))
    x = 0.5 * (xe[1:] + xe[:-1])
    y = 0.5 * (ye[1:] + ye[:-1])
    X, Y = np.meshgrid(x, y, indexing="ij")
    R = np.sqrt(1 - Y ** 2)
    grid = np.stack([R * np.cos(X), Y, R * np.sin(X)], -1).reshape(-1, 3)
    rhs = float(np.sum(g(grid) * hist.reshape(-1)) / hist.sum())
    assert abs(lhs - rhs) < 0.02
    # importance: the sky (upper hemisphere) is brighter than the ground
    assert dirs[:, 1].mean() > 0.2


def furnace_scene(ptgb, env_rgba=None, albedo=0.6):
    s = ptgb.Scene()
    m = s.lambertian((albedo, albedo, albedo))
    s.sphere((0, 0, 0), 1.0, m)
    if env_rgba is None:
        s.miss_constant((1.0, 1.0, 1.0))
    else:
        s.miss_env(env_rgba)
    s.set_camera((0, 0, 4), (0, 0, 0), (0, 1, 0), 30.0, 1.0, 0.0, 4.0)
    return s


def test_white_furnace_exact(oracle_mod, ptgb_mod):
    """Lambertian sphere in a uniform white environment: every path that hits
    the sphere carries exactly albedo (f cos / pdf = albedo, one bounce)."""
    s = furnace_scene(ptgb_mod)
    o = oracle_mod.Oracle(s)
    acc, _ = o.render(32, 32, 4, mode=1, rr_enable=0)
    img = acc[..., :3] / 4
    assert np.allclose(img[12:20, 12:20], 0.6, atol=1e-5)   # sphere
    assert np.allclose(img[:3, :3], 1.0, atol=1e-6)         # background


def test_furnace_with_environment_nee(oracle_mod, ptgb_mod):
    """Same furnace lit by a constant HDR map (x2 gain of the miss program):
    NEE through the environment CDF + MIS gives albedo x 1 on average."""
    env = np.full((32, 64, 4), 0.5, dtype=np.float32)
    s = furnace_scene(ptgb_mod, env)
    o = oracle_mod.Oracle(s)
    acc, st = o.render(16, 16, 64, mode=1, rr_enable=0)
    img = acc[..., :3] / 64
    center = img[6:10, 6:10]
    assert st["shadow_rays"] > 0
    assert abs(center.mean() - 0.6) < 0.02
