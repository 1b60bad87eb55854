"""The CPU oracle pinned to the reference's own code.

oracle/_ref/libref.so compiles the reference's device programs (programs/ of
joaovbs96/OptiX-Path-Tracer: raygen.cu, miss.cu, hit.cu, the intersection and
HitRecord programs of hitables/{sphere,aarect,box,triangle}.cu, the
closest-hit programs of materials/*.cu with light_sample.cuh's Direct_Light,
pdfs/{rect,sphere}_pdf.cu, textures/{constant,image,checkered,noise,
gradient}_texture.cu and textures/vector.cu, and the
headers random.cuh, sampling.cuh, math/trigonometric.cuh,
materials/{material,microfacets}.cuh and the BRDF headers) unmodified, over
an OptiX 6 stand-in and a CPU emulation of its runtime (oracle/refhost).
Where OptiX is silent or closed, the stand-in applies the conventions that
the oracle and the CUDA kernels state: the Duff ONB, Malley cosine sampling,
ptmath elementary functions, left-to-right evaluation of several rnd() in
one argument list, zero for uninitialised locals, closest-hit order for
shadow any-hit, a watertight test for RTX-mode triangles.

Every comparison here is bit-exact: the oracle's restatement and the
reference's compiled programs give identical floats, from the RNG streams and
BRDF samples up to whole paths.  The CUDA kernels are in turn checked
against the oracle (tests/test_gpu_parity.py and the others).

These tests need the reference's source tree (the harness is built from it
where it lies); they skip where it is absent.
"""
import numpy as np
import pytest

import refpin

pytestmark = pytest.mark.skipif(not refpin.available(),
                                reason="the reference's source tree is not available")

N = 100_000


def unit(v):
    return (v / np.linalg.norm(v, axis=-1, keepdims=True)).astype(np.float32)


@pytest.fixture(scope="module")
def rng():
    return np.random.default_rng(20261204)


def test_tea_lcg_rnd_streams(rng):
    for a, b in rng.integers(0, 2 ** 32, size=(2000, 2), dtype=np.uint64):
        assert refpin.tea64("ref", int(a), int(b)) == refpin.tea64("or", int(a), int(b))
    for seed in (0, 1, 0xDEADBEEF, 2 ** 32 - 1):
        assert np.array_equal(refpin.lcg_stream("ref", seed, N), refpin.lcg_stream("or", seed, N))
        assert np.array_equal(refpin.rnd_stream("ref", seed, N), refpin.rnd_stream("or", seed, N))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_sampling_helpers(kind):
    """random_in_unit_disk / _in_unit_sphere / _on_unit_sphere."""
    a = refpin.sampling("ref", kind, 12345, N)
    b = refpin.sampling("or", kind, 12345, N)
    assert np.array_equal(a, b)


MATERIALS = [
    ("lambertian", 0, (0.7, 0.6, 0.5), None, 0.0, 0.0),
    ("diffuse_light", 3, (4.0, 4.0, 3.0), None, 0.0, 0.0),
    ("oren_nayar", 4, (0.6, 0.7, 0.6), None, 0.4, 0.0),
    ("oren_nayar_saturated", 4, (0.6, 0.7, 0.6), None, 1.7, 0.0),
    ("torrance_sparrow", 5, (0.9, 0.6, 0.3), None, 0.3, 0.3),
    ("torrance_sparrow_aniso", 5, (0.9, 0.6, 0.3), None, 0.08, 0.45),
    ("torrance_sparrow_min_roughness", 5, (0.9, 0.6, 0.3), None, 0.0, 1e-4),
    ("ashikhmin_shirley_aniso", 6, (0.5, 0.5, 0.7), (0.1, 0.1, 0.1), 50.0, 400.0),
    ("ashikhmin_shirley_iso", 6, (0.7, 0.5, 0.5), (0.2, 0.2, 0.2), 80.0, 80.0),
    ("ashikhmin_shirley_clamped", 6, (0.7, 0.5, 0.5), (0.2, 0.2, 0.2), 0.5, 12.0),
]


@pytest.mark.parametrize("name,mtype,c0,c1,p0,p1", MATERIALS, ids=[m[0] for m in MATERIALS])
def test_brdf_sample_and_evaluate(rng, name, mtype, c0, c1, p0, p1):
    """Sample(surface, P, Wo, N, seed) and Evaluate(surface, P, Wo, Wi, N,
    pdf) of the BRDF headers, with the host classes' parameter conversions
    (materials.hpp:173-174,192-198,227-238), at sampled and at arbitrary
    directions."""
    wo = unit(rng.normal(size=(N, 3)))
    nrm = unit(rng.normal(size=(N, 3)))
    seeds = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32)
    wi_r, s_r = refpin.brdf_sample("ref", mtype, c0, c1, p0, p1, wo, nrm, seeds)
    wi_o, s_o = refpin.brdf_sample("or", mtype, c0, c1, p0, p1, wo, nrm, seeds)
    assert np.array_equal(s_r, s_o), "random numbers drawn differ"
    assert np.array_equal(wi_r, wi_o, equal_nan=True)
    for wi in (wi_r, unit(rng.normal(size=(N, 3)))):
        f_r, pdf_r = refpin.brdf_eval("ref", mtype, c0, c1, p0, p1, wo, wi, nrm)
        f_o, pdf_o = refpin.brdf_eval("or", mtype, c0, c1, p0, p1, wo, wi, nrm)
        assert np.array_equal(f_r, f_o, equal_nan=True)
        assert np.array_equal(pdf_r, pdf_o, equal_nan=True)


def helper_inputs(rng, fn):
    a = np.zeros((N, 8), np.float32)
    if fn == 0:      # schlick(cosine, ref_idx)
        a[:, 0] = rng.uniform(-1, 1, N)
        a[:, 1] = rng.uniform(1.0, 2.5, N)
    elif fn == 1:    # Refract(v, n, ni_over_nt): includes total internal reflection
        a[:, 0:3] = rng.normal(size=(N, 3))
        a[:, 3:6] = unit(rng.normal(size=(N, 3)))
        a[:, 6] = rng.uniform(0.3, 2.0, N)
    elif fn == 2:    # GGX_Sample(origin, (rx, ry), nu, nv): includes normal incidence
        o = unit(rng.normal(size=(N, 3)))
        o[: N // 20] = unit(np.array([1e-3, 1.0, -2e-3]) + 1e-4 * rng.normal(size=(N // 20, 3)))
        a[:, 0:3] = o
        a[:, 3:5] = rng.uniform(0, 1, (N, 2))
        a[:, 5] = rng.uniform(1e-3, 0.5, N) ** 2
        a[:, 6] = np.where(rng.uniform(size=N) < 0.5, a[:, 5], rng.uniform(1e-3, 0.5, N) ** 2)
    elif fn == 3:    # GGX_D, GGX_G, GGX_PDF
        a[:, 0:3] = unit(rng.normal(size=(N, 3)))
        a[:, 3:6] = unit(rng.normal(size=(N, 3)))
        a[:, 6] = rng.uniform(1e-3, 0.5, N) ** 2
        a[:, 7] = np.where(rng.uniform(size=N) < 0.5, a[:, 6], rng.uniform(1e-3, 0.5, N) ** 2)
    elif fn == 4:    # Sample_Quadrant(nu, nv, rx, ry)
        a[:, 0:2] = rng.uniform(1, 1000, (N, 2))
        a[:, 2:4] = rng.uniform(0, 1, (N, 2))
    else:            # AbsCosTheta, SinTheta, CosPhi, SinPhi (abs(float) must stay a float)
        a[:, 0:3] = unit(rng.normal(size=(N, 3)))
    return a


@pytest.mark.parametrize("fn", [0, 1, 2, 3, 4, 5],
                         ids=["schlick", "refract", "ggx_sample", "ggx_d_g_pdf",
                              "sample_quadrant", "trigonometric"])
def test_material_helpers(rng, fn):
    a = helper_inputs(rng, fn)
    r = refpin.helper("ref", fn, a)
    o = refpin.helper("or", fn, a)
    assert np.array_equal(r, o, equal_nan=True)
    if fn == 5:
        assert np.array_equal(r[:, 0], np.abs(a[:, 1]))   # AbsCosTheta of a negative y


def light_scene(ptgb):
    s = ptgb.Scene()
    m = s.lambertian((0.5, 0.5, 0.5))
    s.sphere((0.0, -100.0, 0.0), 99.0, m)
    s.light_rect(-1.0, 1.0, -0.5, 0.5, 3.0, ptgb.PT_X_AXIS, (5.0, 5.0, 5.0))
    s.light_rect(-1.0, 1.0, -0.5, 0.5, 2.5, ptgb.PT_Y_AXIS, (5.0, 4.0, 3.0))
    s.light_rect(-1.0, 1.0, -0.5, 0.5, -2.0, ptgb.PT_Z_AXIS, (1.0, 2.0, 3.0))
    s.light_sphere((0.5, 1.5, 0.2), 0.3, (6.0, 6.0, 6.0))
    s.miss_constant((0.0, 0.0, 0.0))
    s.set_camera((0.0, 1.0, 4.0), (0.0, 0.0, 0.0), (0, 1, 0), 45.0, 1.0, 0.0, 4.0)
    return s


@pytest.mark.parametrize("k", [0, 1, 2, 3], ids=["rect_x", "rect_y", "rect_z", "sphere"])
def test_light_sample_and_pdf(rng, ptgb_mod, oracle_mod, k):
    """rect_pdf.cu Sample_X/Y/Z + PDF_X/Y/Z, sphere_pdf.cu Sample + PDF."""
    s = light_scene(ptgb_mod)
    R, O = refpin.RefPrograms(s), oracle_mod.Oracle(s)
    P = rng.uniform(-1.5, 1.5, (20000, 3)).astype(np.float32)
    seeds = rng.integers(0, 2 ** 32, len(P), dtype=np.uint64).astype(np.uint32)
    wr, pr, sr = R.light(k, P, seeds)
    wo, po, so = refpin.oracle_light(O, k, P, seeds)
    assert np.array_equal(sr, so)
    assert np.array_equal(wr, wo, equal_nan=True)     # NaN where P is inside a sphere light
    assert np.array_equal(pr, po, equal_nan=True)
    if k < 3:
        assert (pr > 0).mean() > 0.5
    else:
        # sphere_pdf.cu:70-71 builds the sampling frame around the sample
        # itself rather than the direction to the sphere, so most samples
        # miss it and their pdf is 0: reproduced on both sides
        assert 0 < (pr > 0).sum() < len(pr) // 2


def single_prim_scenes(ptgb):
    P = ptgb
    out = {}

    def base():
        s = P.Scene()
        s.miss_constant((0.0, 0.0, 0.0))
        s.set_camera((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), (0, 1, 0), 40.0, 1.0, 0.0, 5.0)
        return s

    s = base()
    s.sphere((0.2, -0.1, 0.3), 0.8, s.lambertian((1, 1, 1)))
    out["sphere"] = s
    for ax in (0, 1, 2):
        for flip in (False, True):
            s = base()
            s.rect(-0.7, 0.9, -0.4, 0.6, 0.25, flip, ax, s.lambertian((1, 1, 1)))
            out[f"rect_{'xyz'[ax]}_{int(flip)}"] = s
    s = base()
    s.box((-0.5, -0.3, -0.6), (0.4, 0.7, 0.2), s.lambertian((1, 1, 1)))
    out["box"] = s
    xf = P.compose([P.mat_translate((0.3, -0.2, 0.1)), P.mat_rotate(-18.0, P.PT_Y_AXIS),
                    P.mat_rotate(25.0, P.PT_X_AXIS)])
    s = base()
    s.box((-0.5, -0.3, -0.6), (0.4, 0.7, 0.2), s.lambertian((1, 1, 1)), xf)
    out["box_transformed"] = s
    s = base()
    s.rect(-0.7, 0.9, -0.4, 0.6, 0.25, True, P.PT_Y_AXIS, s.lambertian((1, 1, 1)), xf)
    out["rect_transformed"] = s
    s = base()
    verts, idx, nrm, uvs, _ = P.heightfield_mesh(6, 0.2, seed=5, extent=1.5)
    s.mesh(verts, idx, s.lambertian((1, 1, 1)), normals=nrm, uvs=uvs)
    out["mesh"] = s
    return out


@pytest.mark.parametrize("name", ["sphere", "rect_x_0", "rect_x_1", "rect_y_0", "rect_y_1",
                                  "rect_z_0", "rect_z_1", "box", "box_transformed",
                                  "rect_transformed", "mesh"])
def test_intersection_and_hitrecord(rng, ptgb_mod, oracle_mod, name):
    """Intersection programs (both sphere roots, rect axes and flips, the box
    slabs and its float-equality normals, transformed instances, RTX-mode
    triangles through the Attributes program) and Get_HitRecord on random
    rays from outside and inside: same primitive, t, P, normals, uv, Wo."""
    s = single_prim_scenes(ptgb_mod)[name]
    R, O = refpin.RefPrograms(s), oracle_mod.Oracle(s)
    hits = 0
    for _ in range(4000):
        o = rng.uniform(-2.5, 2.5, 3).astype(np.float32)
        if rng.uniform() < 0.3:
            o = (o * 0.15).astype(np.float32)            # starts inside or near the shape
        target = rng.uniform(-0.8, 0.8, 3).astype(np.float32)
        d = (target - o).astype(np.float32)
        if rng.uniform() < 0.5:
            d = (d * rng.uniform(0.1, 10.0)).astype(np.float32)  # unnormalised directions
        pr, tr, rr = R.probe(o, d)
        po, to, ro = refpin.oracle_probe(O, o, d)
        assert pr == po, (o, d)
        if pr >= 0:
            hits += 1
            assert tr == to
            # P, shading normal, u, v, geometric normal
            assert np.array_equal(rr[:11], ro[:11]), (name, o, d, rr, ro)
            if name.endswith("_transformed"):
                # Wo: the reference's HitRecord programs take it from the ray
                # they are given, which OptiX hands over in the primitive's
                # object space; the oracle and the kernels use the world-space
                # view direction.  (No pinned scene puts a Wo-dependent
                # material on a transformed primitive.)
                assert np.allclose(ro[11:14], -d / np.linalg.norm(d), atol=1e-6)
            else:
                assert np.array_equal(rr[11:14], ro[11:14])
    assert hits > 400


def test_moving_sphere_program(rng, oracle_mod):
    """programs/hitables/moving_sphere.cu (compiled over the stand-in, its
    time taken from the ray's payload) against the oracle's moving sphere on
    random rays at random times, also outside [time0, time1] (the centre is
    extrapolated): the same hit, t, P, shading normal, u, v and Wo; and its
    get_bounds box lies inside the oracle's box (which also covers the
    camera's times)."""
    hits = 0
    for _ in range(4000):
        c0 = rng.uniform(-1, 1, 3).astype(np.float32)
        c1 = (c0 + rng.uniform(-0.8, 0.8, 3)).astype(np.float32)
        r = np.float32(rng.uniform(0.2, 0.9))
        t0 = np.float32(rng.uniform(-0.5, 0.5))
        t1 = np.float32(t0 + rng.uniform(0.1, 2.0))
        f9 = np.array(list(c0) + [r, t0, t1] + list(c1), np.float32)
        time = np.float32(rng.uniform(t0 - 0.5, t1 + 0.5))
        o = rng.uniform(-3, 3, 3).astype(np.float32)
        d = (rng.uniform(-0.8, 0.8, 3) - o).astype(np.float32)
        if rng.uniform() < 0.5:
            d = (d * rng.uniform(0.1, 10.0)).astype(np.float32)
        tmin = np.float32(1e-3 if rng.uniform() < 0.5 else 1e-6)
        hr, outr, boxr = refpin.msphere(f9, o, d, tmin, np.float32(1e20), time)
        ho, outo, boxo = oracle_mod.msphere(f9, o, d, tmin, np.float32(1e20), time, t0, t1)
        assert hr == ho, (f9, o, d, time)
        if hr:
            hits += 1
            assert np.array_equal(outr, outo), (f9, o, d, time, outr, outo)
        assert np.all(boxo[:3] <= boxr[:3]) and np.all(boxo[3:] >= boxr[3:])
    assert hits > 500


def test_software_triangle_program_against_watertight(rng, ptgb_mod):
    """The reference's non-RTX triangle program (triangle.cu:26-58,
    Moller-Trumbore without a watertight guarantee) against the watertight
    test that stands in for the RTX hardware test: they agree on hit or
    miss except for rays within float rounding of an edge, and on t to a
    few ulps where both hit."""
    s = ptgb_mod.Scene()
    verts, idx, nrm, uvs, _ = ptgb_mod.heightfield_mesh(4, 0.2, seed=6, extent=1.5)
    s.mesh(verts, idx, s.lambertian((1, 1, 1)))
    s.miss_constant((0.0, 0.0, 0.0))
    s.set_camera((0.0, 2.0, 0.0), (0.0, 0.0, 0.0), (0, 0, 1), 40.0, 1.0, 0.0, 2.0)
    R = refpin.RefPrograms(s)
    agree, both, rel = 0, 0, []
    n = 20000
    for _ in range(n):
        o = np.array([rng.uniform(-1.4, 1.4), 1.5, rng.uniform(-1.4, 1.4)], np.float32)
        d = np.array([rng.uniform(-0.3, 0.3), -1.0, rng.uniform(-0.3, 0.3)], np.float32)
        pr, tr, _ = R.probe(o, d)                 # RTX path: watertight + Attributes
        sw = R.triangle_sw(pr, o, d) if pr >= 0 else None
        if pr >= 0 and sw is not None:
            both += 1
            agree += 1
            rel.append(abs(sw[0] - tr) / tr)
        elif pr < 0:
            agree += 1
    assert agree / n > 0.999
    assert both > n // 2
    assert max(rel) < 1e-5


def full_scenes(ptgb):
    P = ptgb
    env = P.sky_env(64, 32)
    zoo_cyl = P.material_zoo(40, 30)
    zoo_cyl.miss_env(env, spherical=False)
    zoo_img = P.material_zoo(40, 30)
    zoo_img.miss_env(env, kind=P.MISS_IMG)
    zoo_const = P.material_zoo(40, 30)
    zoo_const.miss_constant((0.3, 0.4, 0.5))
    return {
        "cornell_reference": (P.cornell_reference(40, 40), 40, 40),
        "cornell_c1": (P.cornell_c1(40, 40), 40, 40),
        "spheres": (P.random_spheres(64, 36), 64, 36),
        "zoo": (P.material_zoo(40, 30), 40, 30),
        "zoo_env_cylindrical": (zoo_cyl, 40, 30),
        "zoo_env_image": (zoo_img, 40, 30),
        "zoo_constant": (zoo_const, 40, 30),
        "heightfield_env": (P.heightfield_scene(48, 27, cells=10, env_w=64, env_h=32), 48, 27),
        "textures": (P.texture_zoo(64, 48), 64, 48),
    }


@pytest.mark.parametrize("name", ["cornell_reference", "cornell_c1", "spheres", "zoo",
                                  "zoo_env_cylindrical", "zoo_env_image", "zoo_constant",
                                  "heightfield_env", "textures"])
def test_whole_paths(ptgb_mod, oracle_mod, name):
    """renderPixel of raygen.cu, with every program it reaches, gives the
    oracle's first hits and per-path radiance bit for bit (reference mode,
    Russian roulette after depth 10 as raygen.cu:112 hard-codes)."""
    s, w, h = full_scenes(ptgb_mod)[name]
    R, O = refpin.RefPrograms(s), oracle_mod.Oracle(s)
    for frame in (0, 3):
        rp, rm, rt = R.first_hits(w, h, frame)
        op, om, ot = O.first_hits(w, h, frame)
        assert np.array_equal(rp, op) and np.array_equal(rm, om)
        assert np.array_equal(rt, ot)
        pix = np.arange(w * h)
        r = R.render_paths(w, h, frame, pix)
        o = O.render_paths(w, h, frame, pix)
        assert np.array_equal(r, o, equal_nan=True), (
            f"{np.sum(~np.all(r == o, axis=1))} of {len(pix)} paths differ")
    assert R.stats()["ext_rays"] > 2 * w * h
