"""Python harness over libpt.so (the C ABI of include/pt.h).

Used by the tests and the benchmark.  It mirrors the reference's host scene
API (host_includes/): a ``Scene`` records materials, primitives, lights, the
miss program and the camera in call order and replays them into a GPU
context (``GpuRenderer``) - or, in tests, into the CPU oracle.  Scene
generators for the benchmark configurations live here too.

The GPU path is the only compute path in this module: if libpt.so cannot be
loaded, ``load_library`` raises.
"""
import ctypes
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# PT_LIB overrides the library path (A/B builds of the same sources)
LIB_PATH = os.environ.get("PT_LIB") or os.path.join(HERE, "libpt.so")

PT_X_AXIS, PT_Y_AXIS, PT_Z_AXIS = 0, 1, 2
MISS_GRADIENT, MISS_CONSTANT, MISS_HDR, MISS_IMG = 0, 1, 2, 3
MAT_LAMBERTIAN, MAT_METAL, MAT_DIELECTRIC, MAT_DIFFUSE_LIGHT = 0, 1, 2, 3
MAT_OREN_NAYAR, MAT_TORRANCE_SPARROW, MAT_ASHIKHMIN_SHIRLEY = 4, 5, 6
PRIM_TRIANGLE, PRIM_SPHERE, PRIM_RECT, PRIM_BOX = 0, 1, 2, 3
TEX_CONSTANT, TEX_CHECKER, TEX_NOISE, TEX_IMAGE, TEX_GRADIENT, TEX_VECTOR = 0, 1, 2, 3, 4, 5
NO_HIT = 0xFFFFFFFF

STATUS = {0: "PT_OK", -1: "PT_EINVAL", -2: "PT_ENOMEM", -3: "PT_ECUDA", -4: "PT_ETIMEOUT",
          -5: "PT_EQUEUE", -6: "PT_ESTATE"}


class PtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Options(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("path_slots", ctypes.c_int),
                ("enable_counters", ctypes.c_int), ("enable_timing", ctypes.c_int),
                ("bvh_builder", ctypes.c_int), ("bvh_width", ctypes.c_int),
                ("shade_order", ctypes.c_int), ("refetch_lanes", ctypes.c_int)]


class RenderParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in
                ("width", "height", "spp", "frame0", "max_depth", "rr_enable", "rr_depth",
                 "mode", "guide")]


class Stats(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_uint64), ("ext_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("node_fetches", ctypes.c_uint64),
                ("prim_tests", ctypes.c_uint64), ("bvh_nodes", ctypes.c_uint64),
                ("bvh_bytes", ctypes.c_uint64), ("bvh_depth", ctypes.c_int),
                ("build_ms", ctypes.c_double), ("render_ms", ctypes.c_double),
                ("iterations", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("stage_ms", ctypes.c_double * 5), ("graph_launches", ctypes.c_uint64),
                ("guide_samples", ctypes.c_uint64), ("upload_bytes", ctypes.c_uint64)]


class BatchItem(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("params", RenderParams),
                ("accum_rgba", ctypes.c_void_p)]


class Tune(ctypes.Structure):
    _fields_ = [("path_slots", ctypes.c_int), ("trace_block", ctypes.c_int),
                ("shade_block", ctypes.c_int), ("bvh_width", ctypes.c_int),
                ("chunk_paths", ctypes.c_int), ("shade_order", ctypes.c_int),
                ("refetch_lanes", ctypes.c_int), ("sample_paths_per_s", ctypes.c_double)]


_F3 = ctypes.c_float * 3
_F12 = ctypes.c_float * 12
_P = ctypes.c_void_p
_U32P = ctypes.POINTER(ctypes.c_uint32)

# name -> argtypes (all return int status except where noted)
SIGNATURES = {
    "pt_context_create": [ctypes.POINTER(Options), ctypes.POINTER(_P)],
    "pt_context_destroy": [_P],
    "pt_material_lambertian": [_P, _F3, _U32P],
    "pt_material_metal": [_P, _F3, ctypes.c_float, _U32P],
    "pt_material_dielectric": [_P, _F3, _F3, ctypes.c_float, ctypes.c_float, _U32P],
    "pt_material_diffuse_light": [_P, _F3, _U32P],
    "pt_material_oren_nayar": [_P, _F3, ctypes.c_float, _U32P],
    "pt_material_torrance_sparrow": [_P, _F3, ctypes.c_float, ctypes.c_float, _U32P],
    "pt_material_ashikhmin_shirley": [_P, _F3, _F3, ctypes.c_float, ctypes.c_float, _U32P],
    "pt_texture_constant": [_P, _F3, _U32P],
    "pt_texture_checker": [_P, ctypes.c_uint32, ctypes.c_uint32, _U32P],
    "pt_texture_noise": [_P, ctypes.c_float, ctypes.c_int, _P, _P, _U32P],
    "pt_noise_tables": [_P, _P],
    "pt_texture_image": [_P, _P, ctypes.c_int, ctypes.c_int, _U32P],
    "pt_texture_gradient": [_P, _F3, _F3, _F3, _U32P],
    "pt_texture_vector": [_P, _P, ctypes.c_int, _U32P],
    "pt_material_set_texture": [_P, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32],
    "pt_mesh_set_texture_index": [_P, ctypes.c_uint32, ctypes.c_size_t, _P],
    "pt_add_sphere": [_P, _F3, ctypes.c_float, ctypes.c_uint32, _P, _U32P],
    "pt_add_moving_sphere": [_P, _F3, _F3, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_uint32, _P, _U32P],
    "pt_add_rect": [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                    ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, _P, _U32P],
    "pt_add_box": [_P, _F3, _F3, ctypes.c_uint32, _P, _U32P],
    "pt_add_mesh": [_P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P, ctypes.c_uint32, _P, _P,
                    _P, _U32P],
    "pt_obj_load": [ctypes.c_char_p, ctypes.POINTER(_P)],
    "pt_obj_free": [_P],
    "pt_obj_info": [_P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t),
                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "pt_obj_get": [_P, _P, _P, _P, _P],
    "pt_obj_material": [_P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t, _P, _P,
                        ctypes.c_char_p, ctypes.c_size_t],
    "pt_add_obj": [_P, _P, ctypes.c_uint32, _P, _U32P],
    "pt_hdr_load": [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _P],
    "pt_image_load": [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                      _P],
    "pt_hdr_save": [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int],
    "pt_png_save": [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int],
    "pt_add_light_rect": [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, ctypes.c_int, _F3],
    "pt_add_light_sphere": [_P, _F3, ctypes.c_float, _F3],
    "pt_set_env_gradient": [_P, _F3, _F3],
    "pt_set_env_constant": [_P, _F3],
    "pt_set_env_map": [_P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "pt_set_camera": [_P, _F3, _F3, _F3, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                      ctypes.c_float, ctypes.c_float, ctypes.c_float],
    "pt_commit": [_P],
    "pt_render": [_P, ctypes.POINTER(RenderParams), _P, _P],
    "pt_render_paths": [_P, ctypes.POINTER(RenderParams), _P, _P],
    "pt_render_accum64": [_P, ctypes.POINTER(RenderParams), _P, _P],
    "pt_trace_first_hits": [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P, _P],
    "pt_resolve_display": [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P],
    "pt_get_stats": [_P, ctypes.POINTER(Stats)],
    "pt_render_noalloc": [_P, ctypes.POINTER(RenderParams), _P, _P],
    "pt_guide_init": [_P, ctypes.c_uint64],
    "pt_guide_set_training": [_P, ctypes.c_float, ctypes.c_int, ctypes.c_float, ctypes.c_int],
    "pt_guide_set_wait_limit": [_P, ctypes.c_uint32],
    "pt_guide_get_params": [_P, _P],
    "pt_guide_set_params": [_P, _P],
    "pt_guide_get_state": [_P, _P, ctypes.POINTER(ctypes.c_int64)],
    "pt_guide_set_state": [_P, _P, ctypes.c_int64],
    "pt_guide_bounds": [_P, _P, _P],
    "pt_guide_eval": [_P, _P, ctypes.c_int, _P],
    "pt_guide_gradient": [_P, _P, ctypes.c_int, _P, _P],
    "pt_guide_train": [_P, _P, ctypes.c_int, ctypes.c_float, _P],
    "pt_batch_create": [ctypes.POINTER(Options), ctypes.POINTER(_P)],
    "pt_batch_destroy": [_P],
    "pt_batch_render": [_P, ctypes.POINTER(BatchItem), ctypes.c_int, _P],
    "pt_batch_autotune": [_P, ctypes.POINTER(BatchItem), ctypes.c_int, ctypes.POINTER(Tune)],
    "pt_batch_set_tune": [_P, ctypes.POINTER(Tune)],
    "pt_batch_get_tune": [_P, ctypes.POINTER(Tune)],
    "pt_batch_get_stats": [_P, ctypes.POINTER(Stats)],
}

_lib = None


def load_library(path=LIB_PATH):
    """Loads libpt.so and declares every entry point; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.pt_last_error.argtypes = [_P]
    lib.pt_last_error.restype = ctypes.c_char_p
    lib.pt_version.argtypes = []
    lib.pt_version.restype = ctypes.c_char_p
    lib.pt_batch_last_error.argtypes = [_P]
    lib.pt_batch_last_error.restype = ctypes.c_char_p
    lib.pt_io_last_error.argtypes = []
    lib.pt_io_last_error.restype = ctypes.c_char_p
    lib.pt_image_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def f3(v):
    return _F3(*[float(x) for x in v])


# ----------------------------------------------------------- file formats
PT_OBJ_NO_MATERIAL = 0xFFFFFFFF
PT_OBJ_MTL = 0xFFFFFFFE


def _io_check(lib, rc):
    if rc != 0:
        raise PtError(rc, lib.pt_io_last_error().decode())


class ObjMesh:
    """A Wavefront OBJ file read by pt_obj_load (de-indexed triangles)."""

    def __init__(self, path):
        self.lib = load_library()
        h = _P()
        _io_check(self.lib, self.lib.pt_obj_load(str(path).encode(), ctypes.byref(h)))
        self.h = h
        self.dir = os.path.dirname(os.path.abspath(str(path)))
        nt, nm = ctypes.c_size_t(), ctypes.c_size_t()
        hn, hu = ctypes.c_int(), ctypes.c_int()
        _io_check(self.lib, self.lib.pt_obj_info(h, ctypes.byref(nt), ctypes.byref(nm),
                                                 ctypes.byref(hn), ctypes.byref(hu)))
        self.n_tris, self.n_materials = nt.value, nm.value
        self.verts = np.zeros((self.n_tris, 3, 3), np.float32)
        self.normals = np.zeros((self.n_tris, 3, 3), np.float32) if hn.value else None
        self.uvs = np.zeros((self.n_tris, 3, 2), np.float32) if hu.value else None
        self.mat = np.zeros(self.n_tris, np.uint32)
        _io_check(self.lib, self.lib.pt_obj_get(h, _ptr(self.verts), _ptr(self.normals),
                                                _ptr(self.uvs), _ptr(self.mat)))

    def material(self, k):
        name = ctypes.create_string_buffer(256)
        tex = ctypes.create_string_buffer(256)
        ka = np.zeros(3, np.float32)
        kd = np.zeros(3, np.float32)
        _io_check(self.lib, self.lib.pt_obj_material(self.h, k, name, 256, _ptr(ka), _ptr(kd),
                                                     tex, 256))
        return {"name": name.value.decode(), "Ka": ka, "Kd": kd, "map_Kd": tex.value.decode()}

    def close(self):
        if self.h:
            self.lib.pt_obj_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def image_load(path):
    """An image file read by pt_image_load (PNG, PPM, Radiance HDR): HxWx4
    float32, first file row first."""
    lib = load_library()
    w, h = ctypes.c_int(), ctypes.c_int()
    rc = lib.pt_image_load(str(path).encode(), ctypes.byref(w), ctypes.byref(h), None)
    if rc != 0:
        raise PtError(rc, lib.pt_image_last_error().decode())
    out = np.zeros((h.value, w.value, 4), np.float32)
    rc = lib.pt_image_load(str(path).encode(), ctypes.byref(w), ctypes.byref(h), _ptr(out))
    if rc != 0:
        raise PtError(rc, lib.pt_image_last_error().decode())
    return out


def hdr_load(path):
    """A Radiance HDR file as an HxWx4 float32 array (pt_hdr_load)."""
    lib = load_library()
    w, h = ctypes.c_int(), ctypes.c_int()
    _io_check(lib, lib.pt_hdr_load(str(path).encode(), ctypes.byref(w), ctypes.byref(h), None))
    out = np.zeros((h.value, w.value, 4), np.float32)
    _io_check(lib, lib.pt_hdr_load(str(path).encode(), ctypes.byref(w), ctypes.byref(h), _ptr(out)))
    return out


def hdr_save(path, accum, spp):
    """Save_HDR of an HxWx4 float32 accumulation (pt_hdr_save)."""
    lib = load_library()
    a = np.ascontiguousarray(accum, np.float32)
    _io_check(lib, lib.pt_hdr_save(str(path).encode(), a.shape[1], a.shape[0], _ptr(a), int(spp)))


def png_save(path, accum, spp):
    """Save_PNG of an HxWx4 float32 accumulation (pt_png_save)."""
    lib = load_library()
    a = np.ascontiguousarray(accum, np.float32)
    _io_check(lib, lib.pt_png_save(str(path).encode(), a.shape[1], a.shape[0], _ptr(a), int(spp)))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


# ----------------------------------------------------------------- transforms
def mat_identity():
    return np.eye(4)


def mat_translate(v):
    m = np.eye(4)
    m[:3, 3] = v
    return m


def mat_rotate(angle_deg, axis):
    """Right-handed rotation about a coordinate axis (Matrix4x4::rotate of
    host_includes/transforms.hpp:126 with an axis unit vector)."""
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4)
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    m[i, i] = c
    m[i, j] = -s
    m[j, i] = s
    m[j, j] = c
    return m


def mat_scale(v):
    m = np.eye(4)
    m[0, 0], m[1, 1], m[2, 2] = v
    return m


def compose(ops, reverse=False):
    """World matrix of a transform list.  Hitable_List::addElementsTo applies
    the last-called transform innermost (host_includes/hitables.hpp:518-523,
    transforms.hpp:299-329); Hitable::addTo reverses the list first
    (hitables.hpp:61-70).  Returns 12 float32 (row-major 3x4) or None."""
    if not ops:
        return None
    seq = list(reversed(ops)) if reverse else list(ops)
    m = np.eye(4)
    for op in seq:
        m = m @ op
    return np.ascontiguousarray(m[:3, :4], dtype=np.float32).reshape(12)


# --------------------------------------------------------------------- scene
class Scene:
    """Call-order record of the reference's scene construction API."""

    def __init__(self):
        self.materials = []   # (kind, c0, c1, p0, p1)
        self.textures = []    # (kind, a, b, c[9], data, perm, ids)
        self.mat_textures = []  # (material, slot, texture) in call order
        self.tex_index = {}   # mesh item index -> per-face texture index (uint32)
        self.items = []       # ("sphere"|"msphere"|"rect"|"box"|"mesh", args...)
        self.add_obj = {}     # item index -> (ObjMesh, material or None): load with pt_add_obj
        self.lights = []      # ("rect"|"sphere", args..., emission)
        self.miss = ("constant", (0.0, 0.0, 0.0))
        self.camera = None
        self.n_prims = 0

    # materials (host_includes/materials.hpp)
    def lambertian(self, albedo):
        self.materials.append((MAT_LAMBERTIAN, tuple(albedo), None, 0.0, 0.0))
        return len(self.materials) - 1

    def metal(self, albedo, fuzz):
        self.materials.append((MAT_METAL, tuple(albedo), None, float(fuzz), 0.0))
        return len(self.materials) - 1

    def dielectric(self, base, extinction, ref_idx, density=0.0):
        self.materials.append((MAT_DIELECTRIC, tuple(base), tuple(extinction), float(ref_idx),
                               float(density)))
        return len(self.materials) - 1

    def diffuse_light(self, emission):
        self.materials.append((MAT_DIFFUSE_LIGHT, tuple(emission), None, 0.0, 0.0))
        return len(self.materials) - 1

    def oren_nayar(self, albedo, roughness):
        self.materials.append((MAT_OREN_NAYAR, tuple(albedo), None, float(roughness), 0.0))
        return len(self.materials) - 1

    def torrance_sparrow(self, color, nu, nv):
        self.materials.append((MAT_TORRANCE_SPARROW, tuple(color), None, float(nu), float(nv)))
        return len(self.materials) - 1

    def ashikhmin_shirley(self, diffuse, specular, nu, nv):
        self.materials.append((MAT_ASHIKHMIN_SHIRLEY, tuple(diffuse), tuple(specular), float(nu),
                               float(nv)))
        return len(self.materials) - 1

    # textures (host_includes/textures.hpp)
    def _texture(self, kind, a=0, b=0, c=(), data=None, perm=None, ids=None):
        cc = np.zeros(9, np.float32)
        cc[:len(c)] = c
        self.textures.append((kind, int(a), int(b), cc, data, perm, ids))
        return len(self.textures) - 1

    def texture_constant(self, rgb):
        return self._texture(TEX_CONSTANT, c=tuple(rgb))

    def texture_checker(self, odd, even):
        return self._texture(TEX_CHECKER, odd, even)

    def texture_noise(self, scale, axis=PT_X_AXIS, ranvec=None, perm=None):
        """Perlin noise; null tables are the library's defaults (those the
        reference's host class makes with std::mt19937 seeded 0)."""
        if ranvec is None or perm is None:
            r0, p0 = noise_tables()
            ranvec = r0 if ranvec is None else ranvec
            perm = p0 if perm is None else perm
        ranvec = np.ascontiguousarray(ranvec, np.float32).reshape(768)
        perm = np.ascontiguousarray(perm, np.int32).reshape(768)
        return self._texture(TEX_NOISE, axis, 0, (float(scale),), ranvec, perm)

    def texture_image(self, rgba):
        rgba = np.ascontiguousarray(rgba, np.float32)
        assert rgba.ndim == 3 and rgba.shape[2] == 4
        return self._texture(TEX_IMAGE, rgba.shape[1], rgba.shape[0], data=rgba)

    def texture_gradient(self, a, b, c):
        return self._texture(TEX_GRADIENT, c=tuple(a) + tuple(b) + tuple(c))

    def texture_vector(self, ids):
        ids = np.ascontiguousarray(ids, np.uint32)
        return self._texture(TEX_VECTOR, 0, len(ids), ids=ids)

    def set_texture(self, material, slot, texture):
        self.mat_textures.append((int(material), int(slot), int(texture)))

    # geometry (host_includes/hitables.hpp, mesh.hpp)
    def sphere(self, center, radius, mat, xform=None):
        self.items.append(("sphere", tuple(center), float(radius), mat, xform))
        self.n_prims += 1
        return self.n_prims - 1

    def moving_sphere(self, center0, center1, radius, time0, time1, mat, xform=None):
        """Moving_Sphere (hitables.hpp:130-181): centre center0 at time0,
        center1 at time1, linear in the path's time."""
        self.items.append(("msphere", tuple(center0), tuple(center1), float(radius), float(time0),
                           float(time1), mat, xform))
        self.n_prims += 1
        return self.n_prims - 1

    def rect(self, a0, a1, b0, b1, k, flip, axis, mat, xform=None):
        self.items.append(("rect", (a0, a1, b0, b1, k), int(flip), int(axis), mat, xform))
        self.n_prims += 1
        return self.n_prims - 1

    def box(self, p0, p1, mat, xform=None):
        self.items.append(("box", tuple(p0), tuple(p1), mat, xform))
        self.n_prims += 1
        return self.n_prims - 1

    def mesh(self, verts, idx, mat, mat_per_tri=None, normals=None, uvs=None, xform=None,
             tex_index=None):
        verts = np.ascontiguousarray(verts, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1, 3)
        if mat_per_tri is not None:
            mat_per_tri = np.ascontiguousarray(mat_per_tri, dtype=np.uint32)
        if normals is not None:
            normals = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        if uvs is not None:
            uvs = np.ascontiguousarray(uvs, dtype=np.float32).reshape(-1, 2)
        self.items.append(("mesh", verts, idx, mat, mat_per_tri, normals, uvs, xform))
        if tex_index is not None:
            self.tex_index[len(self.items) - 1] = np.ascontiguousarray(tex_index, np.uint32)
        first = self.n_prims
        self.n_prims += len(idx)
        return first

    def obj(self, mesh, material=None, xform=None, via_add_obj=False):
        """An ObjMesh as the reference's Mesh adds it (mesh.hpp:78-98):
        `material` on every face, or (None) one Lambertian coloured by a
        vector texture of the MTL materials (an image texture of map_Kd,
        rows flipped as Image_Texture stores them, else a constant Ka), each
        face indexing its material (faces without usemtl: the first); a grey
        Lambertian without an MTL file.  via_add_obj: the GPU renderer loads
        it through pt_add_obj instead of pt_add_mesh (the oracle always sees
        the triangle arrays)."""
        nt = mesh.n_tris
        mat = material
        tex_index = None
        if material is None and mesh.n_materials == 0:
            mat = self.lambertian((0.5, 0.5, 0.5))
        elif material is None:
            texs = []
            for k in range(mesh.n_materials):
                info = mesh.material(k)
                if info["map_Kd"]:
                    img = image_load(os.path.join(mesh.dir, info["map_Kd"]))
                    texs.append(self.texture_image(img[::-1]))
                else:
                    texs.append(self.texture_constant(tuple(info["Ka"])))
            vec = self.texture_vector(texs)
            mat = self.lambertian((0.0, 0.0, 0.0))
            self.set_texture(mat, 0, vec)
            tex_index = np.where(mesh.mat == PT_OBJ_NO_MATERIAL, 0, mesh.mat).astype(np.uint32)
        first = self.mesh(mesh.verts.reshape(-1, 3), np.arange(3 * nt, dtype=np.uint32).reshape(-1, 3),
                          mat, None, None if mesh.normals is None else mesh.normals.reshape(-1, 3),
                          None if mesh.uvs is None else mesh.uvs.reshape(-1, 2), xform,
                          tex_index=tex_index)
        if via_add_obj:
            self.add_obj[len(self.items) - 1] = (mesh, material)
        return first

    # lights (host_includes/pdfs.hpp)
    def light_rect(self, a0, a1, b0, b1, k, axis, emission):
        self.lights.append(("rect", (a0, a1, b0, b1, k), int(axis), tuple(emission)))

    def light_sphere(self, center, radius, emission):
        self.lights.append(("sphere", tuple(center), float(radius), tuple(emission)))

    # miss programs (host_includes/programs.hpp)
    def miss_gradient(self, c1, c2):
        self.miss = ("gradient", tuple(c1), tuple(c2))

    def miss_constant(self, c=(0.0, 0.0, 0.0)):
        self.miss = ("constant", tuple(c))

    def miss_env(self, rgba, spherical=True, kind=MISS_HDR):
        rgba = np.ascontiguousarray(rgba, dtype=np.float32)
        assert rgba.ndim == 3 and rgba.shape[2] == 4
        self.miss = ("env", rgba, int(spherical), kind)

    def set_camera(self, lookfrom, lookat, vup, vfov, aspect, aperture, focus, t0=0.0, t1=1.0):
        self.camera = (tuple(lookfrom), tuple(lookat), tuple(vup), float(vfov), float(aspect),
                       float(aperture), float(focus), float(t0), float(t1))


def noise_tables():
    """The default Perlin tables of pt_texture_noise: ranvec (256, 3) float32,
    perm (3, 256) int32."""
    lib = load_library()
    r = np.zeros((256, 3), np.float32)
    p = np.zeros((3, 256), np.int32)
    if lib.pt_noise_tables(_ptr(r), _ptr(p)) != 0:
        raise PtError(-1, "pt_noise_tables failed")
    return r, p


def _check(lib, ctx, rc):
    if rc != 0:
        raise PtError(rc, lib.pt_last_error(ctx).decode())


class GpuRenderer:
    """One pt_context with a committed scene."""

    def __init__(self, scene, device=0, path_slots=0, counters=False, timing=False, builder=0,
                 bvh_width=0, shade_order=0, refetch_lanes=0):
        self.lib = load_library()
        opt = Options(device, path_slots, 1 if counters else 0, 1 if timing else 0, builder,
                      bvh_width, shade_order, refetch_lanes)
        ctx = _P()
        rc = self.lib.pt_context_create(ctypes.byref(opt), ctypes.byref(ctx))
        if rc != 0:
            raise PtError(rc, "pt_context_create failed")
        self.ctx = ctx
        self.scene = scene
        self.load(scene)

    def close(self):
        if self.ctx:
            self.lib.pt_context_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        _check(self.lib, self.ctx, rc)

    def load(self, scene):
        L, c = self.lib, self.ctx
        for kind, a, b, cc, data, perm, ids in getattr(scene, "textures", []):
            tid = ctypes.c_uint32()
            if kind == TEX_CONSTANT:
                self._c(L.pt_texture_constant(c, f3(cc[:3]), ctypes.byref(tid)))
            elif kind == TEX_CHECKER:
                self._c(L.pt_texture_checker(c, a, b, ctypes.byref(tid)))
            elif kind == TEX_NOISE:
                self._c(L.pt_texture_noise(c, float(cc[0]), a, _ptr(data), _ptr(perm),
                                           ctypes.byref(tid)))
            elif kind == TEX_IMAGE:
                self._c(L.pt_texture_image(c, _ptr(data), a, b, ctypes.byref(tid)))
            elif kind == TEX_GRADIENT:
                self._c(L.pt_texture_gradient(c, f3(cc[0:3]), f3(cc[3:6]), f3(cc[6:9]),
                                              ctypes.byref(tid)))
            else:
                self._c(L.pt_texture_vector(c, _ptr(ids), b, ctypes.byref(tid)))
        mids = []
        for kind, c0, c1, p0, p1 in scene.materials:
            mid = ctypes.c_uint32()
            if kind == MAT_LAMBERTIAN:
                self._c(L.pt_material_lambertian(c, f3(c0), ctypes.byref(mid)))
            elif kind == MAT_METAL:
                self._c(L.pt_material_metal(c, f3(c0), p0, ctypes.byref(mid)))
            elif kind == MAT_DIELECTRIC:
                self._c(L.pt_material_dielectric(c, f3(c0), f3(c1), p0, p1, ctypes.byref(mid)))
            elif kind == MAT_DIFFUSE_LIGHT:
                self._c(L.pt_material_diffuse_light(c, f3(c0), ctypes.byref(mid)))
            elif kind == MAT_OREN_NAYAR:
                self._c(L.pt_material_oren_nayar(c, f3(c0), p0, ctypes.byref(mid)))
            elif kind == MAT_TORRANCE_SPARROW:
                self._c(L.pt_material_torrance_sparrow(c, f3(c0), p0, p1, ctypes.byref(mid)))
            elif kind == MAT_ASHIKHMIN_SHIRLEY:
                self._c(L.pt_material_ashikhmin_shirley(c, f3(c0), f3(c1), p0, p1,
                                                        ctypes.byref(mid)))
            mids.append(mid.value)
        for m, slot, t in getattr(scene, "mat_textures", []):
            self._c(L.pt_material_set_texture(c, mids[m], slot, t))
        tex_index = getattr(scene, "tex_index", {})
        add_obj = getattr(scene, "add_obj", {})
        for k, it in enumerate(scene.items):
            pid = ctypes.c_uint32()
            if k in add_obj:
                mesh, m = add_obj[k]
                xf = it[7]
                self._c(L.pt_add_obj(c, mesh.h, PT_OBJ_MTL if m is None else mids[m], _ptr(xf),
                                     ctypes.byref(pid)))
            elif it[0] == "sphere":
                _, cen, r, m, xf = it
                self._c(L.pt_add_sphere(c, f3(cen), r, mids[m], _ptr(xf), ctypes.byref(pid)))
            elif it[0] == "msphere":
                _, c0, c1, r, t0, t1, m, xf = it
                self._c(L.pt_add_moving_sphere(c, f3(c0), f3(c1), r, t0, t1, mids[m], _ptr(xf),
                                               ctypes.byref(pid)))
            elif it[0] == "rect":
                _, (a0, a1, b0, b1, k), flip, axis, m, xf = it
                self._c(L.pt_add_rect(c, a0, a1, b0, b1, k, flip, axis, mids[m], _ptr(xf),
                                      ctypes.byref(pid)))
            elif it[0] == "box":
                _, p0, p1, m, xf = it
                self._c(L.pt_add_box(c, f3(p0), f3(p1), mids[m], _ptr(xf), ctypes.byref(pid)))
            else:
                _, v, idx, m, mpt, nrm, uv, xf = it
                assert mids == list(range(len(mids)))  # ids are assigned in call order
                self._c(L.pt_add_mesh(c, _ptr(v), len(v), _ptr(idx), len(idx), _ptr(mpt),
                                      mids[m] if m is not None else 0, _ptr(nrm), _ptr(uv),
                                      _ptr(xf), ctypes.byref(pid)))
                if k in tex_index:
                    ti = tex_index[k]
                    self._c(L.pt_mesh_set_texture_index(c, pid.value, len(ti), _ptr(ti)))
        for lt in scene.lights:
            if lt[0] == "rect":
                _, (a0, a1, b0, b1, k), axis, e = lt
                self._c(L.pt_add_light_rect(c, a0, a1, b0, b1, k, axis, f3(e)))
            else:
                _, cen, r, e = lt
                self._c(L.pt_add_light_sphere(c, f3(cen), r, f3(e)))
        ms = scene.miss
        if ms[0] == "gradient":
            self._c(L.pt_set_env_gradient(c, f3(ms[1]), f3(ms[2])))
        elif ms[0] == "constant":
            self._c(L.pt_set_env_constant(c, f3(ms[1])))
        else:
            rgba = ms[1]
            self._c(L.pt_set_env_map(c, ms[3], _ptr(rgba), rgba.shape[1], rgba.shape[0], ms[2]))
        if scene.camera is not None:
            cf, ca, cu, vfov, aspect, ap, fd, t0, t1 = scene.camera
            self._c(L.pt_set_camera(c, f3(cf), f3(ca), f3(cu), vfov, aspect, ap, fd, t0, t1))
        self._c(L.pt_commit(c))

    @staticmethod
    def params(width, height, spp, frame0=0, max_depth=50, rr_enable=1, rr_depth=10, mode=0,
               guide=0):
        return RenderParams(width, height, spp, frame0, max_depth, rr_enable, rr_depth, mode,
                            guide)

    def render(self, params, acc=None, stream=None):
        """Accumulates into acc (numpy float32 HxWx4, or a device pointer int)."""
        if acc is None:
            acc = np.zeros((params.height, params.width, 4), dtype=np.float32)
        ptr = acc if isinstance(acc, int) else _ptr(acc)
        self._c(self.lib.pt_render(self.ctx, ctypes.byref(params), ptr, stream))
        return acc

    def render64(self, params, acc=None, stream=None):
        """Accumulates into acc (numpy float64 HxWx4, or a device pointer int)."""
        if acc is None:
            acc = np.zeros((params.height, params.width, 4), dtype=np.float64)
        ptr = acc if isinstance(acc, int) else _ptr(acc)
        self._c(self.lib.pt_render_accum64(self.ctx, ctypes.byref(params), ptr, stream))
        return acc

    # ---- learned guide
    GUIDE_PARAMS = 24320

    def guide_init(self, seed=0):
        self._c(self.lib.pt_guide_init(self.ctx, seed))

    def guide_training(self, lr=1e-2, steps=12, exponent=1.0, max_bounces=4):
        self._c(self.lib.pt_guide_set_training(self.ctx, lr, steps, exponent, max_bounces))

    def guide_params(self):
        out = np.zeros(self.GUIDE_PARAMS, np.float32)
        self._c(self.lib.pt_guide_get_params(self.ctx, _ptr(out)))
        return out

    def guide_set_params(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._c(self.lib.pt_guide_set_params(self.ctx, _ptr(w)))

    def guide_state(self):
        """(weights + Adam moments as 3 x GUIDE_PARAMS floats, Adam step)"""
        out = np.zeros(3 * self.GUIDE_PARAMS, np.float32)
        step = ctypes.c_int64()
        self._c(self.lib.pt_guide_get_state(self.ctx, _ptr(out), ctypes.byref(step)))
        return out, step.value

    def guide_set_state(self, state, step):
        s = np.ascontiguousarray(state, dtype=np.float32)
        self._c(self.lib.pt_guide_set_state(self.ctx, _ptr(s), int(step)))

    def guide_bounds(self):
        bmin = np.zeros(3, np.float32)
        binv = np.zeros(3, np.float32)
        self._c(self.lib.pt_guide_bounds(self.ctx, _ptr(bmin), _ptr(binv)))
        return bmin, binv

    def guide_eval(self, samples):
        s = np.ascontiguousarray(samples, dtype=np.float32)
        out = np.zeros((len(s), 48), np.float32)
        self._c(self.lib.pt_guide_eval(self.ctx, _ptr(s), len(s), _ptr(out)))
        return out

    def guide_gradient(self, samples):
        s = np.ascontiguousarray(samples, dtype=np.float32)
        g = np.zeros(self.GUIDE_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self._c(self.lib.pt_guide_gradient(self.ctx, _ptr(s), len(s), _ptr(g), _ptr(loss)))
        return g, float(loss[0])

    def guide_train(self, samples, lr=1e-2):
        s = np.ascontiguousarray(samples, dtype=np.float32)
        loss = np.zeros(1, np.float32)
        self._c(self.lib.pt_guide_train(self.ctx, _ptr(s), len(s), lr, _ptr(loss)))
        return float(loss[0])

    def render_paths(self, params, out=None):
        if out is None:
            out = np.zeros((params.height, params.width, 3), dtype=np.float32)
        self._c(self.lib.pt_render_paths(self.ctx, ctypes.byref(params), _ptr(out), None))
        return out

    def first_hits(self, width, height, frame):
        prim = np.zeros(width * height, dtype=np.uint32)
        mat = np.zeros(width * height, dtype=np.uint32)
        t = np.zeros(width * height, dtype=np.float32)
        self._c(self.lib.pt_trace_first_hits(self.ctx, width, height, frame, _ptr(prim),
                                             _ptr(mat), _ptr(t), None))
        return prim, mat, t

    def resolve(self, acc, frame):
        h, w = acc.shape[:2]
        out = np.zeros((h, w, 4), dtype=np.uint8)
        self._c(self.lib.pt_resolve_display(self.ctx, _ptr(acc), w, h, frame, _ptr(out), None))
        return out

    def stats(self):
        s = Stats()
        self._c(self.lib.pt_get_stats(self.ctx, ctypes.byref(s)))
        return _stats_dict(s)


def _stats_dict(s):
    d = {k: getattr(s, k) for k, _ in Stats._fields_}
    d["stage_ms"] = list(s.stage_ms)
    return d


class Batch:
    """A pt_batch: many committed scenes (GpuRenderer contexts) rendered in
    one wavefront."""

    def __init__(self, device=0, path_slots=0, counters=False, timing=False, bvh_width=0,
                 shade_order=0, refetch_lanes=0):
        self.lib = load_library()
        opt = Options(device, path_slots, 1 if counters else 0, 1 if timing else 0, 0, bvh_width,
                      shade_order, refetch_lanes)
        b = _P()
        rc = self.lib.pt_batch_create(ctypes.byref(opt), ctypes.byref(b))
        if rc != 0:
            raise PtError(rc, "pt_batch_create failed")
        self.b = b

    def close(self):
        if self.b:
            self.lib.pt_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        if rc != 0:
            raise PtError(rc, self.lib.pt_batch_last_error(self.b).decode())

    @staticmethod
    def _items(jobs):
        """jobs: list of (GpuRenderer, RenderParams, acc) with acc a numpy
        float32 HxWx4 array or a device pointer int."""
        arr = (BatchItem * len(jobs))()
        for k, (r, p, acc) in enumerate(jobs):
            arr[k].scene = r.ctx.value
            arr[k].params = p
            arr[k].accum_rgba = acc if isinstance(acc, int) else acc.ctypes.data
        return arr

    def render(self, jobs, stream=None):
        arr = self._items(jobs)
        self._c(self.lib.pt_batch_render(self.b, arr, len(jobs), stream))
        return [acc for _, _, acc in jobs]

    def autotune(self, jobs):
        arr = self._items(jobs)
        t = Tune()
        self._c(self.lib.pt_batch_autotune(self.b, arr, len(jobs), ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Tune._fields_}

    def set_tune(self, path_slots, trace_block, shade_block, bvh_width, chunk_paths=0,
                 shade_order=0, refetch_lanes=0):
        t = Tune(path_slots, trace_block, shade_block, bvh_width, chunk_paths, shade_order,
                 refetch_lanes, 0.0)
        self._c(self.lib.pt_batch_set_tune(self.b, ctypes.byref(t)))

    def tune(self):
        t = Tune()
        self._c(self.lib.pt_batch_get_tune(self.b, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Tune._fields_}

    def stats(self):
        s = Stats()
        self._c(self.lib.pt_batch_get_stats(self.b, ctypes.byref(s)))
        return _stats_dict(s)


# ------------------------------------------------------------ scene content
class SplitMix64:
    """splitmix64 (Steele, Lea & Flood 2014): the seeded stream of the
    synthetic scenes."""

    def __init__(self, seed):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self):
        return (self.next() >> 40) * (1.0 / (1 << 24))


def cornell_reference(width=500, height=500):
    """host_includes/scenes.hpp:188-260 (Cornell): Le 7, one green
    165x330x165 box translated (265,0,295) then rotated 15 deg about Y."""
    s = Scene()
    red = s.lambertian((0.65, 0.05, 0.05))
    white = s.lambertian((0.73, 0.73, 0.73))
    green = s.lambertian((0.12, 0.45, 0.15))
    light = s.diffuse_light((7.0, 7.0, 7.0))
    s.light_rect(213.0, 343.0, 227.0, 332.0, 554.0, PT_Y_AXIS, (7.0, 7.0, 7.0))
    s.miss_constant((0.0, 0.0, 0.0))
    s.rect(0, 555, 0, 555, 555, True, PT_X_AXIS, red)
    s.rect(0, 555, 0, 555, 0, False, PT_X_AXIS, green)
    s.rect(213, 343, 227, 332, 554, True, PT_Y_AXIS, light)
    s.rect(0, 555, 0, 555, 555, True, PT_Y_AXIS, white)
    s.rect(0, 555, 0, 555, 0, False, PT_Y_AXIS, white)
    s.rect(0, 555, 0, 555, 555, True, PT_Z_AXIS, white)
    xf = compose([mat_translate((265.0, 0.0, 295.0)), mat_rotate(15.0, PT_Y_AXIS)])
    s.box((0, 0, 0), (165, 330, 165), green, xf)
    s.set_camera((278, 278, -800), (278, 278, 0), (0, 1, 0), 40.0, width / height, 0.0, 10.0)
    return s


def cornell_c1(width=512, height=512):
    """Plain Cornell box of the first benchmark configuration: white walls
    and two white boxes, light 130x105 with emission 15."""
    s = Scene()
    red = s.lambertian((0.65, 0.05, 0.05))
    white = s.lambertian((0.73, 0.73, 0.73))
    green = s.lambertian((0.12, 0.45, 0.15))
    light = s.diffuse_light((15.0, 15.0, 15.0))
    s.light_rect(213.0, 343.0, 227.0, 332.0, 554.0, PT_Y_AXIS, (15.0, 15.0, 15.0))
    s.miss_constant((0.0, 0.0, 0.0))
    s.rect(0, 555, 0, 555, 555, True, PT_X_AXIS, green)
    s.rect(0, 555, 0, 555, 0, False, PT_X_AXIS, red)
    s.rect(213, 343, 227, 332, 554, True, PT_Y_AXIS, light)
    s.rect(0, 555, 0, 555, 555, True, PT_Y_AXIS, white)
    s.rect(0, 555, 0, 555, 0, False, PT_Y_AXIS, white)
    s.rect(0, 555, 0, 555, 555, True, PT_Z_AXIS, white)
    s.box((0, 0, 0), (165, 165, 165), white,
          compose([mat_translate((130.0, 0.0, 65.0)), mat_rotate(-18.0, PT_Y_AXIS)]))
    s.box((0, 0, 0), (165, 330, 165), white,
          compose([mat_translate((265.0, 0.0, 295.0)), mat_rotate(15.0, PT_Y_AXIS)]))
    s.set_camera((278, 278, -800), (278, 278, 0), (0, 1, 0), 40.0, width / height, 0.0, 10.0)
    return s


def random_spheres(width=1920, height=1080, seed=0, grid=11):
    """Random-spheres scene of the second benchmark configuration (the
    reference's InOneWeekend, host_includes/scenes.hpp:17-93, with a seeded
    splitmix64 stream): ground r=1000, 22x22 small spheres (80% Lambertian,
    15% metal, 5% glass), three r=1 spheres, gradient sky."""
    rng = SplitMix64(seed)
    U = rng.uniform
    s = Scene()
    s.miss_gradient((1.0, 1.0, 1.0), (0.5, 0.7, 1.0))
    ground = s.lambertian((0.5, 0.5, 0.5))
    s.sphere((0.0, -1000.0, 0.0), 1000.0, ground)
    for a in range(-grid, grid):
        for b in range(-grid, grid):
            choose = U()
            cx = a + 0.9 * U()
            cz = b + 0.9 * U()
            center = (cx, 0.2, cz)
            if choose < 0.8:
                alb = (U() * U(), U() * U(), U() * U())
                m = s.lambertian(alb)
            elif choose < 0.95:
                alb = (0.5 * (1 + U()), 0.5 * (1 + U()), 0.5 * (1 + U()))
                m = s.metal(alb, 0.5 * U())
            else:
                m = s.dielectric((1.0, 1.0, 1.0), (U(), U(), U()), 1.5)
            s.sphere(center, 0.2, m)
    s.sphere((4.0, 1.0, 0.0), 1.0, s.dielectric((1, 1, 1), (1, 1, 1), 1.5))
    s.sphere((0.0, 1.0, 0.5), 1.0, s.lambertian((0.4, 0.2, 0.1)))
    s.sphere((-4.0, 1.0, 1.0), 1.0, s.metal((0.7, 0.6, 0.5), 0.0))
    s.set_camera((13, 2, 3), (0, 0, 0), (0, 1, 0), 20.0, width / height, 0.1, 10.0)
    return s


def moving_spheres(width=640, height=360, seed=0, grid=5):
    """Motion-blur form of the random spheres (the reference's
    Moving_Sphere, hitables.hpp:130-181): the diffuse small spheres rise by
    up to 0.5 between time 0 and time 1, the camera's shutter spans [0, 1];
    a ceiling light quad over the scene is sampled by NEE, so shadow rays
    meet the moving spheres at their path's time too."""
    rng = SplitMix64(seed)
    U = rng.uniform
    s = Scene()
    s.miss_gradient((1.0, 1.0, 1.0), (0.5, 0.7, 1.0))
    ground = s.lambertian((0.5, 0.5, 0.5))
    s.sphere((0.0, -1000.0, 0.0), 1000.0, ground)
    for a in range(-grid, grid):
        for b in range(-grid, grid):
            choose = U()
            center = (a + 0.9 * U(), 0.2, b + 0.9 * U())
            if choose < 0.7:
                m = s.lambertian((U() * U(), U() * U(), U() * U()))
                s.moving_sphere(center, (center[0], center[1] + 0.5 * U(), center[2]), 0.2, 0.0,
                                1.0, m)
            elif choose < 0.9:
                m = s.metal((0.5 * (1 + U()), 0.5 * (1 + U()), 0.5 * (1 + U())), 0.5 * U())
                s.sphere(center, 0.2, m)
            else:
                s.moving_sphere(center, (center[0] + 0.3 * U(), center[1], center[2]), 0.2, 0.25,
                                0.75, s.dielectric((1.0, 1.0, 1.0), (U(), U(), U()), 1.5))
    s.sphere((0.0, 1.0, 0.5), 1.0, s.lambertian((0.4, 0.2, 0.1)))
    s.moving_sphere((-3.0, 1.0, 1.0), (-3.0, 1.6, 1.0), 1.0, 0.0, 1.0, s.metal((0.7, 0.6, 0.5), 0.0))
    lt = s.diffuse_light((8.0, 8.0, 8.0))
    s.rect(-1.5, 1.5, -1.5, 1.5, 5.0, 1, 1, lt)
    s.light_rect(-1.5, 1.5, -1.5, 1.5, 5.0, 1, (8.0, 8.0, 8.0))
    s.set_camera((13, 2, 3), (0, 0, 0), (0, 1, 0), 20.0, width / height, 0.1, 10.0, 0.0, 1.0)
    return s


def _hash01(i, j, seed):
    """Uniform [0,1) lattice values: splitmix64 finaliser of (i, j, seed)."""
    with np.errstate(over="ignore"):
        return _hash01_impl(i, j, seed)


def _hash01_impl(i, j, seed):
    z = (i.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)
         ^ j.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)
         ^ np.uint64(seed) * np.uint64(0x165667B19E3779F9))
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))


def fbm(x, z, octaves=6, seed=0, base_freq=4.0):
    """Fractional Brownian motion of value noise (lattice values from
    _hash01, smoothstep interpolation), roughly in [-1, 1]."""
    total = np.zeros_like(x, dtype=np.float64)
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        X, Z = x * freq, z * freq
        xi, zi = np.floor(X), np.floor(Z)
        fx, fz = X - xi, Z - zi
        xi, zi = xi.astype(np.int64), zi.astype(np.int64)
        ux, uz = fx * fx * (3 - 2 * fx), fz * fz * (3 - 2 * fz)
        s = seed * 131 + o
        v00, v10 = _hash01(xi, zi, s), _hash01(xi + 1, zi, s)
        v01, v11 = _hash01(xi, zi + 1, s), _hash01(xi + 1, zi + 1, s)
        n = (v00 * (1 - ux) + v10 * ux) * (1 - uz) + (v01 * (1 - ux) + v11 * ux) * uz
        total += amp * (2.0 * n - 1.0)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def heightfield_mesh(cells=1024, amplitude=0.1, seed=0, extent=1.0):
    """(cells+1)^2 vertices over [-extent, extent]^2 in x/z, y = amplitude *
    fBm (6 octaves); 2*cells^2 triangles; per-vertex normals and uvs."""
    n = cells + 1
    lin = np.linspace(-extent, extent, n)
    X, Z = np.meshgrid(lin, lin, indexing="xy")
    Y = amplitude * fbm(X, Z, 6, seed)
    verts = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(np.float32)
    dx = 2 * extent / cells
    gy, gx = np.gradient(Y, dx, dx)
    nrm = np.stack([-gx, np.ones_like(gx), -gy], axis=-1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    uu, vv = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="xy")
    uvs = np.stack([uu, vv], axis=-1).reshape(-1, 2).astype(np.float32)
    i, j = np.meshgrid(np.arange(cells), np.arange(cells), indexing="xy")
    v0 = (j * n + i).reshape(-1)
    v1, v2, v3 = v0 + 1, v0 + n, v0 + n + 1
    idx = np.empty((2 * cells * cells, 3), dtype=np.uint32)
    idx[0::2] = np.stack([v0, v2, v1], axis=-1)
    idx[1::2] = np.stack([v1, v2, v3], axis=-1)
    tile_of_tri = np.repeat(((j * 16 // cells) * 16 + (i * 16 // cells)).reshape(-1), 2)
    return verts, idx, nrm.reshape(-1, 3).astype(np.float32), uvs, tile_of_tri


def sky_env(width=2048, height=1024, sun_peak=5e4, sun_dir=(0.4, 0.6, -0.69), sigma=0.03):
    """Synthetic float32 HDR environment (RGBA, row 0 at v = 0) in the
    spherical mapping of programs/miss.cu:64-77: sky gradient, dark ground,
    Gaussian sun lobe of the given peak radiance."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    U, V = np.meshgrid(u, v, indexing="xy")
    lon, lat = U * 2 * np.pi, V * np.pi
    y = np.cos(lat)
    x, z = np.sin(lat) * np.cos(lon), np.sin(lat) * np.sin(lon)
    t = np.clip(y, 0, 1)[..., None]
    sky = (1 - t) * np.array([1.0, 1.0, 1.0]) + t * np.array([0.3, 0.5, 1.0])
    ground = np.array([0.15, 0.12, 0.1])
    col = np.where((y >= 0)[..., None], sky, ground)
    sd = np.array(sun_dir, dtype=np.float64)
    sd /= np.linalg.norm(sd)
    ang = np.arccos(np.clip(x * sd[0] + y * sd[1] + z * sd[2], -1, 1))
    col = col + sun_peak * np.exp(-0.5 * (ang / sigma) ** 2)[..., None] * np.array([1, 0.9, 0.8])
    rgba = np.concatenate([col, np.zeros_like(col[..., :1])], axis=-1)
    return np.ascontiguousarray(rgba, dtype=np.float32)


def heightfield_scene(width=1920, height=1080, cells=1024, seed=0, env_w=2048, env_h=1024,
                      env=None):
    """Triangle heightfield of the third benchmark configuration: fBm terrain
    with one material per tile (16x16 tiles) drawn from Torrance-Sparrow
    (roughness U[0.05,0.5]), Ashikhmin-Shirley (nu,nv U[10,1000]) and
    Oren-Nayar (sigma U[0,0.5]); HDR sky with a sun lobe (`env`, if given,
    is a ready sky_env array)."""
    rng = SplitMix64(seed ^ 0xC3)
    U = rng.uniform
    s = Scene()
    mats = []
    for _ in range(256):
        k = int(U() * 3)
        col = (0.3 + 0.6 * U(), 0.3 + 0.6 * U(), 0.3 + 0.6 * U())
        if k == 0:
            r = 0.05 + 0.45 * U()
            mats.append(s.torrance_sparrow(col, r, r))
        elif k == 1:
            mats.append(s.ashikhmin_shirley(col, (0.04 + 0.2 * U(),) * 3, 10 + 990 * U(),
                                            10 + 990 * U()))
        else:
            mats.append(s.oren_nayar(col, 0.5 * U()))
    verts, idx, nrm, uvs, tile = heightfield_mesh(cells, 0.1, seed)
    mpt = np.asarray(mats, dtype=np.uint32)[tile]
    s.mesh(verts, idx, mats[0], mat_per_tri=mpt, normals=nrm, uvs=uvs)
    s.miss_env(sky_env(env_w, env_h) if env is None else env, spherical=True)
    s.set_camera((0.0, 0.9, 1.9), (0.0, 0.0, 0.0), (0, 1, 0), 45.0, width / height, 0.0, 2.0)
    return s


def guide_box_scene(width=1920, height=1080, cells=1024, seed=0, env_w=2048, env_h=1024,
                    env=None, opening=0.005):
    """The hard-indirect variant of the heightfield scene (the learned-guide
    configuration): the terrain inside a closed white Lambertian box whose
    only opening, a square in the ceiling covering `opening` of the box's
    surface, lets the HDR sky in.  The camera is inside the box."""
    s = heightfield_scene(width, height, cells=cells, seed=seed, env_w=env_w, env_h=env_h,
                          env=env)
    wall = s.lambertian((0.7, 0.7, 0.7))
    x0, x1, y0, y1, z0, z1 = -1.02, 1.02, -0.2, 1.2, -1.02, 1.02
    area = 2 * (x1 - x0) * (z1 - z0) + 2 * (x1 - x0) * (y1 - y0) + 2 * (z1 - z0) * (y1 - y0)
    side = (opening * area) ** 0.5
    hx0, hz0 = 0.35 - side / 2, 0.25 - side / 2
    hx1, hz1 = hx0 + side, hz0 + side
    s.rect(y0, y1, z0, z1, x0, False, PT_X_AXIS, wall)       # normals face inside
    s.rect(y0, y1, z0, z1, x1, True, PT_X_AXIS, wall)
    s.rect(x0, x1, y0, y1, z0, False, PT_Z_AXIS, wall)
    s.rect(x0, x1, y0, y1, z1, True, PT_Z_AXIS, wall)
    s.rect(x0, x1, z0, z1, y0, False, PT_Y_AXIS, wall)       # floor under the terrain
    s.rect(x0, hx0, z0, z1, y1, True, PT_Y_AXIS, wall)       # ceiling around the opening
    s.rect(hx1, x1, z0, z1, y1, True, PT_Y_AXIS, wall)
    s.rect(hx0, hx1, z0, hz0, y1, True, PT_Y_AXIS, wall)
    s.rect(hx0, hx1, hz1, z1, y1, True, PT_Y_AXIS, wall)
    s.set_camera((0.0, 0.75, 0.98), (0.0, 0.0, -0.3), (0, 1, 0), 60.0, width / height, 0.0, 2.0)
    return s


def rel_mse(img, ref, eps=1e-2):
    """Mean over pixels and channels of (x - r)^2 / (r^2 + eps)."""
    x = np.asarray(img, np.float64)[..., :3]
    r = np.asarray(ref, np.float64)[..., :3]
    return float(np.mean((x - r) ** 2 / (r * r + eps)))


def batch_workload(n=64, seed=4, env_w=1024, env_h=512):
    """The batched multi-scene workload: n seeded heightfield scenes with
    triangle counts log-uniform over [1e3, 1e6], square images of 256, 512 or
    1024 pixels a side and spp uniform over 16..256.  Returns a list of
    (scene, size, spp, triangles)."""
    rng = SplitMix64(seed)
    U = rng.uniform
    env = sky_env(env_w, env_h)
    out = []
    for k in range(n):
        tris = 1e3 * 1000.0 ** U()
        cells = max(16, int(round((tris / 2) ** 0.5)))
        res = (256, 512, 1024)[min(2, int(U() * 3))]
        spp = 16 + min(240, int(U() * 241))
        out.append((heightfield_scene(res, res, cells=cells, seed=100 + k, env=env), res, spp,
                    2 * cells * cells))
    return out


def material_zoo(width=128, height=96, cells=12):
    """Small scene touching every primitive, material, light and transform
    path: spheres of all seven BRDFs, a transformed box, rects, a heightfield
    mesh with per-triangle TS/AS/ON materials, two lights (rect + sphere),
    gradient sky."""
    s = Scene()
    lam = s.lambertian((0.7, 0.6, 0.5))
    met = s.metal((0.8, 0.8, 0.9), 0.2)
    die = s.dielectric((1, 1, 1), (0.5, 0.5, 0.5), 1.5)
    on = s.oren_nayar((0.6, 0.7, 0.6), 0.4)
    ts = s.torrance_sparrow((0.9, 0.6, 0.3), 0.3, 0.3)
    ash = s.ashikhmin_shirley((0.5, 0.5, 0.7), (0.1, 0.1, 0.1), 50.0, 400.0)
    ash_iso = s.ashikhmin_shirley((0.7, 0.5, 0.5), (0.2, 0.2, 0.2), 80.0, 80.0)
    lt = s.diffuse_light((6.0, 6.0, 5.0))
    s.miss_gradient((1.0, 1.0, 1.0), (0.5, 0.7, 1.0))
    verts, idx, nrm, uvs, tile = heightfield_mesh(cells, 0.15, seed=3, extent=3.0)
    mpt = np.array([ts, ash, on, ash_iso], dtype=np.uint32)[tile % 4]
    s.mesh(verts, idx, ts, mat_per_tri=mpt, normals=nrm, uvs=uvs)
    for k, m in enumerate([lam, met, die, on, ts, ash]):
        s.sphere((-2.5 + k, 0.55, 0.0), 0.4, m)
    s.box((-0.3, 0.0, -0.3), (0.3, 0.6, 0.3), lam,
          compose([mat_translate((0.5, 0.2, -1.2)), mat_rotate(30.0, PT_Y_AXIS)]))
    s.rect(-1.0, 1.0, -1.0, 1.0, 2.5, True, PT_Y_AXIS, lt)
    s.light_rect(-1.0, 1.0, -1.0, 1.0, 2.5, PT_Y_AXIS, (6.0, 6.0, 5.0))
    s.sphere((1.8, 1.8, -1.0), 0.3, lt)
    s.light_sphere((1.8, 1.8, -1.0), 0.3, (6.0, 6.0, 5.0))
    s.rect(-3, 3, 0, 2, -2.0, False, PT_Z_AXIS, on)
    s.set_camera((0.0, 1.6, 4.5), (0.0, 0.3, 0.0), (0, 1, 0), 45.0, width / height, 0.05, 4.5)
    return s


# ------------------------------------------------------------ headless CLI
SCENES = {"cornell": cornell_c1, "cornell_reference": cornell_reference,
          "spheres": random_spheres, "heightfield": heightfield_scene,
          "guide_box": guide_box_scene, "zoo": material_zoo, "moving_spheres": moving_spheres}


def main(argv=None):
    """Headless render (the reference's GUI launch loop, main.cpp:174-354,
    without a window): builds one of the synthetic scenes, renders `spp`
    frames through the C ABI, prints the render statistics as one JSON line
    and optionally writes the image (Save_PNG / Save_HDR conventions)."""
    import argparse
    import json
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--scene", default="cornell", choices=sorted(SCENES))
    ap.add_argument("--width", type=int, default=512)
    ap.add_argument("--height", type=int, default=512)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--frame0", type=int, default=0)
    ap.add_argument("--mode", type=int, default=0, help="0 reference, 1 consistent (NEE + MIS)")
    ap.add_argument("--max-depth", type=int, default=50)
    ap.add_argument("--rr-depth", type=int, default=10)
    ap.add_argument("--builder", type=int, default=0, help="0 auto, 1 host SAH, 2 GPU LBVH")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", default="", help="image path (.png or .hdr)")
    a = ap.parse_args(argv)
    scene = SCENES[a.scene](a.width, a.height)
    r = GpuRenderer(scene, device=a.device, builder=a.builder)
    prm = GpuRenderer.params(a.width, a.height, a.spp, frame0=a.frame0, max_depth=a.max_depth,
                             rr_depth=a.rr_depth, mode=a.mode)
    acc = r.render(prm)
    st = r.stats()
    st.update(scene=a.scene, width=a.width, height=a.height, spp=a.spp, mode=a.mode)
    if a.out:
        (hdr_save if a.out.lower().endswith(".hdr") else png_save)(a.out, acc, a.spp)
    r.close()
    print(json.dumps(st))


if __name__ == "__main__":
    main()


def checker_image(w=64, h=32, seed=7):
    """A small seeded RGBA float image (row 0 at v = 0) for image textures."""
    rng = SplitMix64(seed)
    img = np.zeros((h, w, 4), np.float32)
    for y in range(h):
        for x in range(w):
            base = 0.8 if ((x // 8) + (y // 8)) % 2 else 0.2
            img[y, x, :3] = (base * (0.5 + 0.5 * rng.uniform()), base * x / w, base * y / h)
    img[..., 3] = 1.0
    return img


def texture_zoo(width=96, height=72):
    """Every texture callable of the reference on every material it can
    colour: checker (of a checker), Perlin noise, an image, a gradient, and a
    vector texture indexed per face on a heightfield mesh with uvs; textured
    Lambertian, Oren-Nayar, metal, dielectric, Torrance-Sparrow,
    Ashikhmin-Shirley (both colours) and an emitter; a rect light and a
    gradient sky."""
    s = Scene()
    red = s.texture_constant((0.8, 0.1, 0.1))
    white = s.texture_constant((0.9, 0.9, 0.9))
    fine = s.texture_checker(red, white)
    blue = s.texture_constant((0.1, 0.2, 0.8))
    check = s.texture_checker(fine, blue)
    noise = s.texture_noise(4.0, PT_Y_AXIS)
    image = s.texture_image(checker_image())
    grad = s.texture_gradient((0.9, 0.2, 0.2), (0.2, 0.9, 0.2), (0.2, 0.2, 0.9))
    vec = s.texture_vector([check, noise, image, grad])
    lam = s.lambertian((0.5, 0.5, 0.5))
    s.set_texture(lam, 0, vec)
    mats = []
    for k, (ctor, args) in enumerate([
            (s.lambertian, ((0.5, 0.5, 0.5),)), (s.oren_nayar, ((0.6, 0.6, 0.6), 0.3)),
            (s.metal, ((0.8, 0.8, 0.8), 0.1)),
            (s.dielectric, ((1.0, 1.0, 1.0), (0.5, 0.5, 0.5), 1.5)),
            (s.torrance_sparrow, ((0.9, 0.6, 0.3), 0.3, 0.3)),
            (s.ashikhmin_shirley, ((0.5, 0.5, 0.7), (0.1, 0.1, 0.1), 50.0, 400.0))]):
        m = ctor(*args)
        s.set_texture(m, 0, (check, noise, image, grad, noise, check)[k])
        mats.append(m)
    s.set_texture(mats[5], 1, grad)
    glow = s.diffuse_light((3.0, 3.0, 3.0))
    s.set_texture(glow, 0, check)
    verts, idx, nrm, uvs, tile = heightfield_mesh(8, 0.15, seed=9, extent=3.0)
    s.mesh(verts, idx, lam, normals=nrm, uvs=uvs, tex_index=(tile % 5).astype(np.uint32))
    for k, m in enumerate(mats):
        s.sphere((-2.5 + k, 0.55, 0.3 * (k % 2)), 0.45, m)
    s.box((-0.3, 0.0, -0.3), (0.3, 0.6, 0.3), mats[0],
          compose([mat_translate((0.6, 0.1, -1.3)), mat_rotate(25.0, PT_Y_AXIS)]))
    s.rect(-3, 3, 0, 2, -2.0, False, PT_Z_AXIS, mats[1])
    s.rect(-0.8, 0.8, -0.8, 0.8, 2.6, True, PT_Y_AXIS, glow)
    s.light_rect(-0.8, 0.8, -0.8, 0.8, 2.6, PT_Y_AXIS, (3.0, 3.0, 3.0))
    s.miss_gradient((1.0, 1.0, 1.0), (0.5, 0.7, 1.0))
    s.set_camera((0.0, 1.6, 4.5), (0.0, 0.3, 0.0), (0, 1, 0), 45.0, width / height, 0.05, 4.5)
    return s


SCENES["textures"] = texture_zoo
