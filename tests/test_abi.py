"""The C ABI library loads without a GPU and exports every entry point that
include/pt.h declares."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        names += re.findall(r"PT_API\s+[\w\s\*]+?\b(pt_\w+)\s*\(", text)
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    assert len(names) >= 25
    for n in ("pt_context_create", "pt_commit", "pt_render", "pt_trace_first_hits"):
        assert n in names


def test_library_exports_declared_symbols(ptgb_mod):
    lib = ctypes.CDLL(ptgb_mod.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header(ptgb_mod):
    names = set(declared_symbols())
    covered = set(ptgb_mod.SIGNATURES) | {"pt_last_error", "pt_version", "pt_batch_last_error",
                                          "pt_io_last_error", "pt_image_last_error"}
    assert names == covered, names ^ covered


def test_version_string(ptgb_mod):
    lib = ptgb_mod.load_library()
    assert b"sm_103a" in lib.pt_version()


def test_context_options_checked_without_gpu(ptgb_mod):
    """pt_context_create rejects out-of-range options before it touches the
    device (pt.h: bvh_width 2..8, shade_order 0..2, refetch_lanes 0..32)."""
    lib = ptgb_mod.load_library()
    for field, value in (("refetch_lanes", 33), ("refetch_lanes", -1), ("bvh_width", 9),
                         ("bvh_width", 1), ("shade_order", 3)):
        opt = ptgb_mod.Options()
        setattr(opt, field, value)
        ctx = ctypes.c_void_p()
        rc = lib.pt_context_create(ctypes.byref(opt), ctypes.byref(ctx))
        assert rc == -1 and not ctx.value, (field, value, rc)


def test_batch_options_checked_without_gpu(ptgb_mod):
    lib = ptgb_mod.load_library()
    opt = ptgb_mod.Options()
    opt.refetch_lanes = 40
    b = ctypes.c_void_p()
    assert lib.pt_batch_create(ctypes.byref(opt), ctypes.byref(b)) == -1 and not b.value
