"""The C ABI library builds for sm_103a, loads without a GPU, and exports every
entry point include/pike.h declares (no compute calls are made here)."""
import ctypes

from pike_gb300 import _lib


def test_header_declares_the_pass_api():
    syms = _lib.header_symbols()
    for name in ("pk_create", "pk_configure", "pk_camera", "pk_trace", "pk_shade_hit", "pk_trace_shadow",
                 "pk_shade_miss", "pk_accumulate", "pk_postprocess", "pk_render_frame", "pk_bvh_build",
                 "pk_env_build", "pk_scene_flatten", "pk_materials_set"):
        assert name in syms


def test_library_exports_every_declared_symbol(pk_built):
    lib = ctypes.CDLL(pk_built)
    missing = [s for s in _lib.header_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.pk_version() == 10000


def test_binding_covers_every_declared_symbol(pk_built):
    L = _lib.load()
    for s in _lib.header_symbols():
        assert getattr(L, s).restype is not None


def test_create_without_gpu_fails_cleanly(pk_built):
    import torch
    if torch.cuda.is_available():
        return
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.pk_create(ctypes.byref(h), 0) != _lib.PK_OK
    assert not h.value
