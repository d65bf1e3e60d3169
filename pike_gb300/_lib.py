"""ctypes binding of libpike.so (C ABI declared in include/pike.h).

There is no CPU fallback: if the CUDA library has not been built, loading it
raises.  Build it with ``python -m pike_gb300.build`` or
``__graft_entry__.build()``.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpike.so")
HEADER = os.path.join(HERE, "..", "include", "pike.h")

PK_OK, PK_ERR_ARG, PK_ERR_CUDA, PK_ERR_STATE, PK_ERR_DEVICE, PK_ERR_UNSUPPORTED = range(6)
PK_BVH_SWEEP = 0
PK_BVH_BINNED = 1
PK_ACCUM_RUNNING_MEAN, PK_ACCUM_COMPENSATED = 0, 1
PK_ENV_HISTOGRAM, PK_ENV_ALIAS = 0, 1
PK_QUEUE_RAYS, PK_QUEUE_SHADOW, PK_QUEUE_MISS = 0, 1, 2
PK_TRACE_CHUNKED, PK_TRACE_PERSISTENT, PK_TRACE_COMPACT_RECORDS, PK_TRACE_WIDE, PK_TRACE_EXACT = 0, 1, 2, 4, 8
PK_OVERLAP_AUTO = -1


class PikeError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pike error {code}: {msg}")
        self.code = code


class CameraState(C.Structure):
    """pk_camera_state: CameraPass.setCameraState's fields (camera_pass.js:118-125)."""
    _fields_ = [("pos", C.c_float * 3), ("dir", C.c_float * 3), ("fov", C.c_float), ("focal_depth", C.c_float),
                ("aperture_size", C.c_float), ("distortion", C.c_float), ("bokeh", C.c_float),
                ("invocation_offset", C.c_uint32)]


def camera_struct(state: dict) -> CameraState:
    """pk_camera_state of a CameraState dict (pos, dir, fov, focalDepth,
    apertureSize, distortion, bokeh, invocationOffset)."""
    cs = CameraState()
    cs.pos[:] = [float(v) for v in state["pos"]]
    cs.dir[:] = [float(v) for v in state["dir"]]
    cs.fov = float(state["fov"])
    cs.focal_depth = float(state.get("focalDepth", 0.5))
    cs.aperture_size = float(state.get("apertureSize", 0.0))
    cs.distortion = float(state.get("distortion", 0.0))
    cs.bokeh = float(state.get("bokeh", 0.5))
    cs.invocation_offset = int(state.get("invocationOffset", 0))
    return cs


_lib = None
_P = C.c_void_p


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    with open(HEADER) as f:
        txt = f.read()
    return re.findall(r"^(?:int|const char\*)\s+(pk_\w+)\s*\(", txt, flags=re.M)


def load(path: str = LIB_PATH):
    """Load libpike.so (raises OSError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build the CUDA library first (python -m pike_gb300.build)")
    L = C.CDLL(path)
    u32, i32, f32, f64 = C.c_uint32, C.c_int32, C.c_float, C.c_double
    sig = {
        "pk_create": [C.POINTER(_P), C.c_int], "pk_destroy": [_P], "pk_version": [],
        "pk_configure": [_P, u32, u32, u32],
        "pk_scene_flatten": [_P, _P, _P, _P, _P, u32, _P, u32, f64, _P],
        "pk_scene_flatten_tbn": [_P, _P, _P, _P, _P, _P, _P, u32, _P, u32],
        "pk_scene_upload": [_P, _P, u32, _P, _P, u32], "pk_scene_download": [_P, _P, _P],
        "pk_materials_set": [_P, _P, u32], "pk_materials_upload": [_P, _P, u32, _P, u32],
        "pk_materials_download": [_P, _P, _P, _P, _P], "pk_atlas_upload": [_P, _P, u32, u32],
        "pk_wide_info": [_P, _P, _P], "pk_wide_download": [_P, _P, _P], "pk_exact_download": [_P, _P, _P, _P],
        "pk_diff_render": [_P, _P, _P], "pk_diff_backward": [_P, _P, _P, _P, _P, _P],
        "pk_diff_rays": [_P, _P], "pk_diff_set_env_sampling": [_P, _P, u32, u32],
        "pk_diff_env_info": [_P, _P, _P, _P], "pk_diff_env_download": [_P, _P, _P, _P],
        "pk_batch_create": [_P, _P, u32], "pk_batch_destroy": [_P], "pk_batch_set_requests": [_P, _P, u32],
        "pk_batch_set_config": [_P, C.c_int, C.c_int, C.c_int], "pk_batch_get_config": [_P, _P, _P, _P],
        "pk_batch_autotune": [_P, C.c_uint64, _P], "pk_batch_render": [_P, u32], "pk_batch_reset": [_P],
        "pk_batch_read": [_P, u32, _P], "pk_batch_info": [_P, _P, _P, _P], "pk_batch_latencies": [_P, _P],
        "pk_set_accumulation": [_P, C.c_int],
        "pk_set_env_sampling": [_P, C.c_int], "pk_env_alias_download": [_P, _P, _P],
        "pk_set_frame_overlap": [_P, C.c_int],
        "pk_set_frames_in_flight": [_P, C.c_int],
        "pk_bvh_build": [_P, C.c_int], "pk_bvh_upload": [_P, _P, u32, _P, u32, _P, u32],
        "pk_bvh_info": [_P, _P, _P, _P], "pk_bvh_download": [_P, _P, _P, _P],
        "pk_env_build": [_P, _P, u32, u32], "pk_env_upload": [_P, _P, u32, u32, _P, u32, _P, _P],
        "pk_env_info": [_P, _P, _P, _P], "pk_env_download": [_P, _P, _P, _P],
        "pk_set_render_state": [_P, i32, f32], "pk_set_camera": [_P, C.POINTER(CameraState)],
        "pk_set_postprocess": [_P, f32, f32], "pk_clear_color": [_P], "pk_clear_hits_misses": [_P],
        "pk_clear_rays": [_P], "pk_camera": [_P], "pk_trace": [_P], "pk_shade_hit": [_P], "pk_trace_shadow": [_P],
        "pk_shade_miss": [_P], "pk_accumulate": [_P], "pk_postprocess": [_P],
        "pk_render_frame": [_P, u32], "pk_render_frames": [_P, u32, u32], "pk_sync": [_P],
        "pk_read_counters": [_P, _P], "pk_read_rays": [_P, C.c_int, u32, u32, _P], "pk_read_hits": [_P, u32, u32, _P],
        "pk_read_color": [_P, _P], "pk_read_accum": [_P, _P], "pk_write_accum": [_P, _P],
        "pk_read_display": [_P, _P, _P], "pk_set_counting": [_P, C.c_int], "pk_reset_stats": [_P],
        "pk_read_stats": [_P, _P], "pk_set_timing": [_P, C.c_int], "pk_read_timing": [_P, _P],
        "pk_math_eval": [_P, C.c_int, _P, _P, _P, u32],
        "pk_stream_timer": [_P, C.c_int, C.POINTER(C.c_float)],
        "pk_probe_read_bandwidth": [_P, C.c_uint64, u32, C.POINTER(C.c_float)], "pk_host_alloc": [_P, C.c_size_t, C.POINTER(_P)],
        "pk_host_free": [_P, _P], "pk_read_display_async": [_P, _P],
        "pk_cast_rays": [_P, _P, _P, u32, C.c_int, _P, _P, _P],
        "pk_cast_rays_noalloc": [_P, _P, _P, u32, C.c_int, _P, _P, _P],
        "pk_set_trace_mode": [_P, C.c_int],
        "pk_focus_distance": [_P, _P, _P, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.pk_last_error.argtypes = [_P]
    L.pk_last_error.restype = C.c_char_p
    _lib = L
    return L


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_P)


class Context:
    """One pk_ctx: a CUDA device, a stream and the device memory of one renderer."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = _P()
        rc = self.L.pk_create(C.byref(h), device)
        if rc != PK_OK:
            raise PikeError(rc, "pk_create failed (no CUDA device?)")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.pk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name: str, *args):
        rc = getattr(self.L, name)(self.h, *args)
        if rc != PK_OK:
            raise PikeError(rc, f"{name}: {self.L.pk_last_error(self.h).decode(errors='replace')}")
        return rc

    def timer_start(self):
        self.call("pk_stream_timer", 0, None)

    def timer_stop(self) -> float:
        ms = C.c_float(0.0)
        self.call("pk_stream_timer", 1, C.byref(ms))
        return float(ms.value)

    def pinned(self, shape, dtype) -> "PinnedArray":
        return PinnedArray(self, shape, dtype)

    def last_error(self) -> str:
        return self.L.pk_last_error(self.h).decode(errors="replace")


class PinnedArray:
    """A numpy view of page-locked host memory owned by the library."""

    def __init__(self, ctx: Context, shape, dtype):
        self.ctx = ctx
        dt = np.dtype(dtype)
        n = int(np.prod(shape)) * dt.itemsize
        p = _P()
        ctx.call("pk_host_alloc", n, C.byref(p))
        self.p = p
        buf = (C.c_uint8 * n).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dt).reshape(shape)

    def free(self):
        if self.p is not None and getattr(self.ctx, "h", None):
            self.ctx.call("pk_host_free", self.p)
        self.p = None
