"""Form (2): batched rendering of many requests over resident scenes in one
persistent launch (pk_batch_*), with the measured launch configuration.

``scene_context(src)`` builds a library context holding one scene (GPU BVH,
materials, environment).  ``Batch(contexts)`` renders lists of
``Request``s; ``random_requests`` draws the batching workload (resolutions
log-uniform between 128x128 and 1920x1080, spp in {1, 4, 16, 64}, depth
4..8, cameras on random orbits around each scene).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math

import numpy as np

from . import _lib
from ._lib import CameraState, Context, PikeError, ptr


class BatchRequestC(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("depth", C.c_uint32), ("camera", CameraState)]


@dataclasses.dataclass
class Request:
    scene: int
    width: int
    height: int
    spp: int
    depth: int
    camera: dict

    @property
    def paths(self) -> int:
        return self.width * self.height * self.spp


def scene_context(src, device: int = 0) -> Context:
    """A context with the scene, its GPU-built BVH, materials and environment."""
    ctx = Context(device)
    ctx.call("pk_configure", 64, 64, 64 * 64)
    tr = np.zeros(3)
    ctx.call("pk_scene_flatten", ptr(np.ascontiguousarray(src.pos)), ptr(np.ascontiguousarray(src.normal)),
             ptr(np.ascontiguousarray(src.tangent)), ptr(np.ascontiguousarray(src.uv)), src.pos.shape[0],
             ptr(np.ascontiguousarray(src.tris, np.int32)), src.tris.shape[0], 1.0, ptr(tr))
    mats = np.ascontiguousarray(src.materials, np.float64)
    ctx.call("pk_materials_set", ptr(mats), mats.shape[0])
    ctx.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
    env = np.ascontiguousarray(src.env_rgbe, np.uint8)
    ctx.call("pk_env_build", ptr(env), env.shape[1], env.shape[0])
    return ctx


def orbit_camera(rng: np.random.Generator, radius: float = 2.2, fov: float = math.pi / 3) -> dict:
    """A camera on a random orbit around the normalised scene, looking at its centre."""
    phi = rng.uniform(0.0, 2.0 * math.pi)
    elev = rng.uniform(0.15, 0.6)
    pos = np.array([radius * math.cos(phi) * math.cos(elev), radius * math.sin(elev),
                    radius * math.sin(phi) * math.cos(elev)])
    d = -pos / np.linalg.norm(pos)
    return dict(pos=[float(np.float32(v)) for v in pos], dir=[float(np.float32(v)) for v in d], fov=float(fov),
                focalDepth=0.5, apertureSize=0.0, distortion=0.0, bokeh=0.5, invocationOffset=0)


def random_requests(n: int, n_scenes: int, seed: int = 3) -> list[Request]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        t = rng.uniform()
        w = int(round(128 * (1920 / 128) ** t))
        h = int(round(128 * (1080 / 128) ** t))
        out.append(Request(scene=int(rng.integers(0, n_scenes)), width=w, height=h,
                           spp=int(rng.choice([1, 4, 16, 64])), depth=int(rng.integers(4, 9)),
                           camera=orbit_camera(rng)))
    return out


def _camera_struct(state: dict) -> CameraState:
    cs = CameraState()
    cs.pos[:] = [float(v) for v in state["pos"]]
    cs.dir[:] = [float(v) for v in state["dir"]]
    cs.fov = float(state["fov"])
    cs.focal_depth = float(state.get("focalDepth", 0.5))
    cs.aperture_size = float(state.get("apertureSize", 0.0))
    cs.distortion = float(state.get("distortion", 0.0))
    cs.bokeh = float(state.get("bokeh", 0.5))
    cs.invocation_offset = 0
    return cs


class Batch:
    def __init__(self, contexts: list[Context]):
        self.lib = _lib.load()
        self.contexts = list(contexts)  # kept alive: the batch points into their buffers
        arr = (C.c_void_p * len(contexts))(*[c.h.value for c in contexts])
        h = C.c_void_p()
        rc = self.lib.pk_batch_create(C.byref(h), arr, len(contexts))
        if rc:
            raise PikeError(rc, "pk_batch_create failed")
        self.h = h
        self.requests: list[Request] = []

    def _call(self, name: str, *args):
        rc = getattr(self.lib, name)(self.h, *args)
        if rc:
            self.lib.pk_batch_last_error.restype = C.c_char_p
            msg = self.lib.pk_batch_last_error(self.h)
            raise PikeError(rc, f"{name}: {msg.decode() if msg else ''}")

    def close(self):
        if self.h:
            self.lib.pk_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_requests(self, reqs: list[Request]):
        arr = (BatchRequestC * len(reqs))()
        for i, r in enumerate(reqs):
            arr[i].scene, arr[i].width, arr[i].height = r.scene, r.width, r.height
            arr[i].spp, arr[i].depth = r.spp, r.depth
            arr[i].camera = _camera_struct(r.camera)
        self._call("pk_batch_set_requests", arr, len(reqs))
        self.requests = list(reqs)

    def set_config(self, block: int, stack: int, chunk: int):
        self._call("pk_batch_set_config", block, stack, chunk)

    def config(self) -> tuple[int, int, int]:
        b, s, c = C.c_int(), C.c_int(), C.c_int()
        self._call("pk_batch_get_config", C.byref(b), C.byref(s), C.byref(c))
        return b.value, s.value, c.value

    def autotune(self, sample_paths: int = 0) -> float:
        ms = C.c_float()
        self._call("pk_batch_autotune", C.c_uint64(sample_paths), C.byref(ms))
        return ms.value

    def render(self, frames: int = 1) -> float:
        """Renders `frames` frames of every request; returns the device milliseconds."""
        self._call("pk_batch_render", frames)
        return self.info()[2]

    def reset(self):
        self._call("pk_batch_reset")

    def info(self):
        n, f, ms = C.c_uint64(), C.c_uint32(), C.c_float()
        self._call("pk_batch_info", C.byref(n), C.byref(f), C.byref(ms))
        return int(n.value), int(f.value), float(ms.value)

    def latencies(self) -> np.ndarray:
        """Per-request completion times (ms from the launch) of the last frame."""
        out = np.zeros(len(self.requests), np.float32)
        self._call("pk_batch_latencies", ptr(out))
        return out

    def image(self, i: int) -> np.ndarray:
        r = self.requests[i]
        out = np.zeros((r.height, r.width, 4), np.float32)
        self._call("pk_batch_read", i, ptr(out))
        return out
