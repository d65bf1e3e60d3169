"""Shared setup for the parity tests: one scene prepared on both the GPU (through
the C ABI) and the CPU oracle, with helpers to compare queues bit for bit."""
from __future__ import annotations

import numpy as np

from pike_gb300 import _lib
from pike_gb300._lib import CameraState, Context, ptr
from pike_gb300.passes import read_counters


def camera_struct(state: dict) -> CameraState:
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


class Pair:
    """A synthetic scene set up on the GPU and in the oracle, sharing the same inputs."""

    def __init__(self, src, oracle, ctx: Context | None = None, gpu_bvh: bool = True, gpu_env: bool = True,
                 batch: int | None = None, threads: int | None = None, camera: dict | None = None,
                 trace_mode: int = _lib.PK_TRACE_PERSISTENT):
        self.src = src
        self.P = oracle.Prepared(src, threads=threads, batch=batch)
        self.ctx = ctx or Context(0)
        c = self.ctx
        self.batch = batch or src.width * src.height
        c.call("pk_configure", src.width, src.height, self.batch)
        c.call("pk_set_trace_mode", trace_mode)
        pos, nrm = np.ascontiguousarray(src.pos), np.ascontiguousarray(src.normal)
        tan, uv = np.ascontiguousarray(src.tangent), np.ascontiguousarray(src.uv)
        tris = np.ascontiguousarray(src.tris, np.int32)
        tr = np.zeros(3)
        c.call("pk_scene_flatten", ptr(pos), ptr(nrm), ptr(tan), ptr(uv), pos.shape[0], ptr(tris), tris.shape[0],
               1.0, ptr(tr))
        mats = np.ascontiguousarray(src.materials, np.float64)
        c.call("pk_materials_set", ptr(mats), mats.shape[0])
        if gpu_bvh:
            c.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
        else:
            b = self.P.bvh
            c.call("pk_bvh_upload", ptr(b.nodes), b.nodes.shape[0], ptr(b.tris), b.tris.shape[0], ptr(b.verts),
                   b.verts.shape[0])
        env = np.ascontiguousarray(src.env_rgbe, np.uint8)
        if gpu_env:
            c.call("pk_env_build", ptr(env), env.shape[1], env.shape[0])
        else:
            e = self.P.env
            c.call("pk_env_upload", ptr(env), env.shape[1], env.shape[0], ptr(e.bins), e.bins.shape[0], ptr(e.coords),
                   ptr(e.pdf))
        self.camera = camera or src.camera_state()
        self.set_camera(self.camera)

    def set_camera(self, state: dict):
        self.camera = state
        self.ctx.call("pk_set_camera", camera_struct(state))
        self.P.r.set_camera(state)

    def set_render_state(self, samples: int, theta: float = 0.0):
        self.ctx.call("pk_set_render_state", samples, theta)
        self.P.r.set_render_state(samples, theta)

    # ---- GPU readbacks in the oracle's layouts ----
    def counters(self) -> dict:
        return read_counters(self.ctx)

    def rays(self, queue: int, first: int, count: int) -> np.ndarray:
        out = np.zeros((count, 12), np.float32)
        self.ctx.call("pk_read_rays", queue, first, count, ptr(out))
        return out

    def hits(self, count: int) -> np.ndarray:
        out = np.zeros((count, 16), np.uint32)
        self.ctx.call("pk_read_hits", 0, count, ptr(out))
        return out

    def image(self, which: str) -> np.ndarray:
        out = np.zeros((self.src.height, self.src.width, 4), np.float32)
        if which == "display":
            out8 = np.zeros((self.src.height, self.src.width, 4), np.uint8)
            self.ctx.call("pk_read_display", ptr(out), ptr(out8))
            return out8
        self.ctx.call({"color": "pk_read_color", "accum": "pk_read_accum"}[which], ptr(out))
        return out


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a).view(np.uint32)


def assert_bits_equal(got: np.ndarray, want: np.ndarray, what: str):
    g, w = bits(got), bits(want)
    assert g.shape == w.shape, f"{what}: shape {g.shape} != {w.shape}"
    bad = np.argwhere(g != w)
    if bad.size:
        i = tuple(bad[0])
        raise AssertionError(f"{what}: {bad.shape[0]} words differ; first at {i}: got {g[i]:#x} want {w[i]:#x}")


def assert_bits_equal_nan(got: np.ndarray, want: np.ndarray, what: str):
    """Bit equality where NaNs sit in the same places; their payloads may differ
    (x86 produces a negative quiet NaN where the GPU produces 0x7fffffff)."""
    g, w = np.ascontiguousarray(got, np.float32), np.ascontiguousarray(want, np.float32)
    gn, wn = np.isnan(g), np.isnan(w)
    assert np.array_equal(gn, wn), f"{what}: NaNs differ in {int(np.count_nonzero(gn != wn))} places"
    assert_bits_equal(np.where(gn, np.float32(0), g), np.where(wn, np.float32(0), w), what)
