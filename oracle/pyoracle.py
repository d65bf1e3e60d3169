"""ctypes wrapper around liboracle.so, the CPU restatement of Pike's path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's CPU-baseline legs (as the timed CPU restatement).
The product package never imports this module.

Parity unpinned: the reference has no tests or fixtures and cannot run here;
see oracle/om_build.h and oracle/om_render.h for the reference lines followed.
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(_HERE, f) for f in ("pk_oracle.cpp", "om_math.h", "om_build.h", "om_render.h", "om_render64.h",
                                             "om_render_f64.h", "om_diff.h", "om_wide.h", "Makefile")]
    if force or not os.path.exists(_LIB) or max(os.path.getmtime(s) for s in srcs) > os.path.getmtime(_LIB):
        subprocess.run(["make", "-s", "-C", _HERE, "-B", "liboracle.so"], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB)
        _lib.or_last_error.restype = C.c_char_p
        for name in ("or_bvh_build", "or_env_build", "or_env_build_f32", "or_renderer_new", "or_wide_build"):
            getattr(_lib, name).restype = C.c_void_p
        _lib.or_env_num_bins.restype = C.c_size_t
        _lib.or_shadow_offset.restype = C.c_size_t
        _lib.or_set_render_state.argtypes = [C.c_void_p, C.c_int32, C.c_float]
        _lib.or_set_post.argtypes = [C.c_void_p, C.c_float, C.c_float]
        for name in ("or_bvh_free", "or_env_free", "or_renderer_free", "or_begin_frame", "or_camera", "or_trace",
                     "or_shade_hit", "or_trace_shadow", "or_shade_miss", "or_accumulate", "or_postprocess",
                     "or_reset_stats", "or_clear_color", "or_clear_hits_misses", "or_clear_rays"):
            getattr(_lib, name).argtypes = [C.c_void_p]
        _lib.or_tick.argtypes = [C.c_void_p, C.c_uint32]
        _lib.or_tick_batch.argtypes = [C.c_void_p, C.c_uint32]
        _lib.or_set_threads.argtypes = [C.c_void_p, C.c_int]
        _lib.or_set_track64.argtypes = [C.c_void_p, C.c_int]
        _lib.or_frames64.argtypes = [C.c_void_p]
        _lib.or_frames64.restype = C.c_uint64
        _lib.or_read64.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        _lib.or_render64_new.restype = C.c_void_p
        _lib.or_render64_new.argtypes = [C.c_void_p]
        _lib.or_render64_free.argtypes = [C.c_void_p]
        _lib.or_render64_tick.argtypes = [C.c_void_p, C.c_uint32]
        _lib.or_render64_frames.argtypes = [C.c_void_p]
        _lib.or_render64_frames.restype = C.c_uint64
        _lib.or_render64_read.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _err(what):
    raise RuntimeError(f"{what}: {lib().or_last_error().decode()}")


def flatten(src, scale: float = 1.0, translate=(0.0, 0.0, 0.0)):
    """Row S (scene.js:456-470): returns (pos f64 (V,3), attrs u32 (V,4))."""
    L = lib()
    n = src.pos.shape[0]
    pos = np.ascontiguousarray(src.pos, np.float64)
    nrm = np.ascontiguousarray(src.normal, np.float64)
    tan = np.ascontiguousarray(src.tangent, np.float64)
    uv = np.ascontiguousarray(src.uv, np.float64)
    tr = np.asarray(translate, np.float64)
    pos_out = np.zeros((n, 3), np.float64)
    attrs = np.zeros((n, 4), np.uint32)
    L.or_flatten(_p(pos), _p(nrm), _p(tan), _p(uv), C.c_size_t(n), C.c_double(scale), _p(tr), _p(pos_out), _p(attrs))
    return pos_out, attrs


def flatten_tbn(pos, nrm, tan4, bn, bt4, uv):
    """pk_scene_flatten_tbn restated: (pos f64 (V,3), attrs u32 (V,4))."""
    arrs = [np.ascontiguousarray(a, np.float64) for a in (pos, nrm, tan4, bn, bt4, uv)]
    n = arrs[0].shape[0]
    pos_out = np.zeros((n, 3), np.float64)
    attrs = np.zeros((n, 4), np.uint32)
    lib().or_flatten_tbn(*[_p(a) for a in arrs], C.c_size_t(n), _p(pos_out), _p(attrs))
    return pos_out, attrs


def materials(mats9: np.ndarray):
    """Row M: returns (index table i32 (M,4), layers u8 (L,4))."""
    L = lib()
    m = np.ascontiguousarray(mats9, np.float64)
    idx = np.zeros((m.shape[0], 4), np.int32)
    cap = 4 * m.shape[0]
    layers = np.zeros((cap, 4), np.uint8)
    nl = C.c_size_t(0)
    if L.or_materials(_p(m), C.c_size_t(m.shape[0]), _p(idx), _p(layers), C.c_size_t(cap), C.byref(nl)):
        _err("or_materials")
    return idx, layers[: nl.value].copy()


class BVH:
    """bvh.js + trace_pass.js packing: nodes (N,5) i32, leaf-ordered tris (T,4) i32, verts (V,4) f32."""

    def __init__(self, pos: np.ndarray, tris: np.ndarray):
        L = lib()
        pos = np.ascontiguousarray(pos, np.float64)
        tris = np.ascontiguousarray(tris, np.int32)
        h = L.or_bvh_build(_p(pos), C.c_size_t(pos.shape[0]), _p(tris), C.c_size_t(tris.shape[0]))
        if not h:
            _err("or_bvh_build")
        info = np.zeros(4, np.uint64)
        L.or_bvh_info(C.c_void_p(h), _p(info))
        self.n_nodes, self.n_leaf_tris, self.max_depth, self.largest_leaf = (int(x) for x in info)
        self.nodes = np.zeros((self.n_nodes, 5), np.int32)
        self.tris = np.zeros((self.n_leaf_tris, 4), np.int32)
        self.verts = np.zeros((pos.shape[0], 4), np.float32)
        norm = np.zeros(10, np.float64)
        L.or_bvh_copy(C.c_void_p(h), _p(self.nodes), _p(self.tris), _p(self.verts), _p(norm))
        self._h = h
        self.center, self.scale = norm[:3].copy(), float(norm[3])
        self.root_min, self.root_max = norm[4:7].copy(), norm[7:10].copy()

    def __del__(self):
        if getattr(self, "_h", None):
            lib().or_bvh_free(C.c_void_p(self._h))
            self._h = None

    def cast(self, rays6: np.ndarray) -> np.ndarray:
        """Raycaster.cast (raycaster.js:128-131) of rays {origin, dir} in the normalised frame."""
        rays6 = np.ascontiguousarray(rays6, np.float64)
        out = np.zeros(rays6.shape[0], np.float64)
        lib().or_bvh_cast(C.c_void_p(self._h), _p(rays6), C.c_size_t(rays6.shape[0]), _p(out))
        return out


class Env:
    """env_sampler.js tables: bins (nb,2) i32, coords (N,2) i32, pdf (h,w) f32."""

    def __init__(self, rgbe: np.ndarray):
        L = lib()
        rgbe = np.ascontiguousarray(rgbe, np.uint8)
        h, w = rgbe.shape[:2]
        hd = L.or_env_build(_p(rgbe), C.c_uint32(w), C.c_uint32(h))
        if not hd:
            _err("or_env_build")
        nb = int(L.or_env_num_bins(C.c_void_p(hd)))
        self.rgbe = rgbe
        self.w, self.h = w, h
        self.bins = np.zeros((nb, 2), np.int32)
        self.coords = np.zeros((w * h, 2), np.int32)
        self.pdf = np.zeros((h, w), np.float32)
        tb = np.zeros(2, np.float64)
        L.or_env_copy(C.c_void_p(hd), _p(self.bins), _p(self.coords), _p(self.pdf), _p(tb))
        L.or_env_free(C.c_void_p(hd))
        self.total, self.brightest = float(tb[0]), float(tb[1])


def wide_build(nodes5: np.ndarray, tri4: np.ndarray, verts4: np.ndarray):
    """Form (1)'s compressed 8-wide BVH restated on the host (om_wide.h):
    nodes (n, 20) float32, tris (n_tris, 12) float32, depth."""
    L = lib()
    nodes5 = np.ascontiguousarray(nodes5, np.int32)
    tri4 = np.ascontiguousarray(tri4, np.int32)
    verts4 = np.ascontiguousarray(verts4, np.float32)
    h = L.or_wide_build(_p(nodes5), C.c_uint32(nodes5.size // 5), _p(tri4), C.c_uint32(tri4.size // 4), _p(verts4),
                        C.c_uint32(verts4.size // 4))
    if not h:
        _err("or_wide_build")
    h = C.c_void_p(h)
    L.or_wide_nodes.restype = C.c_uint32
    L.or_wide_depth.restype = C.c_uint32
    n = int(L.or_wide_nodes(h))
    nodes = np.zeros((n, 20), np.float32)
    tris = np.zeros((tri4.size // 4, 12), np.float32)
    L.or_wide_copy(h, _p(nodes), _p(tris))
    depth = int(L.or_wide_depth(h))
    L.or_wide_free(h)
    return nodes, tris, depth


def exact_build(nodes5: np.ndarray, tri4: np.ndarray, verts4: np.ndarray):
    """The FP32 binary reference's records restated on the host: records
    (n_inner, 16) float32, tris (n_tris, 12) float32, root code."""
    L = lib()
    nodes5 = np.ascontiguousarray(nodes5, np.int32)
    tri4 = np.ascontiguousarray(tri4, np.int32)
    verts4 = np.ascontiguousarray(verts4, np.float32)
    n_inner = max(int((nodes5.reshape(-1, 5)[:, 1] <= -1).sum()), 1)
    rec = np.zeros((n_inner, 16), np.float32)
    tris = np.zeros((max(tri4.size // 4, 1), 12), np.float32)
    root = C.c_int32(0)
    if L.or_exact_build(_p(nodes5), C.c_uint32(nodes5.size // 5), _p(tri4), C.c_uint32(tri4.size // 4), _p(verts4),
                        C.c_uint32(verts4.size // 4), _p(rec), _p(tris), C.byref(root)):
        _err("or_exact_build")
    return rec, tris, int(root.value)


class EnvF32:
    """The differentiable renderer's sampling tables of an FP32 RGB map (h, w, 3)
    (pk_diff_set_env_sampling): bins (nb,2), coords (N,2), pdf (h,w); the C
    handle stays alive for the oracle's diff_render / diff_grad."""

    def __init__(self, rgb: np.ndarray):
        L = lib()
        rgb = np.ascontiguousarray(rgb, np.float32)
        h, w = rgb.shape[:2]
        hd = L.or_env_build_f32(_p(rgb), C.c_uint32(w), C.c_uint32(h))
        if not hd:
            _err("or_env_build_f32")
        self._h = hd
        nb = int(L.or_env_num_bins(C.c_void_p(hd)))
        self.w, self.h = w, h
        self.bins = np.zeros((nb, 2), np.int32)
        self.coords = np.zeros((w * h, 2), np.int32)
        self.pdf = np.zeros((h, w), np.float32)
        tb = np.zeros(2, np.float64)
        L.or_env_copy(C.c_void_p(hd), _p(self.bins), _p(self.coords), _p(self.pdf), _p(tb))
        self.total, self.brightest = float(tb[0]), float(tb[1])

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.or_env_free(C.c_void_p(self._h))
            self._h = None


def env_alias(rgbe: np.ndarray, return_weights: bool = False):
    """PK_ENV_ALIAS's table restated in numpy (the precision form; no
    reference counterpart): the radiance of env_sampler.js:43-48 in FP64,
    its total summed in the GPU builder's grouping (blocks of 1024 texels:
    four strided values per thread, a shuffle tree per warp, the eight warp
    sums in order; then 1024 strided partial sums and a halving tree), the
    weights q = rint(radiance * n 2^f / total) with f = 61 - ceil(log2 n),
    and the sweep of Huebschle-Schneider & Sanders ("Parallel Weighted
    Random Sampling", 2022) evaluated from exact integer prefix sums.
    Returns (table (n, 2) uint32 {keep threshold, alias}, pdf (n,) float32),
    or None for a black map; with return_weights, (q, f) instead."""
    c = np.asarray(rgbe, np.uint8).reshape(-1, 4)
    cf = c.astype(np.float64)
    r = np.ldexp(1.0, c[:, 3].astype(np.int64) - 128) * (0.2126 * cf[:, 0] + 0.7152 * cf[:, 1] + 0.0722 * cf[:, 2]) / 255.0
    n = r.size
    nb = (n + 1023) // 1024
    R = np.zeros(nb * 1024)
    R[:n] = r
    R = R.reshape(nb, 4, 256)
    v = ((R[:, 0] + R[:, 1]) + R[:, 2]) + R[:, 3]  # (nb, 256): thread sums (0.0 + x adds nothing)
    v = v.reshape(nb, 8, 32)
    for o in (16, 8, 4, 2, 1):  # __shfl_down_sync: a lane past the warp reads its own value
        src = np.arange(32) + o
        other = np.where(src < 32, v[:, :, np.minimum(src, 31)], v)
        v = v + other
    w = v[:, :, 0]
    partial = np.zeros(nb)
    for k in range(8):
        partial = partial + w[:, k]
    s = np.zeros(1024)
    for t0 in range(0, nb, 1024):
        chunk = partial[t0:t0 + 1024]
        s[:chunk.size] = s[:chunk.size] + chunk
    width = 512
    while width > 0:
        s[:width] = s[:width] + s[width:2 * width]
        width //= 2
    total = s[0]
    if not (total > 0.0 and np.isfinite(total)):
        return None
    lg = 0
    while (1 << lg) < n:
        lg += 1
    frac = 61 - lg
    one = np.uint64(1 << frac)
    q = np.rint(r * (np.ldexp(float(n), frac) / total)).astype(np.uint64)
    if return_weights:
        return q, frac
    light = q < one
    L = np.nonzero(light)[0]
    H = np.nonzero(~light)[0]
    nl, nh = L.size, H.size
    D = np.concatenate([np.zeros(1, np.uint64), np.cumsum(one - q[L], dtype=np.uint64)])  # D(0..nl)
    hexc = q[H] - one
    E = np.concatenate([np.zeros(1, np.uint64), np.cumsum(hexc, dtype=np.uint64)])[:nh]
    Einc = E + hexc

    def thr(p):
        t = np.minimum(p >> np.uint64(frac - 32), np.uint64(0xfffffffe))
        return np.where(p >= one, np.uint64(0xffffffff), t)

    table = np.zeros((n, 2), np.uint64)
    b = np.searchsorted(Einc, D[:nl], side="left")  # first heavy with E(b + 1) >= D(a)
    ok = b < nh
    table[L, 0] = np.where(ok, thr(q[L]), np.uint64(0xffffffff))
    table[L, 1] = np.where(ok, H[np.minimum(b, max(nh - 1, 0))] if nh else L, L)
    a = np.searchsorted(D, Einc, side="right")  # first a in [0, nl] with D(a) > E(b + 1)
    conv = (a <= nl) & (np.arange(nh) + 1 < nh)
    keep = one + hexc + E - D[np.minimum(a, nl)]
    table[H, 0] = np.where(conv, thr(np.where(conv, keep, one)), np.uint64(0xffffffff))
    table[H, 1] = np.where(conv, H[np.minimum(np.arange(nh) + 1, max(nh - 1, 0))], H)
    table = table.astype(np.uint32)
    k32 = np.where(table[:, 0] == 0xFFFFFFFF, np.uint64(1 << 32), table[:, 0].astype(np.uint64))
    mass = k32.copy()
    part = k32 < np.uint64(1 << 32)
    np.add.at(mass, table[part, 1].astype(np.int64), np.uint64(1 << 32) - k32[part])
    pdf = (mass.astype(np.float64) / 4294967296.0 * (1.0 / (2.0 * 3.141592653589793 * 3.141592653589793))).astype(
        np.float32)
    return table, pdf


def camera_bytes(state: dict, width: int, height: int) -> bytes:
    """CameraStateStuct (structs.js:235-249) with dimsMask = W<<16 | H (camera_pass.js:118-125)."""
    dims = ((width & 0xFFFF) << 16) | (height & 0xFFFF)
    return struct.pack("<6fI5fI", *state["pos"], *state["dir"], dims, state["fov"], state["focalDepth"],
                       state["apertureSize"], state["distortion"], state["bokeh"], state["invocationOffset"])


class Renderer:
    """The per-frame passes and RenderState of pike.js, restated on the CPU."""

    def __init__(self, width: int, height: int, batch: int | None = None, threads: int | None = None):
        L = lib()
        self.w, self.h = width, height
        self.batch = batch if batch is not None else width * height
        self.threads = threads if threads is not None else (os.cpu_count() or 1)
        self.h_ = L.or_renderer_new(C.c_uint32(width), C.c_uint32(height), C.c_uint32(self.batch), C.c_int(self.threads))
        self.p = C.c_void_p(self.h_)

    def __del__(self):
        if getattr(self, "h_", None):
            lib().or_renderer_free(self.p)
            self.h_ = None

    def set_scene(self, bvh: BVH, attrs: np.ndarray, mat_index: np.ndarray, layers: np.ndarray):
        self._keep = [np.ascontiguousarray(bvh.nodes, np.int32), np.ascontiguousarray(bvh.tris, np.int32),
                      np.ascontiguousarray(bvh.verts, np.float32), np.ascontiguousarray(attrs, np.uint32),
                      np.ascontiguousarray(mat_index, np.int32), np.ascontiguousarray(layers, np.uint8)]
        n, t, v, a, m, l = self._keep
        lib().or_set_scene(self.p, _p(n), C.c_size_t(n.shape[0]), _p(t), C.c_size_t(t.shape[0]), _p(v),
                           C.c_size_t(v.shape[0]), _p(a), _p(m), C.c_size_t(m.shape[0]), _p(l), C.c_size_t(l.shape[0]))

    def set_atlas(self, layers: np.ndarray):
        """(n, res, res, 4) uint8 atlas layers in place of the 1x1 colour layers."""
        self._atlas = np.ascontiguousarray(layers, np.uint8)
        n, res = self._atlas.shape[0], self._atlas.shape[1]
        lib().or_set_atlas(self.p, _p(self._atlas), C.c_uint32(res), C.c_size_t(n))

    def set_env(self, env: Env):
        lib().or_set_env(self.p, _p(env.rgbe), C.c_uint32(env.w), C.c_uint32(env.h), _p(env.bins),
                         C.c_size_t(env.bins.shape[0]), _p(env.coords), _p(env.pdf))

    def set_camera(self, state: dict):
        self._cam = C.create_string_buffer(camera_bytes(state, self.w, self.h))
        lib().or_set_camera(self.p, self._cam)

    def set_render_state(self, samples: int, env_theta: float = 0.0):
        lib().or_set_render_state(self.p, samples, env_theta)

    def set_post(self, exposure: float = 1.0, saturation: float = 1.0):
        lib().or_set_post(self.p, exposure, saturation)

    def __getattr__(self, name):
        if name in ("begin_frame", "camera", "trace", "shade_hit", "trace_shadow", "shade_miss", "accumulate",
                    "postprocess", "reset_stats", "clear_color", "clear_hits_misses", "clear_rays"):
            fn = getattr(lib(), "or_" + name)
            return lambda: fn(self.p)
        raise AttributeError(name)

    def tick(self, bounces: int):
        """pike.js tick(): every pixel batch of the frame."""
        lib().or_tick(self.p, bounces)

    def tick_batch(self, bounces: int):
        """One batch of tick() at the camera's own invocationOffset."""
        lib().or_tick_batch(self.p, bounces)

    def counters(self):
        c = np.zeros(6, np.uint32)
        lib().or_counters(self.p, _p(c))
        return dict(samples=int(c[0]), num_hits=int(c[1]), num_misses=int(c[2]), num_rays=int(c[3]),
                    num_shadow=int(c[4]), overflow=int(c[5]))

    def shadow_offset(self) -> int:
        return int(lib().or_shadow_offset(self.p))

    def rays(self, first: int, count: int) -> np.ndarray:
        out = np.zeros((count, 12), np.float32)
        lib().or_read_rays(self.p, C.c_size_t(first), C.c_size_t(count), _p(out))
        return out

    def misses(self, count: int) -> np.ndarray:
        out = np.zeros((count, 12), np.float32)
        lib().or_read_misses(self.p, C.c_size_t(count), _p(out))
        return out

    def hits(self, count: int) -> np.ndarray:
        out = np.zeros((count, 16), np.uint32)
        lib().or_read_hits(self.p, C.c_size_t(count), _p(out))
        return out

    def color(self) -> np.ndarray:
        out = np.zeros((self.h, self.w, 4), np.float32)
        lib().or_read_color(self.p, _p(out))
        return out

    def accum(self) -> np.ndarray:
        out = np.zeros((self.h, self.w, 4), np.float32)
        lib().or_read_accum(self.p, _p(out))
        return out

    def display(self):
        out = np.zeros((self.h, self.w, 4), np.float32)
        out8 = np.zeros((self.h, self.w, 4), np.uint8)
        lib().or_read_display(self.p, _p(out), _p(out8))
        return out, out8

    def stats(self) -> dict:
        s = np.zeros(8, np.uint64)
        lib().or_stats(self.p, _p(s))
        return dict(trace_fetch=int(s[0]), trace_tests=int(s[1]), trace_rays=int(s[2]), trace_max_stack=int(s[3]),
                    shadow_fetch=int(s[4]), shadow_tests=int(s[5]), shadow_rays=int(s[6]), shadow_max_stack=int(s[7]))

    def trace_rays(self, rays8: np.ndarray, any_hit: bool = False) -> np.ndarray:
        rays8 = np.ascontiguousarray(rays8, np.float32)
        out = np.zeros((rays8.shape[0], 4), np.uint32)
        lib().or_trace_rays(self.p, _p(rays8), C.c_size_t(rays8.shape[0]), C.c_int(1 if any_hit else 0), _p(out))
        return out

    def _diff_args(self, W, H, albedo, rough, metal, env, tables, spp, depth, sample_base, rough0):
        rough0 = rough if rough0 is None else rough0
        self._dkeep = [np.ascontiguousarray(albedo, np.float64), np.ascontiguousarray(rough, np.float64),
                       np.ascontiguousarray(rough0, np.float64), np.ascontiguousarray(metal, np.float64),
                       np.ascontiguousarray(env, np.float64), tables]
        a, r, r0, m, e, _ = self._dkeep
        assert (e.shape[1], e.shape[0]) == (tables.w, tables.h)
        return [self.p, C.c_uint32(W), C.c_uint32(H), _p(a), _p(r), _p(r0), _p(m), C.c_uint32(r.shape[0]), _p(e),
                C.c_uint32(e.shape[1]), C.c_uint32(e.shape[0]), C.c_void_p(tables._h), C.c_uint32(spp),
                C.c_uint32(depth), C.c_uint32(sample_base)]

    def diff_render(self, W, H, albedo, rough, metal, env, tables, spp, depth, sample_base=0, rough0=None):
        """FP64 oracle of pk_diff_render (camera and env rotation: set_camera,
        set_render_state): (H, W, 3) image and the rays traced."""
        img = np.zeros((H, W, 3), np.float64)
        L = lib()
        L.or_diff_render.restype = C.c_uint64
        rays = L.or_diff_render(*self._diff_args(W, H, albedo, rough, metal, env, tables, spp, depth, sample_base,
                                                 rough0), _p(img))
        return img, int(rays)

    def diff_render32(self, W, H, albedo, rough, metal, env, tables, spp, depth, sample_base=0, rough0=None,
                      rows=None, trace_pixel: int = -1):
        """pk_diff_render's binary32 arithmetic replayed on the CPU: rows
        (y0, y1) of the (H, W, 4) float32 image, and the rays traced."""
        y0, y1 = rows if rows is not None else (0, H)
        img = np.zeros((y1 - y0, W, 4), np.float32)
        L = lib()
        L.or_diff_render32.restype = C.c_uint64
        rays = L.or_diff_render32(*self._diff_args(W, H, albedo, rough, metal, env, tables, spp, depth, sample_base,
                                                   rough0), C.c_uint32(y0), C.c_uint32(y1), _p(img),
                                  C.c_int64(trace_pixel))
        return img, int(rays)

    def diff_grad(self, W, H, albedo, rough, metal, env, tables, spp, depth, dimage, sample_base=0, rough0=None):
        """FP64 oracle of pk_diff_backward for dLoss/dimage = dimage (H, W, 3)."""
        d = np.ascontiguousarray(dimage, np.float64)
        ga = np.zeros((np.asarray(albedo).shape[0], 3))
        gr = np.zeros(np.asarray(rough).shape[0])
        ge = np.zeros(np.asarray(env).shape)
        lib().or_diff_grad(*self._diff_args(W, H, albedo, rough, metal, env, tables, spp, depth, sample_base, rough0),
                           _p(d), _p(ga), _p(gr), _p(ge))
        return ga, gr, ge

    def set_track64(self, on: bool = True, share_texels: bool = False):
        """FP64 companion: every ray also carries an FP64 throughput and every
        contribution is recomputed in FP64 along the same paths (om_render64.h).
        share_texels: the two nearest-texel lookups (the env pdf texel of the
        bounce MIS weight, the env texel of a miss) use the FP32 evaluation's
        texel indices, isolating the arithmetic error from texel flips."""
        lib().or_set_track64(self.p, C.c_int((2 if share_texels else 1) if on else 0))

    def _read64(self, which: int) -> np.ndarray:
        out = np.zeros((self.h, self.w, 4), np.float64)
        if lib().or_read64(self.p, C.c_int(which), _p(out)):
            raise RuntimeError("FP64 companion is off")
        return out

    def accum64(self) -> np.ndarray:
        """accumulate.wgsl's running mean of the FP64 per-frame colours."""
        return self._read64(0)

    def std64(self) -> np.ndarray:
        """Per-pixel sample standard deviation of the FP64 per-frame colours."""
        n = int(lib().or_frames64(self.p))
        return np.sqrt(self._read64(2) / max(n - 1, 1))

    def frames64(self) -> int:
        return int(lib().or_frames64(self.p))

    def env_roundtrip(self, cx: int, cy: int):
        """sampleEnv's direction for texel (cx, cy) and envPdf's texel index of it."""
        d = np.zeros(3, np.float32)
        i = np.zeros(2, np.int32)
        lib().or_env_roundtrip(self.p, C.c_int32(cx), C.c_int32(cy), _p(d), _p(i))
        return d, (int(i[0]), int(i[1]))

    def set_env_alias(self, table2: np.ndarray, pdf: np.ndarray):
        """Sample the environment from an alias table (the library's
        PK_ENV_ALIAS) with its pdf texture in place of the histogram's."""
        t = np.ascontiguousarray(table2, np.uint32)
        p = np.ascontiguousarray(pdf, np.float32)
        lib().or_set_env_alias(self.p, _p(t), _p(p), C.c_size_t(p.size))

    def render64(self) -> "Render64":
        """An independent binary64 renderer (om_render_f64.h) of this
        renderer's scene, environment, camera and current sample index."""
        return Render64(self)

    def set_canonical(self, on: bool = True):
        """Trace by testing every triangle (min (t, slot)): the 8-wide traversal's answer."""
        lib().or_set_canonical(self.p, C.c_int(1 if on else 0))

    def brute_rays(self, rays8: np.ndarray, any_hit: bool = False) -> np.ndarray:
        """Every triangle tested: closest = min (t, slot); the order-independent answer."""
        rays8 = np.ascontiguousarray(rays8, np.float32)
        out = np.zeros((rays8.shape[0], 4), np.uint32)
        lib().or_brute_rays(self.p, _p(rays8), C.c_size_t(rays8.shape[0]), C.c_int(1 if any_hit else 0), _p(out))
        return out


MATH_FN = {"sin": 0, "cos": 1, "tan": 2, "atan2": 3, "acos": 4, "exp2": 5, "log2": 6, "pow": 7, "snorm16": 8}


def math_fn(name: str, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    yp = _p(np.ascontiguousarray(y, np.float32)) if y is not None else None
    if y is not None:
        y = np.ascontiguousarray(y, np.float32)
        yp = _p(y)
    lib().or_math(C.c_int(MATH_FN[name]), _p(x), yp, _p(out), C.c_size_t(x.size))
    return out


def hash_stream(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().or_hash_stream(C.c_uint32(seed), _p(out), C.c_size_t(n))
    return out


class Prepared:
    """Everything the oracle renderer needs for one synthetic scene."""

    def __init__(self, src, threads: int | None = None, batch: int | None = None):
        self.src = src
        self.pos, self.attrs = flatten(src)
        self.mat_index, self.layers = materials(src.materials)
        self.bvh = BVH(self.pos, src.tris)
        self.env = Env(src.env_rgbe)
        self.r = Renderer(src.width, src.height, batch=batch, threads=threads)
        self.r.set_scene(self.bvh, self.attrs, self.mat_index, self.layers)
        self.r.set_env(self.env)
        self.r.set_camera(src.camera_state())


class Render64:
    """The reference path rendered in binary64 end to end (om_render_f64.h):
    its own rays, hits, queues and branches from the same hash streams."""

    def __init__(self, r: "Renderer"):
        self.w, self.h = r.w, r.h
        self.p = lib().or_render64_new(r.p)

    def __del__(self):
        if getattr(self, "p", None):
            lib().or_render64_free(self.p)
            self.p = None

    def tick(self, bounces: int):
        lib().or_render64_tick(self.p, C.c_uint32(bounces))

    def frames(self) -> int:
        return int(lib().or_render64_frames(self.p))

    def _read(self, which: int) -> np.ndarray:
        out = np.zeros((self.h, self.w, 4), np.float64)
        lib().or_render64_read(self.p, C.c_int(which), _p(out))
        return out

    def accum(self) -> np.ndarray:
        """accumulate.wgsl's running mean in double."""
        return self._read(0)

    def std(self) -> np.ndarray:
        """Per-pixel sample standard deviation of the per-frame colours."""
        return np.sqrt(self._read(2) / max(self.frames() - 1, 1))

    def color(self) -> np.ndarray:
        """The last frame's colour buffer (before accumulation)."""
        return self._read(3)
