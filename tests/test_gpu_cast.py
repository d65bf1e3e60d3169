"""pk_cast_rays: ray queries on caller-owned device buffers, checked ray by
ray against the oracle's traversal (bit-exact t, triangle index, barycentrics)."""
import ctypes as C

import numpy as np
import pytest

from pike_gb300 import synth
from pike_gb300._lib import ptr

from helpers import Pair

pytestmark = pytest.mark.gpu


def query_rays(src, n, seed):
    """Rays from random points inside the scene's normalised frame in random directions."""
    rng = np.random.default_rng(seed)
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = rng.uniform(-0.9, 0.9, (n, 3))
    v = rng.normal(size=(n, 3))
    d[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return o, d


def cast(ctx, o, d, any_hit):
    torch = pytest.importorskip("torch")
    n = o.shape[0]
    to, td = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    hits = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    idx = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.call("pk_cast_rays", C.c_void_p(to.data_ptr()), C.c_void_p(td.data_ptr()), n, 1 if any_hit else 0,
             C.c_void_p(hits.data_ptr()), C.c_void_p(idx.data_ptr()), C.c_void_p(cnt.data_ptr()))
    k = int(cnt.item())
    return hits.cpu().numpy().view(np.uint32), idx[:k].cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("any_hit", [False, True])
def test_cast_rays_match_oracle(oracle, pk_built, any_hit):
    src = synth.displaced_sphere_scene(subdivisions=6, width=16, height=16, env_size=(64, 32))
    pair = Pair(src, oracle)
    o, d = query_rays(src, 100_000, 5)
    hits, idx = cast(pair.ctx, o, d, any_hit)
    rays8 = np.concatenate([o, d], axis=1)
    ref = pair.P.r.trace_rays(rays8, any_hit=any_hit)
    hit = ref[:, 1] != 0xFFFFFFFF
    assert np.array_equal(hits[:, 1], ref[:, 1])
    if not any_hit:
        assert np.array_equal(hits[hit, 0], ref[hit, 0]) and np.array_equal(hits[hit, 2], ref[hit, 2])
    assert np.array_equal(idx, np.flatnonzero(hit).astype(np.uint32))


def test_cast_rays_empty_and_tiny(oracle, pk_built):
    src = synth.small_scene(width=8, height=8)
    pair = Pair(src, oracle)
    for n in (1, 31, 33):
        o, d = query_rays(src, n, n)
        hits, idx = cast(pair.ctx, o, d, False)
        ref = pair.P.r.trace_rays(np.concatenate([o, d], axis=1))
        assert np.array_equal(hits[:, 1], ref[:, 1])
        assert np.array_equal(idx, np.flatnonzero(ref[:, 1] != 0xFFFFFFFF).astype(np.uint32))


def test_focus_distance_matches_raycaster(oracle, pk_built):
    """pk_focus_distance (double-precision autofocus cast) equals the oracle's
    Raycaster.cast restatement bit for bit, and focalDepth = 1 - 1/t."""
    src = synth.displaced_sphere_scene(subdivisions=5, width=16, height=16, env_size=(64, 32))
    pair = Pair(src, oracle)
    rng = np.random.default_rng(9)
    rays = np.zeros((64, 6))
    rays[:, :3] = rng.uniform(-0.9, 0.9, (64, 3))
    v = rng.normal(size=(64, 3))
    rays[:, 3:] = v / np.linalg.norm(v, axis=1, keepdims=True)
    st = src.camera_state()
    rays[0] = [*st["pos"], *st["dir"]]
    want = pair.P.bvh.cast(rays)
    for i in range(rays.shape[0]):
        o = (C.c_double * 3)(*rays[i, :3])
        d = (C.c_double * 3)(*rays[i, 3:])
        t, fd = C.c_double(0.0), C.c_double(0.0)
        pair.ctx.call("pk_focus_distance", o, d, C.byref(t), C.byref(fd))
        assert np.float64(t.value).view(np.uint64) == np.float64(want[i]).view(np.uint64), i
        assert fd.value == 1.0 - 1.0 / t.value
    assert (want < 1e6).any() and (want == 1e6).any()


@pytest.mark.parametrize("mode_name", ["PK_TRACE_EXACT", "PK_TRACE_WIDE", "PK_TRACE_COMPACT_RECORDS"])
def test_cast_rays_ignore_the_trace_mode(oracle, pk_built, mode_name):
    """Ray queries traverse the drop-in's records whatever the context's trace
    mode selects for the render passes: after switching the mode (which builds
    the outward-rounded binary records or the 8-wide BVH) the hits still equal
    the oracle's trace.wgsl / trace_shadow.wgsl answers bit for bit."""
    from pike_gb300 import _lib
    src = synth.displaced_sphere_scene(subdivisions=5, width=16, height=16, env_size=(64, 32))
    pair = Pair(src, oracle)
    pair.ctx.call("pk_set_trace_mode", _lib.PK_TRACE_PERSISTENT | getattr(_lib, mode_name))
    o, d = query_rays(src, 50_000, 21)
    rays8 = np.concatenate([o, d], axis=1)
    for any_hit in (False, True):
        hits, idx = cast(pair.ctx, o, d, any_hit)
        ref = pair.P.r.trace_rays(rays8, any_hit=any_hit)
        hit = ref[:, 1] != 0xFFFFFFFF
        assert np.array_equal(hits[:, 1], ref[:, 1])
        assert np.array_equal(hits[hit, 0], ref[hit, 0])
        assert np.array_equal(idx, np.flatnonzero(hit).astype(np.uint32))
