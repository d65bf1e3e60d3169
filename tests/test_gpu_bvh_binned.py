"""PK_BVH_BINNED: the binned SAH build (not the reference's topology).  The
tree must hold every triangle once in leaves of at most 8, children after
parents, and trace to the same closest hits as brute force (checked through
the order-independent 8-wide traversal)."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import ptr

from helpers import Pair

pytestmark = pytest.mark.gpu


def download(ctx, n_verts):
    nn, nt = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    norm = np.zeros(4)
    ctx.call("pk_bvh_info", ptr(nn), ptr(nt), ptr(norm))
    nodes = np.zeros((int(nn[0]), 5), np.int32)
    tris = np.zeros((int(nt[0]), 4), np.int32)
    verts = np.zeros((n_verts, 4), np.float32)
    ctx.call("pk_bvh_download", ptr(nodes), ptr(tris), ptr(verts))
    return nodes, tris, verts, norm


@pytest.mark.parametrize("sub", [1, 6])
def test_binned_structure(oracle, pk_built, sub):
    src = synth.displaced_sphere_scene(subdivisions=sub, width=16, height=16, env_size=(64, 32))
    pair = Pair(src, oracle)
    c = pair.ctx
    c.call("pk_bvh_build", _lib.PK_BVH_BINNED)
    nodes, tris, verts, norm = download(c, src.pos.shape[0])
    T = src.tris.shape[0]
    assert tris.shape[0] == T
    # same multiset of triangles
    a = np.sort(tris.view(np.dtype((np.void, 16))).ravel())
    b = np.sort(np.ascontiguousarray(src.tris, np.int32).view(np.dtype((np.void, 16))).ravel())
    assert np.array_equal(a, b)
    seen = np.zeros(T, np.int64)
    reached = np.zeros(nodes.shape[0], np.int64)
    reached[0] = 1
    for i in range(nodes.shape[0]):
        if nodes[i, 1] > -1:
            size, base = nodes[i, 1] >> 24, nodes[i, 1] & 0xFFFFFF
            assert 1 <= size <= 8
            seen[base:base + size] += 1
        else:
            l = nodes[i, 0]
            assert l > i and l + 1 < nodes.shape[0]
            reached[l] += 1
            reached[l + 1] += 1
    assert (seen == 1).all() and (reached == 1).all()
    # the same normalisation as the reference build (root box of the same triangles)
    nn, nt = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    ref_norm = np.zeros(4)
    c2 = Pair(src, oracle).ctx
    c2.call("pk_bvh_info", ptr(nn), ptr(nt), ptr(ref_norm))
    assert np.array_equal(norm, ref_norm)


def test_binned_closest_hits_equal_bruteforce(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=6, width=96, height=64, env_size=(128, 64))
    pair = Pair(src, oracle, threads=16)
    c = pair.ctx
    c.call("pk_bvh_build", _lib.PK_BVH_BINNED)
    c.call("pk_set_trace_mode", _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE)
    _, gtris, _, _ = download(c, src.pos.shape[0])
    otris = pair.P.bvh.tris
    pair.set_render_state(0)
    for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
        c.call("pk_" + name)
    for bounce in range(2):
        n = pair.counters()["num_rays"]
        rays = pair.rays(_lib.PK_QUEUE_RAYS, 0, n)
        c.call("pk_clear_hits_misses")
        c.call("pk_trace")
        hits = pair.hits(pair.counters()["num_hits"])
        want = pair.P.r.brute_rays(np.ascontiguousarray(rays[:, :8]))
        hit = want[:, 1] != 0xFFFFFFFF
        assert hits.shape[0] == int(hit.sum())
        assert np.array_equal(hits[:, 0], want[hit, 0])  # t bits
        same = (gtris[hits[:, 1].astype(np.int64)] == otris[want[hit, 1].astype(np.int64)]).all(axis=1)
        assert same.mean() > 0.999  # only exact ties on t may pick another triangle
        for name in ("shade_hit", "trace_shadow", "shade_miss"):
            c.call("pk_" + name)


def test_binned_frames_render(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=6, width=128, height=96, env_size=(256, 128))
    pair = Pair(src, oracle)
    c = pair.ctx
    c.call("pk_set_render_state", 0, 0.0)
    c.call("pk_render_frames", 8, 4)
    sweep = pair.image("accum").copy()
    c.call("pk_bvh_build", _lib.PK_BVH_BINNED)
    c.call("pk_set_render_state", 0, 0.0)
    c.call("pk_render_frames", 8, 4)
    binned = pair.image("accum")
    assert pair.counters()["err"] == 0 and np.isfinite(binned).all()
    # different trees, same scene: images agree up to the reference's box truncation and noise
    assert abs(binned[..., :3].mean() / sweep[..., :3].mean() - 1.0) < 0.02
