"""The 8-wide compressed BVH (PK_TRACE_WIDE): closest hits equal the minimum
of (t, triangle slot) over every triangle the reference's test accepts, any
hits equal "some triangle accepted", so whole frames match the oracle run
with brute-force traversal bit for bit; against the drop-in traversal they
differ only where its inward-truncated boxes lose a hit or triangles tie."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import ptr

from helpers import Pair, assert_bits_equal

pytestmark = pytest.mark.gpu

WIDE = _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE
EXACT = _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_EXACT


def wide_pair(oracle, src, mode=WIDE, **kw) -> Pair:
    pair = Pair(src, oracle, **kw)
    pair.ctx.call("pk_set_trace_mode", mode)
    pair.P.r.set_canonical(True)
    return pair


def wide_nodes(ctx, n_tris):
    n, depth = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    ctx.call("pk_wide_info", ptr(n), ptr(depth))
    nodes = np.zeros((int(n[0]), 20), np.float32)
    tris = np.zeros((n_tris, 12), np.float32)
    ctx.call("pk_wide_download", ptr(nodes), ptr(tris))
    return nodes, tris, int(depth[0])


@pytest.mark.parametrize("make", [
    lambda: synth.displaced_sphere_scene(subdivisions=6, width=16, height=16, env_size=(64, 32)),
    lambda: synth.triangle_soup_scene(n_tris=60_000, width=16, height=16, env_size=(64, 32)),
    lambda: synth.small_scene(width=16, height=16),
], ids=["sphere6", "soup60k", "small"])
def test_gpu_builds_equal_host_restatement(oracle, pk_built, make):
    """The GPU builders of the 8-wide BVH and of the FP32 binary reference
    (pk_wide.cu) give the host restatement's records (oracle/om_wide.h) bit
    for bit: nodes, triangle records, depth, root code."""
    src = make()
    pair = Pair(src, oracle)
    ctx = pair.ctx
    n_nodes, n_tris = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    ctx.call("pk_bvh_info", ptr(n_nodes), ptr(n_tris), ptr(np.zeros(4)))
    nodes5 = np.zeros((int(n_nodes[0]), 5), np.int32)
    tri4 = np.zeros((int(n_tris[0]), 4), np.int32)
    verts = np.zeros_like(pair.P.bvh.verts)
    ctx.call("pk_bvh_download", ptr(nodes5), ptr(tri4), ptr(verts))
    ctx.call("pk_set_trace_mode", WIDE)
    nodes, tris, depth = wide_nodes(ctx, int(n_tris[0]))
    hn, ht, hd = oracle.wide_build(nodes5, tri4, verts)
    assert (nodes.shape, depth) == (hn.shape, hd)
    assert np.array_equal(nodes.view(np.uint32), hn.view(np.uint32))
    assert np.array_equal(tris.view(np.uint32), ht.view(np.uint32))
    ctx.call("pk_set_trace_mode", EXACT)
    rec, et, root = oracle.exact_build(nodes5, tri4, verts)
    grec = np.zeros_like(rec)
    gtris = np.zeros_like(et)
    groot = np.zeros(1, np.int32)
    ctx.call("pk_exact_download", ptr(grec), ptr(gtris), ptr(groot))
    assert int(groot[0]) == root
    assert np.array_equal(grec.view(np.uint32), rec.view(np.uint32))
    assert np.array_equal(gtris.view(np.uint32), et.view(np.uint32))


def test_trace_mode_rules(pk_built, oracle):
    src = synth.small_scene(width=8, height=8)
    pair = Pair(src, oracle)
    for bad in (_lib.PK_TRACE_WIDE | _lib.PK_TRACE_EXACT | 1, _lib.PK_TRACE_EXACT, 16):
        with pytest.raises(_lib.PikeError) as e:
            pair.ctx.call("pk_set_trace_mode", bad)
        assert e.value.code == _lib.PK_ERR_ARG


@pytest.mark.parametrize("make", [
    lambda: synth.displaced_sphere_scene(subdivisions=5, width=16, height=16, env_size=(64, 32)),
    lambda: synth.triangle_soup_scene(n_tris=20_000, width=16, height=16, env_size=(64, 32)),
], ids=["sphere5", "soup20k"])
def test_wide_structure(oracle, pk_built, make):
    """Compressed wide nodes (pk_wide.h): internal children come after their
    parent, contiguous from child_base in slot order, and every node but the
    root is referenced once; leaf children hold 1-3 triangle records at
    tri_base + offset, every record is referenced once and the records carry
    every binary slot once, with that slot's vertices; every decoded leaf
    child box contains its triangles' vertices (outward rounding)."""
    src = make()
    pair = wide_pair(oracle, src)
    n_tris = src.tris.shape[0]
    nodes, tris, depth = wide_nodes(pair.ctx, n_tris)
    words = nodes.view(np.uint32)
    meta = np.ascontiguousarray(nodes[:, 6:8]).view(np.uint8)
    q = np.ascontiguousarray(nodes[:, 8:20]).view(np.uint8).reshape(-1, 6, 8)  # qlo xyz, qhi xyz
    seen = np.zeros(n_tris, np.int64)
    referenced = np.zeros(nodes.shape[0], np.int64)
    verts = tris[:, :9].reshape(-1, 3, 3)
    for i in range(nodes.shape[0]):
        imask = words[i, 3] >> 24
        child_base, tri_base = int(words[i, 4]), int(words[i, 5])
        p = nodes[i, :3].astype(np.float64)
        e = np.array([(words[i, 3] >> (8 * a)) & 0xFF for a in range(3)], np.int64) - 127
        s = np.ldexp(1.0, e)
        rank = 0
        for k in range(8):
            m = int(meta[i, k])
            if (imask >> k) & 1:
                assert m == 0x20 | k
                c = child_base + rank
                rank += 1
                assert c > i
                referenced[c] += 1
                continue
            if m == 0:
                continue
            count = {1: 1, 3: 2, 7: 3}[m >> 5]
            off = m & 31
            assert off + count <= 24
            r0 = tri_base + off
            seen[r0:r0 + count] += 1
            lo = (p + s * q[i, 0:3, k]).astype(np.float32)
            hi = (p + s * q[i, 3:6, k]).astype(np.float32)
            v = verts[r0:r0 + count].reshape(-1, 3)
            assert (v >= lo).all() and (v <= hi).all(), f"node {i} slot {k}: box does not contain its triangles"
    assert (seen == 1).all()
    assert referenced[0] == 0 and (referenced[1:] == 1).all()
    slots = tris[:, 9].view(np.uint32)
    assert np.array_equal(np.sort(slots), np.arange(n_tris, dtype=np.uint32))
    # each record holds its binary slot's vertices
    tri4 = pair.P.bvh.tris.reshape(-1, 4)
    bverts = pair.P.bvh.verts.reshape(-1, 4)[:, :3]
    want = bverts[tri4[slots, :3]].reshape(-1, 9)
    assert np.array_equal(tris[:, :9].view(np.uint32), want.astype(np.float32).view(np.uint32))
    assert 2 <= depth <= 16


@pytest.mark.parametrize("mode", [WIDE, EXACT], ids=["wide", "exact-binary"])
@pytest.mark.parametrize("make", [
    lambda: synth.small_scene(width=64, height=48),
    lambda: synth.displaced_sphere_scene(subdivisions=4, width=64, height=40, env_size=(128, 64)),
])
def test_wide_frames_match_bruteforce_oracle(oracle, pk_built, make, mode):
    src = make()
    pair = wide_pair(oracle, src, mode=mode, threads=16)
    pair.ctx.call("pk_set_render_state", 0, 0.0)
    pair.ctx.call("pk_render_frames", 2, 4)
    pair.ctx.call("pk_sync")
    P = pair.P.r
    P.set_render_state(0)
    for _ in range(2):
        P.tick(4)
    assert_bits_equal(pair.image("accum"), P.accum(), "wide traversal vs brute-force oracle")
    assert pair.counters()["err"] == 0


@pytest.mark.parametrize("mode", [WIDE, EXACT], ids=["wide", "exact-binary"])
def test_wide_pass_hits_match_bruteforce(oracle, pk_built, mode):
    """Camera and two bounces of rays through the pass path: every closest hit
    (slot, t, barycentrics) equals the brute-force answer."""
    src = synth.displaced_sphere_scene(subdivisions=6, width=120, height=80, env_size=(128, 64))
    pair = wide_pair(oracle, src, mode=mode, threads=16)
    c, P = pair.ctx, pair.P.r
    pair.set_render_state(0)
    for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
        c.call("pk_" + name)
    for bounce in range(3):
        n = pair.counters()["num_rays"]
        rays = pair.rays(_lib.PK_QUEUE_RAYS, 0, n)
        c.call("pk_trace")
        hits = pair.hits(pair.counters()["num_hits"])
        want = P.brute_rays(np.ascontiguousarray(rays[:, :8]))
        hit = want[:, 1] != 0xFFFFFFFF
        assert hits.shape[0] == int(hit.sum()), f"bounce {bounce}: hit count"
        # the hit list is in ray order; hit records carry {t, slot, bary}
        assert np.array_equal(hits[:, 1], want[hit, 1]), f"bounce {bounce}: slots"
        assert np.array_equal(hits[:, 0], want[hit, 0]), f"bounce {bounce}: t"
        assert np.array_equal(hits[:, 2], want[hit, 2]), f"bounce {bounce}: barycentrics"
        for name in ("shade_hit", "trace_shadow", "shade_miss"):
            c.call("pk_" + name)


def brute_rows(pair, rays: np.ndarray) -> np.ndarray:
    """The oracle's brute-force answers in per_ray's layout (a miss as {0,
    0xffffffff, 0}; the oracle reports a miss with t = MAX_T)."""
    want = pair.P.r.brute_rays(np.ascontiguousarray(rays[:, :8]))[:, :3].copy()
    want[want[:, 1] == 0xFFFFFFFF] = [0, 0xFFFFFFFF, 0]
    return want


def per_ray(hits: np.ndarray, rays: np.ndarray) -> np.ndarray:
    """Hit records -> (n, 3) {t, slot, bary} per queue ray (slot 0xffffffff: miss).
    Records carry their ray, whose 12 words identify it in the queue."""
    index = {rays[i].tobytes(): i for i in range(rays.shape[0])}
    out = np.zeros((rays.shape[0], 3), np.uint32)
    out[:, 1] = 0xFFFFFFFF
    for h in hits:
        out[index[h[4:16].view(np.float32).tobytes()]] = h[:3]
    return out


def test_wide_vs_dropin_agreement(oracle, pk_built):
    """Closest-hit triangle ids of the drop-in traversal (Moller-Trumbore on
    the reference's snorm16 boxes) agree with the wide one (watertight test)
    except on rays where the drop-in's inward-truncated boxes lose a hit, a
    tie on t resolves differently or the two triangle tests disagree at an
    edge; on every differing ray the wide answer (slot, t, barycentrics)
    equals brute force, and such rays are rare.  t and barycentrics come from
    different triangle tests, so only the triangle id is compared."""
    src = synth.displaced_sphere_scene(subdivisions=7, width=320, height=180, env_size=(256, 128))
    pair = Pair(src, oracle)
    c = pair.ctx
    pair.set_render_state(0)
    for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
        c.call("pk_" + name)
    total = differ = 0
    for bounce in range(3):
        n = pair.counters()["num_rays"]
        rays = pair.rays(_lib.PK_QUEUE_RAYS, 0, n)
        res = []
        for mode in (_lib.PK_TRACE_PERSISTENT, WIDE):
            c.call("pk_set_trace_mode", mode)
            c.call("pk_clear_hits_misses")
            c.call("pk_trace")
            res.append(per_ray(pair.hits(pair.counters()["num_hits"]), rays))
        plain, wide = res
        bad = np.flatnonzero(plain[:, 1] != wide[:, 1])
        total += n
        differ += bad.size
        if bad.size:
            assert np.array_equal(wide[bad], brute_rows(pair, rays[bad])), f"bounce {bounce}: wide differs from brute force"
        # a sample of all rays, not only the differing ones: the wide answer is brute force
        pick = np.random.default_rng(bounce).choice(n, size=min(n, 3000), replace=False)
        assert np.array_equal(wide[pick], brute_rows(pair, rays[pick])), f"bounce {bounce}: wide differs from brute force"
        for name in ("shade_hit", "trace_shadow", "shade_miss"):
            c.call("pk_" + name)
    assert total > 100_000
    assert differ <= total // 10_000, f"{differ} of {total} rays differ"
