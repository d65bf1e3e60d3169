"""Form (2): one persistent launch over many requests and resident scenes.
Images agree with the drop-in's in distribution (the hit RNG seeds differ by
construction), duplicate requests agree to rounding, every supported launch
configuration gives the same image, and bad requests are rejected."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import PikeError, ptr
from pike_gb300.batch import Batch, Request, orbit_camera, random_requests, scene_context

from helpers import camera_struct

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(pk_built):
    a = synth.small_scene()
    b = synth.displaced_sphere_scene(subdivisions=5, width=16, height=16, env_size=(256, 128))
    return [a, b], [scene_context(a), scene_context(b)]


def plain_mean(ctx, src_cam: dict, w: int, h: int, spp: int, depth: int) -> np.ndarray:
    ctx.call("pk_configure", w, h, w * h)
    ctx.call("pk_set_camera", camera_struct(src_cam))
    ctx.call("pk_set_render_state", 0, 0.0)
    ctx.call("pk_render_frames", spp, depth)
    out = np.zeros((h, w, 4), np.float32)
    ctx.call("pk_read_accum", ptr(out))
    return out


def block_means(img: np.ndarray, k: int = 8) -> np.ndarray:
    h, w = img.shape[0] // k * k, img.shape[1] // k * k
    return img[:h, :w, :3].reshape(h // k, k, w // k, k, 3).mean(axis=(1, 3))


def test_batch_matches_dropin_in_distribution(scenes):
    srcs, ctxs = scenes
    cam = srcs[0].camera_state()
    req = Request(scene=0, width=64, height=48, spp=128, depth=4, camera=cam)
    batch = Batch(ctxs)
    batch.set_requests([req])
    batch.render(1)
    got = batch.image(0)
    want = plain_mean(ctxs[0], cam, 64, 48, 128, 4)
    assert np.isfinite(got).all() and got[..., :3].mean() > 0.05
    assert abs(got[..., :3].mean() / want[..., :3].mean() - 1.0) < 0.01
    bg, bw = block_means(got), block_means(want)
    assert np.abs(bg - bw).max() < 0.05 * bw.max()


def test_duplicate_requests_agree_and_shapes(scenes):
    srcs, ctxs = scenes
    rng = np.random.default_rng(5)
    cam = orbit_camera(rng)
    reqs = [Request(1, 96, 64, 4, 6, cam), Request(0, 40, 30, 16, 4, srcs[0].camera_state()),
            Request(1, 96, 64, 4, 6, cam)]
    batch = Batch(ctxs)
    batch.set_requests(reqs)
    batch.render(2)
    a, b, c = batch.image(0), batch.image(1), batch.image(2)
    assert a.shape == (64, 96, 4) and b.shape == (30, 40, 4)
    assert np.allclose(a, c, rtol=1e-5, atol=1e-6)  # same paths; only the summation order may differ
    n, frames, ms = batch.info()
    assert n == 96 * 64 * 4 * 2 + 40 * 30 * 16 and frames == 2 and ms > 0
    lat = batch.latencies()  # of the last frame
    assert (lat > 0).all() and (lat <= ms).all()


def test_configurations_agree(scenes):
    srcs, ctxs = scenes
    reqs = random_requests(6, 2, seed=9)
    for r in reqs:  # keep the test small
        r.width, r.height, r.spp = max(16, r.width // 8), max(16, r.height // 8), min(r.spp, 4)
    batch = Batch(ctxs)
    batch.set_requests(reqs)
    ref = None
    for cfg in [(64, 16, 1), (128, 32, 4), (256, 32, 16), (256, 16, 64), (128, 8, 4)]:
        batch.set_config(*cfg)
        batch.reset()
        batch.render(1)
        imgs = [batch.image(i) for i in range(len(reqs))]
        if ref is None:
            ref = imgs
        for x, y in zip(imgs, ref):
            assert np.allclose(x, y, rtol=1e-5, atol=1e-6), cfg
    best = batch.autotune(0)
    assert best > 0 and batch.config() in {(b, s, c) for b in (64, 128, 256) for s in (8, 16, 32) for c in (1, 4, 16)}


def test_bad_requests_are_rejected(scenes):
    srcs, ctxs = scenes
    batch = Batch(ctxs)
    cam = srcs[0].camera_state()
    for bad in (Request(2, 16, 16, 1, 4, cam), Request(0, 0, 16, 1, 4, cam), Request(0, 16, 16, 0, 4, cam),
                Request(0, 16, 16, 1, 0, cam), Request(0, 16, 16, 1, 17, cam)):
        with pytest.raises(PikeError) as e:
            batch.set_requests([bad])
        assert e.value.code == _lib.PK_ERR_ARG
    with pytest.raises(PikeError):
        batch.set_config(96, 16, 4)
    with pytest.raises(PikeError) as e:
        batch.render(1)  # no requests yet
    assert e.value.code == _lib.PK_ERR_STATE


def test_batch_pixel_exact_where_seeds_coincide(scenes):
    """One sample of depth 1: the batch and the drop-in trace the same camera
    rays (seeded by pixel and sample) to the same closest hits.  Shading seeds
    differ by construction (the batch uses the bounce index, the drop-in the
    hit-queue slot), except for the first hit of the queue (slot 0 = bounce
    0).  So every pixel whose camera ray misses, and the pixel of hit slot 0,
    must be bit-exact between the two."""
    srcs, ctxs = scenes
    src, ctx = srcs[0], ctxs[0]  # ground and boxes under the sky: some camera rays miss
    W, H = 64, 48
    cam = src.camera_state()
    batch = Batch(ctxs)
    batch.set_requests([Request(scene=0, width=W, height=H, spp=1, depth=1, camera=cam)])
    batch.render(1)
    got = batch.image(0)
    want = plain_mean(ctx, cam, W, H, 1, 1)
    # which camera rays hit: the pass path's first trace, in queue order
    ctx.call("pk_set_render_state", 0, 0.0)
    for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera", "trace"):
        ctx.call("pk_" + name)
    cnt = np.zeros(8, np.uint32)
    ctx.call("pk_read_counters", ptr(cnt))
    n_hits = int(cnt[1])  # {samples, num_hits, ...}
    hits = np.zeros((n_hits, 16), np.uint32)
    ctx.call("pk_read_hits", 0, n_hits, ptr(hits))
    hit_pix = hits[:, 15] & 0x0FFFFFFF  # the pixel index in the ray's tp.w
    assert 0 < n_hits < W * H
    miss = np.ones(W * H, bool)
    miss[hit_pix] = False
    g, w = got.reshape(-1, 4)[:, :3], want.reshape(-1, 4)[:, :3]
    assert np.array_equal(g[miss].view(np.uint32), w[miss].view(np.uint32)), "pixels whose camera ray misses"
    first = int(hit_pix[0])
    assert np.array_equal(g[first].view(np.uint32), w[first].view(np.uint32)), "the pixel of hit slot 0"
