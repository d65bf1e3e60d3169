"""Textured materials: bilinear textureSampleLevel on res x res atlas layers
(shade_hit.wgsl:184-197 with the linear/repeat sampler of shade_hit_pass.js:83-90),
GPU against the oracle, bit for bit."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import ptr

from helpers import Pair, assert_bits_equal

pytestmark = pytest.mark.gpu


def random_atlas(n_layers: int, res: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(0, 256, size=(n_layers, res, res, 4), dtype=np.uint8)


def textured_pair(oracle, src, res: int, seed: int, mode=_lib.PK_TRACE_PERSISTENT) -> Pair:
    pair = Pair(src, oracle, trace_mode=mode)
    n_layers = int(pair.P.layers.shape[0])
    atlas = random_atlas(n_layers, res, seed)
    pair.ctx.call("pk_atlas_upload", ptr(atlas), res, n_layers)
    pair.P.r.set_atlas(atlas)
    return pair


@pytest.mark.parametrize("res", [2, 17, 64])
def test_textured_small_scene_matches_oracle(oracle, pk_built, res):
    src = synth.small_scene(width=128, height=128)
    pair = textured_pair(oracle, src, res, seed=res)
    pair.ctx.call("pk_set_render_state", 0, 0.0)
    pair.ctx.call("pk_render_frames", 2, 4)
    pair.ctx.call("pk_sync")
    pair.P.r.set_render_state(0)
    for _ in range(2):
        pair.P.r.tick(4)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), f"accumulated radiance, {res}x{res} atlas")
    assert pair.counters()["err"] == 0


def test_textured_sphere_pass_path_matches_oracle(oracle, pk_built):
    """Per-pass path with the uv wrap exercised by a uv range wider than [0, 1]."""
    src = synth.displaced_sphere_scene(subdivisions=5, width=96, height=64, env_size=(256, 128))
    src.uv = src.uv * 1.5 - 0.5  # repeat addressing on both sides of the unit square
    pair = textured_pair(oracle, src, 32, seed=7, mode=_lib.PK_TRACE_CHUNKED)
    c, P = pair.ctx, pair.P.r
    for f in range(2):
        c.call("pk_set_render_state", f, 0.0)
        P.set_render_state(f)
        for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
            c.call("pk_" + name)
            getattr(P, name)()
        for _ in range(4):
            for name in ("trace", "shade_hit", "trace_shadow", "shade_miss"):
                c.call("pk_" + name)
                getattr(P, name)()
        c.call("pk_accumulate")
        P.accumulate()
    assert_bits_equal(pair.image("accum"), P.accum(), "accumulated radiance, wrapped uvs")


@pytest.mark.parametrize("res,n", [(0, 1), (2, 0), (1 << 15, 8)])
def test_atlas_upload_rejects_bad_sizes(pk_built, res, n):
    ctx = _lib.Context(0)
    buf = np.zeros(16, np.uint8)
    with pytest.raises(_lib.PikeError) as e:
        ctx.call("pk_atlas_upload", ptr(buf), res, n)
    assert e.value.code == _lib.PK_ERR_ARG
