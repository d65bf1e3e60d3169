"""Pass-by-pass parity of the CUDA path with the oracle (camera.wgsl, trace.wgsl,
shade_hit.wgsl, trace_shadow.wgsl, shade_miss.wgsl, accumulate.wgsl,
postprocess.wgsl), queue order included.  Bit-exact throughout: the library
pins every operation (IEEE binary32, no contraction), so the tolerance on the
floating-point radiance is zero."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth

from helpers import Pair, assert_bits_equal

pytestmark = pytest.mark.gpu

Q_RAYS, Q_SHADOW, Q_MISS = _lib.PK_QUEUE_RAYS, _lib.PK_QUEUE_SHADOW, _lib.PK_QUEUE_MISS


def run_pass_parity(pair: Pair, frames: int, bounces: int):
    P = pair.P.r
    c = pair.ctx
    for f in range(frames):
        pair.set_render_state(f)
        c.call("pk_clear_color")
        c.call("pk_clear_hits_misses")
        c.call("pk_clear_rays")
        P.begin_frame()
        c.call("pk_camera")
        P.camera()
        g, o = pair.counters(), P.counters()
        assert g["num_rays"] == o["num_rays"]
        assert_bits_equal(pair.rays(Q_RAYS, 0, o["num_rays"]), P.rays(0, o["num_rays"]), f"camera rays f{f}")
        for b in range(bounces):
            tag = f"f{f} b{b}"
            c.call("pk_trace")
            P.trace()
            g, o = pair.counters(), P.counters()
            assert (g["num_hits"], g["num_misses"]) == (o["num_hits"], o["num_misses"]), tag
            assert_bits_equal(pair.hits(o["num_hits"]), P.hits(o["num_hits"]), f"hits {tag}")
            assert_bits_equal(pair.rays(Q_MISS, 0, o["num_misses"]), P.misses(o["num_misses"]), f"trace misses {tag}")
            c.call("pk_shade_hit")
            P.shade_hit()
            g, o = pair.counters(), P.counters()
            assert (g["num_rays"], g["num_shadow"]) == (o["num_rays"], o["num_shadow"]), tag
            assert_bits_equal(pair.rays(Q_RAYS, 0, o["num_rays"]), P.rays(0, o["num_rays"]), f"bounce rays {tag}")
            assert_bits_equal(pair.rays(Q_SHADOW, 0, o["num_shadow"]), P.rays(P.shadow_offset(), o["num_shadow"]),
                              f"shadow rays {tag}")
            c.call("pk_trace_shadow")
            P.trace_shadow()
            g, o = pair.counters(), P.counters()
            assert g["num_misses"] == o["num_misses"], tag
            assert_bits_equal(pair.rays(Q_MISS, 0, o["num_misses"]), P.misses(o["num_misses"]), f"all misses {tag}")
            c.call("pk_shade_miss")
            P.shade_miss()
            assert_bits_equal(pair.image("color"), P.color(), f"colour {tag}")
        c.call("pk_accumulate")
        P.accumulate()
        assert_bits_equal(pair.image("accum"), P.accum(), f"accumulate f{f}")
        c.call("pk_postprocess")
        P.postprocess()
        assert np.array_equal(pair.image("display"), P.display()[1]), f"display f{f}"
    assert pair.counters()["err"] == 0


def test_passes_small_scene_oracle_bvh(oracle, pk_built):
    src = synth.small_scene(width=96, height=64)
    run_pass_parity(Pair(src, oracle, gpu_bvh=False, gpu_env=False), frames=2, bounces=4)


@pytest.mark.parametrize("mode", [_lib.PK_TRACE_PERSISTENT, _lib.PK_TRACE_CHUNKED])
def test_passes_small_scene_gpu_bvh(oracle, pk_built, mode):
    src = synth.small_scene(width=128, height=128)
    run_pass_parity(Pair(src, oracle, trace_mode=mode), frames=2, bounces=4)


@pytest.mark.parametrize("mode", [_lib.PK_TRACE_PERSISTENT, _lib.PK_TRACE_CHUNKED,
                                  _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_COMPACT_RECORDS])
def test_passes_sphere_scene(oracle, pk_built, mode):
    src = synth.displaced_sphere_scene(subdivisions=5, width=80, height=48, env_size=(256, 128))
    run_pass_parity(Pair(src, oracle, trace_mode=mode), frames=2, bounces=6)


def test_passes_env_rotation_and_lens(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=4, width=64, height=40, env_size=(128, 64))
    pair = Pair(src, oracle)
    cam = dict(src.camera_state(), apertureSize=0.05, focalDepth=0.7, distortion=0.2, bokeh=0.7)
    pair.set_camera(cam)
    P = pair.P.r
    for f in range(2):
        pair.set_render_state(f, 0.3)
        for name in ("clear_color", "clear_hits_misses", "clear_rays"):
            pair.ctx.call("pk_" + name)
        P.begin_frame()
        for name in ("camera", "trace", "shade_hit", "trace_shadow", "shade_miss", "trace", "shade_hit",
                     "trace_shadow", "shade_miss", "accumulate"):
            pair.ctx.call("pk_" + name)
            getattr(P, name)()
        assert_bits_equal(pair.image("accum"), P.accum(), f"accum f{f}")


def test_multi_batch_invocation_offset(oracle, pk_built):
    """pike.js:133-155: a frame split into batches with invocationOffset; the
    colour buffer is cleared once per frame, the counters once per batch."""
    src = synth.small_scene(width=50, height=30)
    batch = 512
    pair = Pair(src, oracle, batch=batch)
    P = pair.P.r
    c = pair.ctx
    base = src.camera_state()
    for f in range(2):
        pair.set_render_state(f)
        c.call("pk_clear_color")
        P.clear_color()
        for j in range(-(-src.width * src.height // batch)):
            pair.set_camera(dict(base, invocationOffset=j * batch))
            for name in ("clear_hits_misses", "clear_rays", "camera"):
                c.call("pk_" + name)
                getattr(P, name)()
            for _ in range(3):
                for name in ("trace", "shade_hit", "trace_shadow", "shade_miss"):
                    c.call("pk_" + name)
                    getattr(P, name)()
            assert pair.counters()["num_misses"] == P.counters()["num_misses"]
        assert_bits_equal(pair.image("color"), P.color(), f"multi-batch colour f{f}")
        c.call("pk_accumulate")
        P.accumulate()
        assert_bits_equal(pair.image("accum"), P.accum(), f"multi-batch accum f{f}")
