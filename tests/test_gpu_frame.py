"""Whole-frame parity: pk_render_frame (misses shaded inside the traversal
kernels) against the oracle's tick(), and against the GPU's own pass-by-pass
path; plus size-independent properties at the benchmark's full size."""
import ctypes

import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import ptr

from helpers import Pair, assert_bits_equal, camera_struct

pytestmark = pytest.mark.gpu


def fused_frames(pair: Pair, frames: int, bounces: int, start: int = 0):
    pair.ctx.call("pk_set_render_state", start, 0.0)
    pair.ctx.call("pk_render_frames", frames, bounces)
    pair.ctx.call("pk_sync")


def oracle_frames(pair: Pair, frames: int, bounces: int, start: int = 0):
    P = pair.P.r
    P.set_render_state(start)
    for _ in range(frames):
        P.tick(bounces)


def test_fused_small_scene_matches_oracle(oracle, pk_built):
    src = synth.small_scene()  # 256x256, 770 triangles, 4 spp, 4 bounces
    pair = Pair(src, oracle)
    fused_frames(pair, src.spp, src.bounces)
    oracle_frames(pair, src.spp, src.bounces)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), "accumulated radiance")
    assert np.array_equal(pair.image("display"), pair.P.r.display()[1])
    c = pair.counters()
    assert c["samples"] == src.spp and c["err"] == 0


@pytest.mark.parametrize("mode", [_lib.PK_TRACE_PERSISTENT, _lib.PK_TRACE_CHUNKED,
                                  _lib.PK_TRACE_CHUNKED | _lib.PK_TRACE_COMPACT_RECORDS])
def test_fused_sphere_matches_oracle(oracle, pk_built, mode):
    src = synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256))
    pair = Pair(src, oracle, trace_mode=mode)
    fused_frames(pair, 3, 8)
    oracle_frames(pair, 3, 8)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), "accumulated radiance")


@pytest.mark.slow
def test_fused_full_geometry_matches_oracle(oracle, pk_built):
    """The 1.3M-triangle scene and 2048x1024 environment of the benchmark, at a
    reduced resolution the oracle finishes in seconds."""
    src = synth.displaced_sphere_scene(width=192, height=108)
    pair = Pair(src, oracle, threads=16)
    fused_frames(pair, 2, 8)
    oracle_frames(pair, 2, 8)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), "accumulated radiance")


def test_fused_equals_pass_path(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=6, width=320, height=180, env_size=(512, 256))
    a = Pair(src, oracle)
    fused_frames(a, 2, 8)
    fused = a.image("accum")
    # the pass path below runs with the other traversal schedule: results must not depend on it
    a.ctx.call("pk_set_trace_mode", _lib.PK_TRACE_CHUNKED)
    c = a.ctx
    c.call("pk_write_accum", ptr(np.zeros_like(fused)))
    for f in range(2):
        c.call("pk_set_render_state", f, 0.0)
        for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
            c.call("pk_" + name)
        for _ in range(8):
            for name in ("trace", "shade_hit", "trace_shadow", "shade_miss"):
                c.call("pk_" + name)
        c.call("pk_accumulate")
    assert_bits_equal(a.image("accum"), fused, "pass path vs fused frame")


@pytest.mark.slow
def test_full_size_frame_matches_oracle(oracle, pk_built):
    """The benchmark's workload itself: 1920x1080 on the 1.3M-triangle scene
    with the 2048x1024 environment and 8 bounces, one fused frame (in pixel
    batches of 1920x270, as tick() renders them) bit-exact against the
    oracle."""
    src = synth.displaced_sphere_scene()
    pair = Pair(src, oracle, threads=16, batch=src.width * 270)
    fused_frames(pair, 1, 8)
    oracle_frames(pair, 1, 8)
    assert_bits_equal(pair.image("color"), pair.P.r.color(), "1080p frame colour")
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), "1080p accumulated radiance")


def test_full_size_determinism_and_counts(oracle, pk_built):
    """1920x1080 on the 1.3M-triangle scene: two renders are bit-identical, no
    device error flags, and the ray counts obey the queue invariants."""
    src = synth.displaced_sphere_scene()
    pair = Pair(src, oracle, threads=16)
    c = pair.ctx
    c.call("pk_reset_stats")
    fused_frames(pair, 2, 8)
    first = pair.image("accum").copy()
    cnt = pair.counters()
    assert cnt["err"] == 0
    npix = src.width * src.height
    assert npix * 2 <= cnt["rays_traced"] <= npix * 2 * 8 * 2
    c.call("pk_write_accum", ptr(np.zeros_like(first)))
    fused_frames(pair, 2, 8)
    assert_bits_equal(pair.image("accum"), first, "re-render")
    assert np.isfinite(first).all()


def test_empty_queues_all_rays_miss(oracle, pk_built):
    src = synth.small_scene(width=64, height=64)
    pair = Pair(src, oracle)
    st = dict(src.camera_state(), dir=[0.0, 1.0, 0.0])  # looking straight up at the sky
    st["dir"] = [0.0, 0.9999999, 0.0004]
    pair.set_camera(st)
    fused_frames(pair, 1, 4)
    oracle_frames(pair, 1, 4)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), "sky-only frame")
    assert pair.counters()["num_hits"] == 0


def test_odd_resolution_accumulate(oracle, pk_built):
    src = synth.small_scene(width=131, height=77)
    pair = Pair(src, oracle)
    fused_frames(pair, 2, 3)
    oracle_frames(pair, 2, 3)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), "odd resolution")


def test_pass_before_scene_is_an_error(pk_built):
    ctx = _lib.Context(0)
    ctx.call("pk_configure", 8, 8, 64)
    with pytest.raises(_lib.PikeError) as e:
        ctx.call("pk_trace")
    assert e.value.code == _lib.PK_ERR_ARG or e.value.code == _lib.PK_ERR_STATE


def test_malformed_bvh_upload_rejected(oracle, pk_built):
    src = synth.small_scene(width=8, height=8)
    pair = Pair(src, oracle)
    b = pair.P.bvh
    nodes = b.nodes.copy()
    nodes[0, 0] = 10**6  # child index outside the node array
    with pytest.raises(_lib.PikeError):
        pair.ctx.call("pk_bvh_upload", ptr(nodes), nodes.shape[0], ptr(b.tris), b.tris.shape[0], ptr(b.verts),
                      b.verts.shape[0])


def test_counting_kernels_match_oracle_counts(oracle, pk_built):
    """The counting traversal variants report the reference algorithm's node
    fetches and triangle tests; they must equal the oracle's counts."""
    src = synth.displaced_sphere_scene(subdivisions=5, width=96, height=64, env_size=(256, 128))
    pair = Pair(src, oracle)
    c = pair.ctx
    c.call("pk_reset_stats")
    c.call("pk_set_counting", 1)
    fused_frames(pair, 1, 6)
    c.call("pk_set_counting", 0)
    s = np.zeros(10, np.uint64)
    c.call("pk_read_stats", ptr(s))
    P = pair.P.r
    P.reset_stats()
    oracle_frames(pair, 1, 6)
    o = P.stats()
    assert int(s[4]) == o["trace_rays"] and int(s[5]) == o["shadow_rays"]
    assert int(s[0]) == o["trace_fetch"] and int(s[1]) == o["trace_tests"]
    assert int(s[2]) == o["shadow_fetch"] and int(s[3]) == o["shadow_tests"]


@pytest.mark.parametrize("mode,bounces", [(_lib.PK_TRACE_PERSISTENT, 8), (_lib.PK_TRACE_PERSISTENT, 20),
                                          (_lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE, 8)])
def test_frame_overlap_is_bit_identical(oracle, pk_built, mode, bounces):
    """Shadow traversal of bounce b beside the closest-hit traversal of b+1
    against the serial frame, one frame at a time (where the default turns it
    on) and four in flight; 20 bounces wrap the 16 per-bounce ticket slots.
    The persistent binary mode is also checked against the oracle."""
    src = synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256))
    pair = Pair(src, oracle)
    pair.ctx.call("pk_set_trace_mode", mode)  # after the BVH: the 8-wide tree is built from it
    pair.ctx.call("pk_set_frames_in_flight", 1)  # PK_OVERLAP_AUTO: overlapped
    fused_frames(pair, 2, bounces)
    on = pair.image("accum").copy()
    assert pair.counters()["err"] == 0
    pair.ctx.call("pk_set_frame_overlap", 0)
    pair.ctx.call("pk_write_accum", ptr(np.zeros_like(on)))
    fused_frames(pair, 2, bounces)
    assert_bits_equal(pair.image("accum"), on, "serial vs overlapped frame")
    pair.ctx.call("pk_set_frames_in_flight", 4)
    pair.ctx.call("pk_set_frame_overlap", 1)
    pair.ctx.call("pk_write_accum", ptr(np.zeros_like(on)))
    fused_frames(pair, 2, bounces)
    assert_bits_equal(pair.image("accum"), on, "overlapped frames in flight")
    if mode == _lib.PK_TRACE_PERSISTENT:
        oracle_frames(pair, 2, bounces)
        assert_bits_equal(on, pair.P.r.accum(), "overlapped frame vs oracle")


def _orbit(src, f: int) -> dict:
    st = dict(src.camera_state())
    a = 0.05 * f
    x, z = st["dir"][0], st["dir"][2]
    st["dir"] = [x * np.cos(a) - z * np.sin(a), st["dir"][1], x * np.sin(a) + z * np.cos(a)]
    return st


def _stepped_frames(pair: Pair, src, frames: int, bounces: int):
    """A render loop as an application writes it: per frame the render state,
    a moving camera, pk_render_frame and an asynchronous display read into its
    own pinned buffer (all enqueued before one pk_sync)."""
    c = pair.ctx
    bufs = [c.pinned((src.height, src.width, 4), "uint8") for _ in range(frames)]
    for f in range(frames):
        c.call("pk_set_render_state", f, 0.01 * f)
        c.call("pk_set_camera", camera_struct(_orbit(src, f)))
        c.call("pk_render_frame", bounces)
        c.call("pk_read_display_async", bufs[f].array.ctypes.data_as(ctypes.c_void_p))
    c.call("pk_sync")
    out = [b.array.copy() for b in bufs]
    for b in bufs:
        b.free()
    return out


def test_frames_in_flight_bit_identical(oracle, pk_built):
    """Four (the default) and two frames in flight against one at a time: the same
    display after every frame, accumulation, colour of the last frame, counters
    and ray totals; the pass API afterwards starts from the host's render state."""
    src = synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256))
    runs = {}
    for n in (4, 2, 1):
        pair = Pair(src, oracle)
        pair.ctx.call("pk_set_frames_in_flight", n)
        pair.ctx.call("pk_reset_stats")
        disp = _stepped_frames(pair, src, 5, 6)
        s = np.zeros(10, np.uint64)
        pair.ctx.call("pk_read_stats", ptr(s))
        runs[n] = (disp, pair.image("accum").copy(), pair.image("color").copy(), pair.counters(), s.copy())
        c = pair.counters()
        assert c["samples"] == 5 and c["err"] == 0
    d1, a1, c1, k1, s1 = runs[1]
    assert len({d.tobytes() for d in d1}) == 5  # the camera moved: every frame differs
    for n in (4, 2):
        dn, an, cn, kn, sn = runs[n]
        for f in range(5):
            assert np.array_equal(dn[f], d1[f]), f"{n} in flight: display after frame {f}"
        assert_bits_equal(an, a1, f"{n} in flight: accumulation")
        assert_bits_equal(cn, c1, f"{n} in flight: colour of the last frame")
        assert kn == k1 and np.array_equal(sn, s1)
    # the oracle renders the same stepped sequence
    P = pair.P.r
    P.set_render_state(0)
    for f in range(5):
        pair.set_camera(_orbit(src, f))
        P.set_render_state(f, 0.01 * f)
        P.tick(6)
    assert_bits_equal(a1, P.accum(), "stepped frames vs oracle")


def test_passes_after_frames_in_flight(oracle, pk_built):
    """Frames in flight, then pass-by-pass frames on the same context: the
    passes see the render state advanced by the frames and the accumulated
    image equals an all-frames render."""
    src = synth.displaced_sphere_scene(subdivisions=5, width=96, height=64, env_size=(256, 128))
    ref = Pair(src, oracle)
    fused_frames(ref, 4, 6)
    want = ref.image("accum").copy()
    a = Pair(src, oracle)
    fused_frames(a, 3, 6)  # frames 0..2 in flight; frame 3 by passes, no render state set in between
    c = a.ctx
    for name in ("clear_color", "clear_hits_misses", "clear_rays", "camera"):
        c.call("pk_" + name)
    for _ in range(6):
        for name in ("trace", "shade_hit", "trace_shadow", "shade_miss"):
            c.call("pk_" + name)
    c.call("pk_accumulate")
    assert a.counters()["samples"] == 3  # passes do not advance the sample index
    assert_bits_equal(a.image("accum"), want, "passes after frames in flight")



def test_frames_in_flight_across_reconfigure_env_and_switches(oracle, pk_built):
    """Frames in flight, then a new resolution, a new environment and changes
    of the number in flight between frames: every accumulation equals the one
    of the same sequence rendered one frame at a time."""
    src = synth.displaced_sphere_scene(subdivisions=5, width=128, height=96, env_size=(256, 128))
    env2 = np.ascontiguousarray(np.roll(np.asarray(src.env_rgbe, np.uint8), 37, axis=1))
    results = {}
    for piped in (False, True):
        pair = Pair(src, oracle)
        c = pair.ctx
        c.call("pk_set_frames_in_flight", 4 if piped else 1)
        c.call("pk_set_render_state", 0, 0.0)
        c.call("pk_render_frames", 3, 6)
        first = pair.image("accum").copy()
        c.call("pk_configure", 96, 64, 96 * 64)  # new queues and slot buffers while frames may be in flight
        c.call("pk_set_camera", camera_struct(src.camera_state()))
        if piped:
            c.call("pk_set_frames_in_flight", 3)
        c.call("pk_set_render_state", 0, 0.0)
        c.call("pk_render_frames", 5, 6)
        second = np.zeros((64, 96, 4), np.float32)
        c.call("pk_read_accum", ptr(second))
        c.call("pk_env_build", ptr(env2), env2.shape[1], env2.shape[0])
        if piped:
            c.call("pk_set_frames_in_flight", 2)
        c.call("pk_render_frames", 3, 6)
        third = np.zeros((64, 96, 4), np.float32)
        c.call("pk_read_accum", ptr(third))
        results[piped] = (first, second, third, pair.counters())
    for k, name in enumerate(("before", "after reconfigure", "after a new environment")):
        assert_bits_equal(results[True][k], results[False][k], name)
    assert results[True][3]["samples"] == results[False][3]["samples"] == 8
    assert results[True][3]["err"] == 0


def test_frame_scheduling_arguments(oracle, pk_built):
    src = synth.small_scene(width=32, height=32)
    pair = Pair(src, oracle)
    c = pair.ctx
    for bad in (0, 17, -1):
        with pytest.raises(_lib.PikeError) as e:
            c.call("pk_set_frames_in_flight", bad)
        assert e.value.code == _lib.PK_ERR_ARG
    for n in (1, 8, 16):
        c.call("pk_set_frames_in_flight", n)
        c.call("pk_set_frame_overlap", 1 if n == 8 else _lib.PK_OVERLAP_AUTO)
        fused_frames(pair, 17, 3)  # more frames than slots
        assert pair.counters()["samples"] == 17 and pair.counters()["err"] == 0


@pytest.mark.parametrize("batch,bounces", [(512, 3), (500, 8)])
def test_fused_multi_batch_matches_oracle(oracle, pk_built, batch, bounces):
    """tick() over several pixel batches (pike.js:133-154) in one
    pk_render_frame: 1500 pixels in batches of 512, and of 500 (the camera
    dispatch rounds up to 512 invocations, so 12 pixels of each next batch are
    traced twice, as in the reference), 3 and 8 bounces (24 steps wrap the 16
    per-step ticket slots)."""
    src = synth.small_scene(width=50, height=30)
    pair = Pair(src, oracle, batch=batch)
    fused_frames(pair, 2, bounces)
    oracle_frames(pair, 2, bounces)
    assert_bits_equal(pair.image("accum"), pair.P.r.accum(), f"batch {batch}")
    assert pair.counters()["err"] == 0


@pytest.mark.parametrize("mode", [_lib.PK_TRACE_PERSISTENT, _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_WIDE,
                                  _lib.PK_TRACE_PERSISTENT | _lib.PK_TRACE_EXACT])
def test_scheduling_combinations_are_bit_identical(oracle, pk_built, mode):
    """Pixel batches (500 of 1500 pixels) x three frames in flight x forced
    overlap, against one frame at a time without overlap, for every
    persistent traversal; the reference traversal also against the oracle."""
    src = synth.small_scene(width=50, height=30)
    out = []
    for in_flight, overlap in ((1, 0), (3, 1)):
        pair = Pair(src, oracle, batch=500)
        c = pair.ctx
        c.call("pk_set_trace_mode", mode)
        c.call("pk_set_frames_in_flight", in_flight)
        c.call("pk_set_frame_overlap", overlap)
        fused_frames(pair, 5, 6)
        assert pair.counters()["err"] == 0
        out.append(pair.image("accum").copy())
    assert_bits_equal(out[1], out[0], "scheduled vs plain")
    if mode == _lib.PK_TRACE_PERSISTENT:
        oracle_frames(pair, 5, 6)
        assert_bits_equal(out[1], pair.P.r.accum(), "scheduled vs oracle")
