"""The GPU's converged image against the oracle's FP64 evaluation of the same
light paths (om_render64.h), on the 1.3M-triangle scene's geometry family:
bit-identical to the FP32 oracle, the stated relative error against FP64,
and every pixel inside the 3-sigma Monte Carlo band of the FP64 render."""
import numpy as np
import pytest

from pike_gb300 import synth

from helpers import Pair, assert_bits_equal
from test_oracle_fp64 import fp64_stats

pytestmark = pytest.mark.gpu


def test_converged_image_against_fp64_paths(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256))
    frames, bounces = 16, 8
    pair = Pair(src, oracle, threads=16)
    R = pair.P.r
    R.set_track64(True)
    R.set_render_state(0)
    for _ in range(frames):
        R.tick(bounces)
    pair.ctx.call("pk_set_render_state", 0, 0.0)
    pair.ctx.call("pk_render_frames", frames, bounces)
    gpu = pair.image("accum")
    assert_bits_equal(gpu, R.accum(), "GPU vs FP32 oracle")
    s = fp64_stats(gpu[..., :3].astype(np.float64), R.accum64()[..., :3], R.std64()[..., :3], frames)
    print("FP64 comparison:", s)
    assert s["rel_median"] < 1e-6 and s["rel_p99"] < 1e-5, s
    assert s["inside_3sigma"] == 1.0 and s["band_fraction_max"] < 0.1, s
