"""Compensated accumulation (PK_ACCUM_COMPENSATED): the accumulated mean
against an FP64 mean of the same per-frame colours, next to the reference's
running mean (which stays the default and stays bit-exact)."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import ptr

from helpers import Pair

pytestmark = pytest.mark.gpu


def test_compensated_accumulation_error(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=5, width=48, height=32, env_size=(256, 128))
    frames = 96
    errs = {}
    for mode in (_lib.PK_ACCUM_RUNNING_MEAN, _lib.PK_ACCUM_COMPENSATED):
        pair = Pair(src, oracle)
        c = pair.ctx
        c.call("pk_set_accumulation", mode)
        ref = np.zeros((src.height, src.width, 3))
        for f in range(frames):
            c.call("pk_set_render_state", f, 0.0)
            c.call("pk_render_frame", 4)
            ref += np.maximum(pair.image("color")[..., :3].astype(np.float64), 0.0)
        ref /= frames
        acc = pair.image("accum")[..., :3].astype(np.float64)
        errs[mode] = np.abs(acc - ref).max() / ref.max()
    assert errs[_lib.PK_ACCUM_COMPENSATED] <= errs[_lib.PK_ACCUM_RUNNING_MEAN]
    assert errs[_lib.PK_ACCUM_COMPENSATED] < 2.0 ** -21, errs


def test_accumulation_mode_rejects_unknown(oracle, pk_built):
    pair = Pair(synth.small_scene(width=8, height=8), oracle)
    with pytest.raises(_lib.PikeError) as e:
        pair.ctx.call("pk_set_accumulation", 7)
    assert e.value.code == _lib.PK_ERR_ARG
