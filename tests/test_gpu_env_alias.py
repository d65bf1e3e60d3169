"""PK_ENV_ALIAS: environment sampling from an alias table built on the GPU
(FP64 normalisation, fixed-point weights, the parallel sweep from exact
integer prefix sums; the precision form's alternative to env_sampler.js's
equal-mass histogram; no reference counterpart).  The table and its pdf
texture equal the oracle's numpy restatement bit for bit, the table's exact
selection probabilities equal the texels' share of the radiance, and frames
rendered with it equal the oracle's (run on the downloaded table) bit for
bit."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import ptr

from helpers import Pair, assert_bits_equal

pytestmark = pytest.mark.gpu


def radiance(rgbe: np.ndarray) -> np.ndarray:
    """env_sampler.js:43-48: 2^(a-128) * luma(rgb) / 255, in FP64."""
    c = rgbe.reshape(-1, 4).astype(np.float64)
    return np.ldexp(1.0, rgbe.reshape(-1, 4)[:, 3].astype(np.int64) - 128) * (
        0.2126 * c[:, 0] + 0.7152 * c[:, 1] + 0.0722 * c[:, 2]) / 255.0


def alias_tables(ctx, n):
    table = np.zeros((n, 2), np.uint32)
    pdf = np.zeros(n, np.float32)
    ctx.call("pk_env_alias_download", ptr(table), ptr(pdf))
    return table, pdf


@pytest.mark.parametrize("env_size", [(2048, 1024), (96, 48)])
def test_alias_table_probabilities(oracle, pk_built, env_size):
    src = synth.displaced_sphere_scene(subdivisions=4, width=16, height=16, env_size=env_size)
    pair = Pair(src, oracle)
    pair.ctx.call("pk_set_env_sampling", _lib.PK_ENV_ALIAS)
    n = env_size[0] * env_size[1]
    table, pdf = alias_tables(pair.ctx, n)
    thr, alias = table[:, 0].astype(np.float64), table[:, 1].astype(np.int64)
    assert (alias >= 0).all() and (alias < n).all()
    keep = np.where(table[:, 0] == 0xFFFFFFFF, 1.0, thr / 2.0 ** 32)
    p = keep.copy()
    np.add.at(p, alias, 1.0 - keep)
    p /= n  # the table's exact selection probabilities
    L = radiance(src.env_rgbe)
    want = L / L.sum()
    assert abs(p.sum() - 1.0) < 1e-12
    # thresholds are quantised to 2^-32: each entry moves at most 2^-32 / n of probability
    assert np.abs(p - want).sum() < 2.0 ** -30
    assert np.abs(p - want).max() < 1e-12 + 1e-6 * want.max()
    # pdf texture: probability * n / (2 pi^2), in binary32
    np.testing.assert_allclose(pdf.astype(np.float64), p * n / (2.0 * np.pi ** 2), rtol=2e-7, atol=0)
    assert ((pdf > 0) == (want > 0)).all()


@pytest.mark.parametrize("env_size,kind", [((2048, 1024), "sun"), ((96, 48), "sun"), ((64, 32), "sky"),
                                           ((48, 24), "uniform")])
def test_alias_table_equals_restatement(oracle, pk_built, env_size, kind):
    """Bit-exact table and pdf; "uniform" (every texel equal) puts every weight
    within rounding of the mean, so lights and heavies differ by a few units."""
    from oracle import pyoracle
    src = synth.displaced_sphere_scene(subdivisions=4, width=16, height=16, env_size=env_size)
    if kind == "sun":
        rgbe = np.ascontiguousarray(src.env_rgbe, np.uint8)
    elif kind == "sky":
        rgbe = np.ascontiguousarray(synth.rgbe_encode(synth.hdr_env(synth.SEED_BASE + 3, env_size[0], env_size[1],
                                                                    sun=1.0)), np.uint8)
    else:
        rgbe = np.zeros((env_size[1], env_size[0], 4), np.uint8)
        rgbe[...] = (200, 150, 100, 129)
    pair = Pair(src, oracle)
    pair.ctx.call("pk_env_build", ptr(rgbe), env_size[0], env_size[1])
    pair.ctx.call("pk_set_env_sampling", _lib.PK_ENV_ALIAS)
    table, pdf = alias_tables(pair.ctx, env_size[0] * env_size[1])
    want_table, want_pdf = pyoracle.env_alias(rgbe)
    assert np.array_equal(table, want_table)
    assert np.array_equal(pdf.view(np.uint32), want_pdf.view(np.uint32))


def test_alias_frames_match_oracle(oracle, pk_built):
    src = synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256))
    pair = Pair(src, oracle)
    pair.ctx.call("pk_set_env_sampling", _lib.PK_ENV_ALIAS)
    n = 512 * 256
    table, pdf = alias_tables(pair.ctx, n)
    pair.P.r.set_env_alias(table, pdf)
    pair.ctx.call("pk_set_render_state", 0, 0.0)
    pair.ctx.call("pk_render_frames", 3, 8)
    pair.ctx.call("pk_sync")
    R = pair.P.r
    R.set_render_state(0)
    for _ in range(3):
        R.tick(8)
    assert_bits_equal(pair.image("accum"), R.accum(), "alias-table frames vs oracle")
    # switching back gives the reference's histogram frames
    pair.ctx.call("pk_set_env_sampling", _lib.PK_ENV_HISTOGRAM)
    pair.ctx.call("pk_write_accum", ptr(np.zeros((90, 160, 4), np.float32)))
    pair.ctx.call("pk_set_render_state", 0, 0.0)
    pair.ctx.call("pk_render_frames", 1, 8)
    pair.ctx.call("pk_sync")
    P2 = oracle.Prepared(src)
    P2.r.set_render_state(0)
    P2.r.tick(8)
    assert_bits_equal(pair.image("color"), P2.r.color(), "histogram frame after switching back")


def test_alias_mode_rules(oracle, pk_built):
    src = synth.small_scene(width=8, height=8)
    pair = Pair(src, oracle)
    with pytest.raises(_lib.PikeError) as e:
        pair.ctx.call("pk_set_env_sampling", 7)
    assert e.value.code == _lib.PK_ERR_ARG
    with pytest.raises(_lib.PikeError) as e:
        pair.ctx.call("pk_env_alias_download", None, None)
    assert e.value.code == _lib.PK_ERR_STATE
