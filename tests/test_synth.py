"""Synthetic scenes have the shapes the benchmark configurations name."""
import numpy as np

from pike_gb300 import synth


def test_small_scene_shape():
    s = synth.small_scene()
    assert s.n_tris == 770 and (s.width, s.height, s.spp, s.bounces) == (256, 256, 4, 4)
    alb = s.materials[:, :3]
    assert alb.min() >= 0.2 and alb.max() <= 0.8
    assert (s.env_rgbe == np.array([255, 255, 255, 128], np.uint8)).all()


def test_small_scene_deterministic():
    a, b = synth.small_scene(), synth.small_scene()
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.materials, b.materials)


def test_icosphere_counts():
    v, f = synth.icosphere(3)
    assert f.shape[0] == 20 * 4 ** 3 and v.shape[0] == 10 * 4 ** 3 + 2


def test_displaced_sphere_scene_shape():
    s = synth.displaced_sphere_scene(subdivisions=4, env_size=(64, 32))
    assert s.n_tris == 20 * 4 ** 4 + 10
    m = s.materials[:256]
    assert m[:, 4].min() >= 0.05 and m[:, 4].max() <= 1.0
    assert set(np.unique(m[:, 5])) <= {0.0, 1.0}
    assert s.env_rgbe.shape == (32, 64, 4)


def test_rgbe_round_trip():
    x = np.array([[1.0, 0.5, 0.25], [1e4, 1e4, 1e4], [0.0, 0.0, 0.0], [3.0, 1e-3, 7.5]])
    e = synth.rgbe_encode(x).astype(np.float64)
    dec = e[:, :3] / 255.0 * np.ldexp(1.0, (e[:, 3] - 128).astype(int))[:, None]
    # shared exponent: every channel is within half a mantissa step of the largest one
    step = x.max(axis=1, keepdims=True) / 127.0
    assert (np.abs(dec - x) <= step * 0.5 + 1e-30).all()


def test_exp_matches_math():
    x = np.linspace(-20, 20, 10001)
    assert np.allclose(synth._exp(x), np.exp(x), rtol=2e-15)
