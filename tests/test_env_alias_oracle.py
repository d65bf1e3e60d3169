"""The oracle's restatement of PK_ENV_ALIAS's table (no GPU): valid alias
tables whose exact selection probabilities equal the texels' share of the
radiance, with the pdf texture of those probabilities."""
import numpy as np
import pytest

from pike_gb300 import synth


def radiance(rgbe):
    c = rgbe.reshape(-1, 4).astype(np.float64)
    return np.ldexp(1.0, rgbe.reshape(-1, 4)[:, 3].astype(np.int64) - 128) * (
        0.2126 * c[:, 0] + 0.7152 * c[:, 1] + 0.0722 * c[:, 2]) / 255.0


@pytest.mark.parametrize("env_size", [(96, 48), (256, 128), (1, 1), (5, 3)])
def test_restated_alias_table_is_exact(env_size):
    from oracle import pyoracle
    src = synth.displaced_sphere_scene(subdivisions=1, width=8, height=8, env_size=(max(env_size[0], 4), max(env_size[1], 2)))
    rgbe = np.ascontiguousarray(np.asarray(src.env_rgbe, np.uint8)[:env_size[1], :env_size[0]])
    n = env_size[0] * env_size[1]
    table, pdf = pyoracle.env_alias(rgbe)
    alias = table[:, 1].astype(np.int64)
    assert (alias >= 0).all() and (alias < n).all()
    keep = np.where(table[:, 0] == 0xFFFFFFFF, 1.0, table[:, 0] / 2.0 ** 32)
    p = keep.copy()
    np.add.at(p, alias, 1.0 - keep)
    p /= n
    L = radiance(rgbe)
    want = L / L.sum()
    assert abs(p.sum() - 1.0) < 1e-12
    assert np.abs(p - want).sum() < 2.0 ** -30
    np.testing.assert_allclose(pdf.astype(np.float64), p * n / (2.0 * np.pi ** 2), rtol=2e-7, atol=0)
    assert ((pdf > 0) == (want > 0)).all()


def test_restated_alias_table_rejects_black_map():
    from oracle import pyoracle
    assert pyoracle.env_alias(np.zeros((4, 8, 4), np.uint8)) is None
