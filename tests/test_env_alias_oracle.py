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


def sequential_sweep(q, frac):
    """The sweeping alias construction run in order (Huebschle-Schneider &
    Sanders 2022, the sequential algorithm the parallel evaluation restates):
    lights in index order are served by the current heavy while its weight is
    at least one; a heavy whose weight falls below one keeps it and takes the
    next heavy as its alias, which pays its deficit."""
    one = 1 << frac
    q = [int(x) for x in q]
    n = len(q)
    L = [i for i in range(n) if q[i] < one]
    H = [i for i in range(n) if q[i] >= one]
    keep = [one] * n
    alias = list(range(n))
    if not H:
        return keep, alias
    a, b, w = 0, 0, q[H[0]]
    while a < len(L) or w < one:
        if w >= one and a < len(L):
            keep[L[a]] = q[L[a]]
            alias[L[a]] = H[b]
            w -= one - q[L[a]]
            a += 1
        elif w < one and b + 1 < len(H):
            keep[H[b]] = w
            alias[H[b]] = H[b + 1]
            w = q[H[b + 1]] - (one - w)
            b += 1
        else:
            break
    return keep, alias


@pytest.mark.parametrize("env_size", [(96, 48), (40, 20), (5, 3)])
def test_parallel_sweep_equals_sequential_sweep(env_size):
    """The prefix-sum evaluation of the sweep gives the sequential sweep's
    table entry for entry."""
    from oracle import pyoracle
    src = synth.displaced_sphere_scene(subdivisions=1, width=8, height=8, env_size=(max(env_size[0], 4), max(env_size[1], 2)))
    rgbe = np.ascontiguousarray(np.asarray(src.env_rgbe, np.uint8)[:env_size[1], :env_size[0]])
    q, frac = pyoracle.env_alias(rgbe, return_weights=True)
    keep, alias = sequential_sweep(q, frac)
    thr = [0xFFFFFFFF if k >= (1 << frac) else min(k >> (frac - 32), 0xFFFFFFFE) for k in keep]
    table, _ = pyoracle.env_alias(rgbe)
    assert table[:, 1].tolist() == alias
    assert table[:, 0].tolist() == thr
