"""Form (3) on the CPU: the FP64 oracle of the differentiable renderer (the
drop-in's estimator with per-material parameters and detached sampling).  Its
gradient, from dual numbers along the recorded paths, must equal its own
central finite differences (the paths are decided in binary32 with the
sampling roughness held fixed, so the estimator is smooth in the parameters
for fixed seeds), and the image must be linear in the environment radiance
(the sampling tables stay fixed)."""
import numpy as np
import pytest

from pike_gb300 import synth


@pytest.fixture(scope="module")
def setup(oracle):
    src = synth.small_scene(width=20, height=14)
    P = oracle.Prepared(src, threads=4)
    rng = np.random.default_rng(11)
    n = src.materials.shape[0]
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    albedo = f32(rng.uniform(0.2, 0.9, (n, 3)))
    rough = f32(rng.uniform(0.1, 0.9, n))
    metal = (rng.uniform(size=n) < 0.5).astype(np.float64)
    env32 = rng.uniform(0.1, 3.0, (8, 16, 3)).astype(np.float32)
    tables = oracle.EnvF32(env32)
    args = dict(W=src.width, H=src.height, albedo=albedo, rough=rough, metal=metal, env=env32.astype(np.float64),
                tables=tables, spp=3, depth=4, sample_base=5, rough0=rough.copy())
    dimage = rng.normal(size=(src.height, src.width, 3))
    return src, P, args, dimage


def loss(P, args, dimage):
    img, _ = P.r.diff_render(**args)
    return float((img * dimage).sum())


def test_oracle_gradient_matches_central_differences(setup):
    src, P, args, dimage = setup
    ga, gr, ge = P.r.diff_grad(**args, dimage=dimage)
    assert np.abs(ga).max() > 0 and np.abs(gr).max() > 0 and np.abs(ge).max() > 0
    h = 1e-6
    checks = [("albedo", (i, c)) for i in range(ga.shape[0]) for c in range(3)][::7]
    checks += [("rough", (i,)) for i in range(gr.shape[0])][::3]
    flat = np.argsort(-np.abs(ge).ravel())[:12]
    checks += [("env", np.unravel_index(k, ge.shape)) for k in flat]
    for name, idx in checks:
        plus = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in args.items()}
        minus = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in args.items()}
        plus[name][idx] += h
        minus[name][idx] -= h
        fd = (loss(P, plus, dimage) - loss(P, minus, dimage)) / (2 * h)
        g = {"albedo": ga, "rough": gr, "env": ge}[name][idx]
        assert abs(g - fd) <= 1e-6 * max(1.0, abs(fd)), (name, idx, g, fd)


def test_oracle_render_is_linear_in_env(setup):
    """Doubling the environment radiance (tables fixed) doubles the image."""
    src, P, args, _ = setup
    a, _ = P.r.diff_render(**args)
    b, _ = P.r.diff_render(**dict(args, env=2.0 * args["env"]))
    assert np.allclose(b, 2.0 * a, rtol=1e-12, atol=0)


def test_roughness_sampling_only_reweights(setup):
    """Sampling with another roughness moves no ray decision of the evaluation
    parameters; the density ratio makes both unbiased for the same image, so
    over many samples the two images agree within Monte Carlo noise."""
    src, P, args, _ = setup
    a = dict(args, spp=64)
    img0, _ = P.r.diff_render(**a)
    img1, _ = P.r.diff_render(**dict(a, rough0=np.clip(args["rough"] * 0.8 + 0.1, 0.05, 1.0)))
    m0, m1 = img0.mean(), img1.mean()
    assert m0 > 0
    assert abs(m1 - m0) < 0.05 * m0, (m0, m1)
