"""Form (3) on the CPU: the FP64 oracle's analytic gradient of the
differentiable path tracer against its own central finite differences (the
paths do not depend on the parameters, so the estimator is smooth for fixed
seeds and the two must agree to rounding)."""
import numpy as np
import pytest

from pike_gb300 import synth
from pike_gb300.diff import pinhole


@pytest.fixture(scope="module")
def setup(oracle):
    src = synth.small_scene(width=20, height=14)
    P = oracle.Prepared(src, threads=4)
    rng = np.random.default_rng(11)
    n = src.materials.shape[0]
    albedo = rng.uniform(0.2, 0.9, (n, 3))
    rough = rng.uniform(0.1, 0.9, n)
    metal = (rng.uniform(size=n) < 0.5).astype(np.float64)
    env = rng.uniform(0.1, 3.0, (8, 16, 3))
    cam = pinhole(src.camera_state(), src.width, src.height)
    dimage = rng.normal(size=(src.height, src.width, 3))
    return src, P, dict(cam12=cam, albedo=albedo, rough=rough, metal=metal, env=env, spp=3, depth=4, seed=5,
                        W=src.width, H=src.height), dimage


def loss(P, args, dimage):
    img, _ = P.r.diff_render(**args)
    return float((img * dimage).sum())


def test_oracle_gradient_matches_central_differences(setup):
    src, P, args, dimage = setup
    ga, gr, ge = P.r.diff_grad(**args, dimage=dimage)
    assert np.abs(ga).max() > 0 and np.abs(gr).max() > 0 and np.abs(ge).max() > 0
    h = 1e-6
    checks = [("albedo", (i, c)) for i in range(ga.shape[0]) for c in range(3)][::7]
    checks += [("rough", (i,)) for i in range(gr.shape[0])][::5]
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
    """Doubling the environment doubles the image (no term is nonlinear in it)."""
    src, P, args, _ = setup
    a, _ = P.r.diff_render(**args)
    b, _ = P.r.diff_render(**dict(args, env=2.0 * args["env"]))
    assert np.allclose(b, 2.0 * a, rtol=1e-12, atol=0)
