"""Form (3) on the GPU: pk_diff_render against the FP64 oracle render,
pk_diff_backward against the FP64 oracle gradient and against central finite
differences with common random numbers (h = 1e-3) at 32 random parameters,
and a short inverse-rendering run through torch.autograd."""
import numpy as np
import pytest

from pike_gb300 import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def small(oracle):
    from pike_gb300.diff import DiffScene
    src = synth.displaced_sphere_scene(subdivisions=5, width=64, height=48, env_size=(64, 32))
    scene = DiffScene(src, 64, 48, spp=4, depth=4)
    P = oracle.Prepared(src, threads=16)
    albedo, rough, env = scene.source_params(env_size=(64, 32))
    return src, scene, P, albedo, rough, env


def oracle_args(scene, albedo, rough, env, seed=0):
    return dict(cam12=scene.cam12, albedo=albedo.double().cpu().numpy(), rough=rough.double().cpu().numpy(),
                metal=scene.metallic.double().cpu().numpy(), env=env.double().cpu().numpy(), spp=scene.spp,
                depth=scene.depth, seed=seed, W=scene.W, H=scene.H)


def test_forward_matches_fp64_oracle(small):
    src, scene, P, albedo, rough, env = small
    img = scene.render(albedo, rough, env, seed=3)[..., :3].double().cpu().numpy()
    ref, rays = P.r.diff_render(**oracle_args(scene, albedo, rough, env, seed=3))
    assert rays == scene.rays()  # identical paths
    err = np.abs(img - ref) / (np.abs(ref) + 1e-3)
    assert err.max() < 1e-4, err.max()
    assert ref.max() > 0


def test_adjoint_matches_fp64_oracle_gradient(small):
    src, scene, P, albedo, rough, env = small
    rng = np.random.default_rng(4)
    dimg = rng.normal(size=(scene.H, scene.W, 3))
    d4 = np.zeros((scene.H, scene.W, 4), np.float32)
    d4[..., :3] = dimg
    ga, gr, ge = scene.backward(albedo, rough, env, torch.tensor(d4, device="cuda"), seed=3)
    ra, rr, re = P.r.diff_grad(**oracle_args(scene, albedo, rough, env, seed=3), dimage=d4[..., :3])
    for name, g, r in (("albedo", ga, ra), ("roughness", gr, rr), ("env", ge, re)):
        g = g.cpu().numpy()
        scale = np.abs(r).max()
        assert scale > 0, name
        assert np.abs(g - r).max() <= 2e-4 * scale, (name, np.abs(g - r).max(), scale)


def test_adjoint_matches_central_differences(small):
    """32 random parameters, h = 1e-3, common random numbers; loss = per-pixel L2."""
    from pike_gb300.diff import l2_loss
    src, scene, P, albedo, rough, env = small
    rng = np.random.default_rng(8)
    target = scene.render(albedo * 0.8 + 0.1, (rough * 0.5 + 0.3).clamp(0.05, 1.0), env * 1.2, seed=1)
    a0 = torch.full_like(albedo, 0.5)
    r0 = torch.full_like(rough, 0.5)
    e0 = torch.full_like(env, float(env.mean()))
    img = scene.render(a0, r0, e0, seed=1)
    dimg = 2.0 * (img - target) / (3 * scene.W * scene.H)
    dimg[..., 3] = 0
    ga, gr, ge = scene.backward(a0, r0, e0, dimg, seed=1)
    grads = {"albedo": ga, "rough": gr, "env": ge}
    base = {"albedo": a0, "rough": r0, "env": e0}
    picks = []
    for _ in range(12):
        picks.append(("albedo", (int(rng.integers(0, src.materials.shape[0] - 1)), int(rng.integers(0, 3)))))
    for _ in range(10):
        picks.append(("rough", (int(rng.integers(0, src.materials.shape[0] - 1)),)))
    seen = torch.nonzero(ge.abs().sum(-1) > 0).cpu().numpy()
    for k in rng.choice(seen.shape[0], 10, replace=False):
        picks.append(("env", (int(seen[k, 0]), int(seen[k, 1]), int(rng.integers(0, 3)))))
    h = 1e-3
    scale = {k: float(v.abs().max()) for k, v in grads.items()}
    for name, idx in picks:
        vals = []
        for sgn in (1.0, -1.0):
            p = {k: v.clone() for k, v in base.items()}
            p[name][idx] += sgn * h
            out = scene.render(p["albedo"], p["rough"], p["env"], seed=1)
            vals.append(float(l2_loss(out.double(), target.double())))
        fd = (vals[0] - vals[1]) / (2 * h)
        g = float(grads[name][idx])
        # within 1% of the central difference; below 1e-3 of the largest
        # gradient of the parameter kind, within 1e-5 of it (the benchmark's criterion)
        assert abs(g - fd) <= 0.01 * max(abs(fd), 1e-3 * scale[name]), (name, idx, g, fd, scale[name])


def test_inverse_rendering_reduces_loss(small):
    """Adam through torch.autograd with the target's own seed (a deterministic
    objective whose minimum is the hidden parameters)."""
    from pike_gb300.diff import inverse_render, render, l2_loss
    src, scene, P, _, _, _ = small
    albedo, rough, env = scene.source_params(env_size=(64, 32), sun=5.0)
    target = scene.render(albedo, rough, env, seed=0)
    a0 = torch.full_like(albedo, 0.5)
    r0 = torch.full_like(rough, 0.5)
    e0 = torch.full_like(env, float(env.mean()))
    first = float(l2_loss(render(scene, a0, r0, e0, seed=0), target))
    a, r, e, hist = inverse_render(scene, target, a0, r0, e0, steps=40, lr=0.05,
                                   n_free=src.materials.shape[0] - 1, seed_per_step=False)
    assert hist[-1] < 0.5 * first, (first, hist[-5:])
    assert float(a[-1].sub(0.5).abs().max()) == 0.0  # the fixed box material did not move
