"""Form (3) on the GPU: the differentiable renderer is the drop-in's estimator
(images equal the drop-in pipeline's in distribution), pk_diff_render against
the FP64 oracle render, pk_diff_backward against the FP64 oracle gradient and
against central finite differences with common random numbers (h = 1e-3) at
32 parameters, the sampling tables against the oracle's, and a short
inverse-rendering run through torch.autograd."""
import numpy as np
import pytest

from pike_gb300 import synth
from pike_gb300._lib import ptr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def small(oracle):
    from pike_gb300.diff import DiffScene
    src = synth.displaced_sphere_scene(subdivisions=5, width=64, height=48, env_size=(64, 32))
    scene = DiffScene(src, 64, 48, spp=4, depth=4)
    P = oracle.Prepared(src, threads=16)
    albedo, rough, env = scene.source_params(env_size=(64, 32))
    scene.set_env_sampling(env)
    tables = oracle.EnvF32(env.cpu().numpy())
    return src, scene, P, albedo, rough, env, tables


def oracle_args(scene, albedo, rough, env, tables, seed=0, rough0=None):
    d = lambda t: t.double().cpu().numpy()
    return dict(W=scene.W, H=scene.H, albedo=d(albedo), rough=d(rough), metal=d(scene.metallic), env=d(env),
                tables=tables, spp=scene.spp, depth=scene.depth, sample_base=seed * scene.spp,
                rough0=None if rough0 is None else d(rough0))


def test_sampling_tables_match_oracle(small):
    src, scene, P, albedo, rough, env, tables = small
    scene.set_env_sampling(env)
    bins, coords, pdf = scene.env_tables()
    assert np.array_equal(bins, tables.bins)
    assert np.array_equal(coords, tables.coords)
    assert np.array_equal(pdf.view(np.uint32), tables.pdf.view(np.uint32))


def test_forward_matches_fp64_oracle(small):
    src, scene, P, albedo, rough, env, tables = small
    scene.set_env_sampling(env)
    img = scene.render(albedo, rough, env, seed=3)[..., :3].double().cpu().numpy()
    ref, rays = P.r.diff_render(**oracle_args(scene, albedo, rough, env, tables, seed=3))
    assert rays == scene.rays()  # identical paths
    err = np.abs(img - ref) / (np.abs(ref) + 1e-3)
    assert ref.max() > 0
    assert np.quantile(err, 0.999) < 1e-4 and err.max() < 1e-3, (np.quantile(err, 0.999), err.max())


def test_forward_at_other_sampling_roughness_matches_oracle(small):
    """Sampled with another roughness and reweighted by the VNDF density ratio."""
    src, scene, P, albedo, rough, env, tables = small
    scene.set_env_sampling(env)
    r0 = (rough * 0.7 + 0.2).contiguous()
    img = scene.render(albedo, rough, env, seed=2, rough_sampling=r0)[..., :3].double().cpu().numpy()
    ref, rays = P.r.diff_render(**oracle_args(scene, albedo, rough, env, tables, seed=2, rough0=r0))
    assert rays == scene.rays()
    err = np.abs(img - ref) / (np.abs(ref) + 1e-3)
    assert np.quantile(err, 0.999) < 1e-4 and err.max() < 1e-3, (np.quantile(err, 0.999), err.max())


def test_forward_bit_exact_with_binary32_oracle(small):
    """The oracle's binary32 replay of pk_diff_render (the drop-in's shading
    operations, the density ratio, the accumulation order) gives the same
    image bit for bit, at the sampling roughness and away from it."""
    src, scene, P, albedo, rough, env, tables = small
    scene.set_env_sampling(env)
    for seed, r0 in ((5, None), (6, (rough * 0.6 + 0.3).contiguous())):
        img = scene.render(albedo, rough, env, seed=seed, rough_sampling=r0).cpu().numpy()
        ref, rays = P.r.diff_render32(**oracle_args(scene, albedo, rough, env, tables, seed=seed, rough0=r0))
        assert rays == scene.rays()
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (seed, np.abs(img - ref).max())


def test_adjoint_matches_fp64_oracle_gradient(small):
    src, scene, P, albedo, rough, env, tables = small
    scene.set_env_sampling(env)
    rng = np.random.default_rng(4)
    dimg = rng.normal(size=(scene.H, scene.W, 3))
    d4 = np.zeros((scene.H, scene.W, 4), np.float32)
    d4[..., :3] = dimg
    ga, gr, ge = scene.backward(albedo, rough, env, torch.tensor(d4, device="cuda"), seed=3)
    ra, rr, re = P.r.diff_grad(**oracle_args(scene, albedo, rough, env, tables, seed=3), dimage=d4[..., :3])
    for name, g, r in (("albedo", ga, ra), ("roughness", gr, rr), ("env", ge, re)):
        g = g.cpu().numpy()
        scale = np.abs(r).max()
        assert scale > 0, name
        assert np.abs(g - r).max() <= 1e-3 * scale, (name, np.abs(g - r).max(), scale)


def test_adjoint_matches_central_differences(small):
    """32 parameters (12 albedo channels, 10 roughness values, 10 env texel
    channels) drawn at random among those whose gradient is at least 1% of the
    largest of its kind; h = 1e-3, common random numbers, sampling roughness
    and environment tables held; loss = per-pixel L2.  Each adjoint gradient
    within 1% of its central difference."""
    from pike_gb300.diff import l2_loss
    src, scene, P, albedo, rough, env, tables = small
    rng = np.random.default_rng(8)
    scene.set_env_sampling(env * 1.2)
    target = scene.render(albedo * 0.8 + 0.1, (rough * 0.5 + 0.3).clamp(0.05, 1.0), env * 1.2, seed=1)
    n_free = src.materials.shape[0] - 1
    a0 = torch.full_like(albedo, 0.5)
    r0 = torch.full_like(rough, 0.5)
    e0 = torch.full_like(env, float(env.mean()))
    scene.set_env_sampling(e0)
    img = scene.render(a0, r0, e0, seed=1)
    dimg = 2.0 * (img - target) / (3 * scene.W * scene.H)
    dimg[..., 3] = 0
    ga, gr, ge = scene.backward(a0, r0, e0, dimg, seed=1)
    grads = {"albedo": ga, "rough": gr, "env": ge}
    base = {"albedo": a0, "rough": r0, "env": e0}

    def pick(name, k):
        g = grads[name].abs()
        if name != "env":
            g = g[:n_free]
        cand = torch.nonzero(g >= 0.01 * g.max()).cpu().numpy()
        assert cand.shape[0] >= k, name
        return [(name, tuple(int(x) for x in cand[i])) for i in rng.choice(cand.shape[0], k, replace=False)]

    picks = pick("albedo", 12) + pick("rough", 10) + pick("env", 10)
    h = 1e-3
    for name, idx in picks:
        vals = []
        for sgn in (1.0, -1.0):
            p = {k: v.clone() for k, v in base.items()}
            p[name][idx] += sgn * h
            out = scene.render(p["albedo"], p["rough"], p["env"], seed=1, rough_sampling=r0)
            vals.append(float(l2_loss(out.double(), target.double())))
        fd = (vals[0] - vals[1]) / (2 * h)
        g = float(grads[name][idx])
        assert abs(g - fd) <= 0.01 * abs(fd), (name, idx, g, fd)


def test_forward_matches_dropin_in_distribution(small):
    """With the atlas' quantised material values and the RGBE environment
    decoded to FP32, the differentiable renderer and the drop-in pipeline
    render the same image up to Monte Carlo noise (their shading seeds differ
    by construction, and so do their sampling tables: FP32 luma here, RGBE
    bytes there)."""
    src, scene, P, _, _, _, _ = small
    m = src.materials
    q = lambda a: torch.tensor(np.floor(np.clip(a, 0, 1) * 255 + 0.5) / 255, dtype=torch.float32, device="cuda")
    albedo, rough = q(m[:, 0:3]).contiguous(), q(m[:, 4]).contiguous()
    rgbe = np.asarray(src.env_rgbe, np.uint8)
    env = torch.tensor((rgbe[..., :3].astype(np.float32) / 255) * np.ldexp(1.0, rgbe[..., 3].astype(np.int32) - 128)
                       .astype(np.float32)[..., None], device="cuda").contiguous()
    spp = 1024
    from pike_gb300.diff import DiffScene
    ds = DiffScene(src, 64, 48, spp=spp, depth=4)
    ds.set_env_sampling(env)
    got = ds.render(albedo, rough, env, seed=0)[..., :3].double().cpu().numpy()
    ctx = ds.ctx
    ctx.call("pk_env_build", ptr(rgbe), rgbe.shape[1], rgbe.shape[0])
    ctx.call("pk_set_render_state", 0, 0.0)
    ctx.call("pk_render_frames", spp, 4)
    want = np.zeros((48, 64, 4), np.float32)
    ctx.call("pk_read_accum", ptr(want))
    want = want[..., :3].astype(np.float64)
    assert abs(got.mean() / want.mean() - 1) < 0.01, (got.mean(), want.mean())
    bg = got.reshape(6, 8, 8, 8, 3).mean(axis=(1, 3))
    bw = want.reshape(6, 8, 8, 8, 3).mean(axis=(1, 3))
    assert np.abs(bg / bw - 1).max() < 0.05


def test_inverse_rendering_reduces_loss(small):
    """Adam through torch.autograd with fresh, decorrelated samples every step
    (the sampling tables and roughness following the current parameters)
    towards a target rendered with 16x the samples; the L2 error of the
    expected image (estimated from 16 renders) must fall by more than half."""
    from pike_gb300.diff import inverse_render, l2_loss
    src, scene, P, _, _, _, _ = small
    albedo, rough, env = scene.source_params(env_size=(64, 32), sun=5.0)
    scene.set_env_sampling(env)
    target = sum(scene.render(albedo, rough, env, seed=1000 + k) for k in range(16)) / 16
    a0 = torch.full_like(albedo, 0.5)
    r0 = torch.full_like(rough, 0.5)
    e0 = torch.full_like(env, float(env.mean()))

    def bias_loss(a, r, e):
        scene.set_env_sampling(e)
        return float(l2_loss(sum(scene.render(a, r, e, seed=5000 + k) for k in range(16)) / 16, target))

    first = bias_loss(a0, r0, e0)
    a, r, e, hist = inverse_render(scene, target, a0, r0, e0, steps=60, lr=0.05,
                                   n_free=src.materials.shape[0] - 1, seed_per_step=True)
    assert all(np.isfinite(hist))
    last = bias_loss(a, r, e)
    assert last < 0.5 * first, (first, last, hist[-5:])
    assert float(a[-1].sub(0.5).abs().max()) == 0.0  # the fixed box material did not move
