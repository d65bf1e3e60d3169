"""Form (3): differentiable rendering of the drop-in's estimator through the
path-replay adjoint (pk_diff_render / pk_diff_backward), exposed as a
torch.autograd.Function.

``DiffScene`` owns a library context with the scene, its GPU-built BVH and the
camera (pk_set_camera); ``render(scene, albedo, roughness, env)`` returns the
(H, W, 4) image as a differentiable function of

* ``albedo``    (n_mats, 3) float32 CUDA tensor (base colour),
* ``roughness`` (n_mats,)   float32 CUDA tensor (alpha = roughness^2),
* ``env``       (env_h, env_w, 3) float32 CUDA tensor, equirect radiance.

Metallic values are fixed per material (the scene's).  Sampling is detached:
each forward builds the environment sampling tables from the current ``env``
(pk_diff_set_env_sampling) and samples microfacet normals with the current
roughness, so the image is the drop-in's estimator at the current parameters;
backward replays every path from its seed and returns dLoss/dparams
accumulated in FP64 on the device (cast to the parameters' dtype).  The host
side of a JavaScript binding would wrap the same C calls with the same
contract (forward returns the image, backward maps dL/dimage to parameter
gradients).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Context, camera_struct, ptr


class DiffParams(C.Structure):
    _fields_ = [("albedo3", C.c_void_p), ("roughness", C.c_void_p), ("metallic", C.c_void_p),
                ("roughness_sampling", C.c_void_p), ("n_mats", C.c_uint32), ("env_rgb", C.c_void_p),
                ("env_w", C.c_uint32), ("env_h", C.c_uint32), ("spp", C.c_uint32), ("depth", C.c_uint32),
                ("sample_base", C.c_uint32)]


class DiffScene:
    def __init__(self, src, width: int, height: int, spp: int = 16, depth: int = 4, device: int = 0,
                 camera: dict | None = None, env_theta: float = 0.0):
        import torch
        self.src = src
        self.W, self.H, self.spp, self.depth = int(width), int(height), int(spp), int(depth)
        ctx = Context(device)
        self.ctx = ctx
        ctx.call("pk_configure", self.W, self.H, self.W * self.H)
        tr = np.zeros(3)
        ctx.call("pk_scene_flatten", ptr(np.ascontiguousarray(src.pos)), ptr(np.ascontiguousarray(src.normal)),
                 ptr(np.ascontiguousarray(src.tangent)), ptr(np.ascontiguousarray(src.uv)), src.pos.shape[0],
                 ptr(np.ascontiguousarray(src.tris, np.int32)), src.tris.shape[0], 1.0, ptr(tr))
        mats = np.ascontiguousarray(src.materials, np.float64)
        ctx.call("pk_materials_set", ptr(mats), mats.shape[0])
        from . import _lib
        ctx.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
        self.camera_state = dict(camera or src.camera_state())
        self.env_theta = float(env_theta)
        ctx.call("pk_set_camera", C.byref(camera_struct(self.camera_state)))
        ctx.call("pk_set_render_state", 0, self.env_theta)
        self.n_mats = mats.shape[0]
        self.device = torch.device("cuda", device)
        self.metallic = torch.tensor(mats[:, 5], dtype=torch.float32, device=self.device)
        self.env_shape = None

    def source_params(self, env_size=(256, 128), sun: float = 100.0, sigma: float = 1.0, seed: int = 7):
        """The scene's own albedo/roughness and a seeded env map, as CUDA tensors."""
        import torch
        from . import synth
        m = self.src.materials
        env = synth.hdr_env(synth.SEED_BASE + seed, env_size[0], env_size[1], sigma=sigma, sun=sun)
        t = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device=self.device)
        return t(m[:, 0:3]), t(m[:, 4]), t(env)

    def set_env_sampling(self, env) -> None:
        """Environment sampling tables from this map (held until the next call)."""
        import torch
        e = env.detach().contiguous().to(torch.float32)
        torch.cuda.synchronize(self.device)
        self.ctx.call("pk_diff_set_env_sampling", C.c_void_p(e.data_ptr()), e.shape[1], e.shape[0])
        self.env_shape = tuple(e.shape)

    def env_tables(self):
        """Host copies of the sampling tables: bins (nb, 2), coords (N, 2), pdf (h, w)."""
        w, h, nb = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self.ctx.call("pk_diff_env_info", C.byref(w), C.byref(h), C.byref(nb))
        bins = np.zeros((nb.value, 2), np.int32)
        coords = np.zeros((w.value * h.value, 2), np.int32)
        pdf = np.zeros((h.value, w.value), np.float32)
        self.ctx.call("pk_diff_env_download", ptr(bins), ptr(coords), ptr(pdf))
        return bins, coords, pdf

    def _params(self, albedo, rough, env, seed: int, rough_sampling=None) -> DiffParams:
        assert albedo.is_contiguous() and rough.is_contiguous() and env.is_contiguous()
        assert albedo.shape == (self.n_mats, 3) and rough.shape == (self.n_mats,) and env.dim() == 3
        if self.env_shape != tuple(env.shape):
            self.set_env_sampling(env)
        rs = None
        if rough_sampling is not None:
            assert rough_sampling.is_contiguous() and rough_sampling.shape == rough.shape
            rs = rough_sampling.data_ptr()
        return DiffParams(albedo.data_ptr(), rough.data_ptr(), self.metallic.data_ptr(), rs, self.n_mats,
                          env.data_ptr(), env.shape[1], env.shape[0], self.spp, self.depth, int(seed) * self.spp)

    def render(self, albedo, rough, env, seed: int = 0, rough_sampling=None):
        """(H, W, 4) image: sample s of every pixel uses camera.wgsl's sample
        index seed * spp + s.  rough_sampling (default: rough) is the
        roughness the microfacet normals are sampled with."""
        import torch
        img = torch.empty((self.H, self.W, 4), dtype=torch.float32, device=self.device)
        p = self._params(albedo, rough, env, seed, rough_sampling)
        torch.cuda.synchronize(self.device)
        self.ctx.call("pk_diff_render", C.byref(p), C.c_void_p(img.data_ptr()))
        return img

    def backward(self, albedo, rough, env, dimage, seed: int = 0, rough_sampling=None):
        import torch
        ga = torch.zeros((self.n_mats, 3), dtype=torch.float64, device=self.device)
        gr = torch.zeros((self.n_mats,), dtype=torch.float64, device=self.device)
        ge = torch.zeros(tuple(env.shape), dtype=torch.float64, device=self.device)
        d = dimage.contiguous().to(torch.float32)
        p = self._params(albedo, rough, env, seed, rough_sampling)
        torch.cuda.synchronize(self.device)
        self.ctx.call("pk_diff_backward", C.byref(p), C.c_void_p(d.data_ptr()), C.c_void_p(ga.data_ptr()),
                      C.c_void_p(gr.data_ptr()), C.c_void_p(ge.data_ptr()))
        return ga, gr, ge

    def rays(self) -> int:
        n = C.c_ulonglong(0)
        self.ctx.call("pk_diff_rays", C.byref(n))
        return int(n.value)


def _function():
    import torch

    class PikeRender(torch.autograd.Function):
        @staticmethod
        def forward(ctx, albedo, rough, env, scene, seed, grad_seed):
            ctx.scene, ctx.seed = scene, seed if grad_seed is None else grad_seed
            ctx.save_for_backward(albedo, rough, env)
            scene.set_env_sampling(env)  # detached: the tables follow the current map
            return scene.render(albedo.detach().contiguous(), rough.detach().contiguous(), env.detach().contiguous(),
                                seed)

        @staticmethod
        def backward(ctx, grad_image):
            albedo, rough, env = ctx.saved_tensors
            ga, gr, ge = ctx.scene.backward(albedo.detach().contiguous(), rough.detach().contiguous(),
                                            env.detach().contiguous(), grad_image, ctx.seed)
            return ga.to(albedo.dtype), gr.to(rough.dtype), ge.to(env.dtype), None, None, None

    return PikeRender


_FN = None


def render(scene: DiffScene, albedo, rough, env, seed: int = 0, grad_seed: int | None = None):
    """Differentiable image (H, W, 4) of the scene for these parameters.  The
    backward pass replays the paths of `grad_seed` (default: `seed`).  With an
    independent grad_seed the gradient of a loss that is nonlinear in the
    image, such as L2, is unbiased for the loss of the expected image: with the
    same samples in both passes it also carries the gradient of the image's
    Monte Carlo variance."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(albedo, rough, env, scene, seed, grad_seed)


def l2_loss(image, target):
    return ((image[..., :3] - target[..., :3]) ** 2).mean()


def inverse_render(scene: DiffScene, target, albedo, rough, env, steps: int = 200, lr: float = 0.02,
                   n_free: int | None = None, seed_per_step: bool = True, seed: int = 0, env_floor: float = 1e-3,
                   optimise_env: bool = True, lr_final: float | None = None):
    """Adam on (albedo, roughness, env) towards the target image; materials at
    index >= n_free stay fixed.  With seed_per_step, step k renders with seed
    2k and differentiates with the independent samples of seed 2k + 1
    (decorrelated: unbiased gradients of the expected image's L2 error);
    otherwise every step renders and differentiates `seed` (common random
    numbers: a deterministic objective).  With optimise_env=False the map
    stays as given and only the materials move.  The step size follows a
    cosine from lr to lr_final (default lr / 50), which lets the parameters
    settle under Monte Carlo gradient noise.  Returns the parameters and the
    loss history."""
    import torch
    a = albedo.clone().requires_grad_(True)
    r = rough.clone().requires_grad_(True)
    e = env.clone().requires_grad_(optimise_env)
    opt = torch.optim.Adam([a, r, e] if optimise_env else [a, r], lr=lr)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, T_max=max(steps, 1),
                                                       eta_min=lr / 50 if lr_final is None else lr_final)
    keep = None
    if n_free is not None and n_free < a.shape[0]:
        keep = (a.detach()[n_free:].clone(), r.detach()[n_free:].clone())
    hist = []
    for k in range(steps):
        opt.zero_grad()
        if seed_per_step:
            img = render(scene, a, r, e, seed=seed + 2 * k, grad_seed=seed + 2 * k + 1)
        else:
            img = render(scene, a, r, e, seed=seed)
        loss = l2_loss(img, target)
        loss.backward()
        opt.step()
        sched.step()
        with torch.no_grad():
            a.clamp_(0.0, 1.0)
            r.clamp_(0.05, 1.0)
            e.clamp_(min=env_floor)  # a black map has no sampling tables
            if keep is not None:
                a[n_free:] = keep[0]
                r[n_free:] = keep[1]
        hist.append(float(loss.item()))
    return a.detach(), r.detach(), e.detach(), hist
