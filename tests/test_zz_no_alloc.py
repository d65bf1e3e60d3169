"""pk_cast_rays_noalloc: the ray query for callers that must not allocate
device memory when they query (a host that gave its memory budget to its own
pool, or a render thread that cannot afford cudaFree's device-wide wait).
Its scratch is a static device array, so it is checked against the allocating
pk_cast_rays on the same rays, bit for bit, over two calls in a row; the
second call is smaller and uses the other hit mode, so stale scratch from the
first call would show.  Kept in a file of its own that pytest collects last."""
import ctypes as C

import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import Context, ptr

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 20


def _scene_context():
    src = synth.displaced_sphere_scene(subdivisions=5, width=16, height=16, env_size=(64, 32))
    ctx = Context(0)
    ctx.call("pk_configure", src.width, src.height, src.width * src.height)
    tr = np.zeros(3)
    ctx.call("pk_scene_flatten", ptr(src.pos), ptr(src.normal), ptr(src.tangent), ptr(src.uv), src.pos.shape[0],
             ptr(src.tris), src.tris.shape[0], 1.0, ptr(tr))
    ctx.call("pk_materials_set", ptr(src.materials), src.materials.shape[0])
    ctx.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
    return ctx


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    o = np.zeros((n, 4), np.float32)
    d = np.zeros((n, 4), np.float32)
    o[:, :3] = rng.uniform(-0.9, 0.9, (n, 3))
    v = rng.normal(size=(n, 3))
    d[:, :3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    return o, d


def _query(ctx, name, o, d, any_hit):
    torch = pytest.importorskip("torch")
    n = o.shape[0]
    to, td = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    hits = torch.full((n, 4), -7, dtype=torch.int32, device="cuda")
    idx = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.call(name, C.c_void_p(to.data_ptr()), C.c_void_p(td.data_ptr()), n, 1 if any_hit else 0,
             C.c_void_p(hits.data_ptr()), C.c_void_p(idx.data_ptr()), C.c_void_p(cnt.data_ptr()))
    k = int(cnt.item())
    return hits.cpu().numpy(), idx[:k].cpu().numpy(), k


def test_noalloc_matches_allocating_query_twice(pk_built):
    ctx = _scene_context()
    for n, any_hit, seed in ((200_000, False, 11), (70_001, True, 12)):
        o, d = _rays(n, seed)
        h_ref, i_ref, k_ref = _query(ctx, "pk_cast_rays", o, d, any_hit)
        h, i, k = _query(ctx, "pk_cast_rays_noalloc", o, d, any_hit)
        assert k == k_ref and 0 < k < n
        # bit-exact, the tolerance of every parity test in this suite
        assert np.array_equal(h, h_ref)
        assert np.array_equal(i, i_ref)


def test_noalloc_leaves_device_memory_unchanged(pk_built):
    """Free device memory is the same before and after each call (after a
    warm-up call): device memory the entry point kept would show as a drop."""
    torch = pytest.importorskip("torch")
    ctx = _scene_context()
    n = 300_000
    o, d = _rays(n, 13)
    to, td = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    hits = torch.zeros((n, 4), dtype=torch.int32, device="cuda")
    idx = torch.zeros((n,), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    args = [C.c_void_p(to.data_ptr()), C.c_void_p(td.data_ptr()), n, 0, C.c_void_p(hits.data_ptr()),
            C.c_void_p(idx.data_ptr()), C.c_void_p(cnt.data_ptr())]
    torch.cuda.synchronize()
    ctx.call("pk_cast_rays_noalloc", *args)  # warm-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        ctx.call("pk_cast_rays_noalloc", *args)
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0
    assert int(cnt.item()) > 0


def test_noalloc_rejects_more_rays_than_its_scratch(pk_built):
    torch = pytest.importorskip("torch")
    ctx = _scene_context()
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    with pytest.raises(_lib.PikeError) as e:
        ctx.call("pk_cast_rays_noalloc", p, p, MAX_RAYS + 1, 0, p, p, p)
    assert e.value.code == _lib.PK_ERR_ARG
    assert "1048576" in ctx.last_error()
