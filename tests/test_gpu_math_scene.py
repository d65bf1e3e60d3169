"""GPU parity of the arithmetic definitions and of the scene/material/env/BVH
builders against the CPU oracle (bit-exact: these are integer, index and
fixed-expression floating-point results)."""
import numpy as np
import pytest

from pike_gb300 import _lib, synth
from pike_gb300._lib import Context, ptr

from helpers import Pair, assert_bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(pk_built):
    return Context(0)


def _sweep(n, seed=7):
    rng = np.random.default_rng(seed)
    parts = [rng.uniform(-10, 10, n), rng.uniform(-1, 1, n), rng.uniform(0, 1, n), rng.uniform(-200, 200, n),
             np.ldexp(rng.uniform(0.5, 1.0, n), rng.integers(-140, 120, n)), rng.uniform(-150, 130, n)]
    specials = np.array([0.0, -0.0, 1.0, -1.0, 0.5, 2.0, np.pi, -np.pi, np.pi / 2, np.inf, -np.inf, np.nan,
                         1e-45, 1e-38, 3e38, 127.5, 128.0, -150.0, -149.9])
    return np.concatenate(parts + [specials]).astype(np.float32)


@pytest.mark.parametrize("name", ["sin", "cos", "tan", "acos", "exp2", "log2"])
def test_math_unary_bit_exact(ctx, oracle, name):
    x = _sweep(200_000)
    want = oracle.math_fn(name, x)
    got = np.zeros_like(x)
    ctx.call("pk_math_eval", oracle.MATH_FN[name], ptr(x), None, ptr(got), x.size)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert_bits_equal(got[~nan], want[~nan], name)


@pytest.mark.parametrize("name", ["atan2", "pow"])
def test_math_binary_bit_exact(ctx, oracle, name):
    x = _sweep(100_000, 1)
    y = _sweep(100_000, 2)
    if name == "pow":
        x = np.abs(x)
        y = np.clip(y, -40, 40).astype(np.float32)
    want = oracle.math_fn(name, x, y)
    got = np.zeros_like(x)
    ctx.call("pk_math_eval", oracle.MATH_FN[name], ptr(x), ptr(y), ptr(got), x.size)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert_bits_equal(got[~nan], want[~nan], name)


def test_snorm16_decode_all_values(ctx, oracle):
    """The traversal decodes the reference's snorm16 node boxes with a
    reciprocal product and two FMAs; it must equal max(s / 32767, -1) with IEEE
    division for every one of the 65536 values."""
    s = np.arange(-32768, 32768, dtype=np.int32).view(np.float32)
    want = oracle.math_fn("snorm16", s)
    got = np.zeros_like(s)
    ctx.call("pk_math_eval", 8, ptr(s), None, ptr(got), s.size)
    assert_bits_equal(got, want, "snorm16 decode")
    ieee = np.maximum(np.arange(-32768, 32768, dtype=np.float32) / np.float32(32767.0), np.float32(-1.0))
    assert_bits_equal(want, ieee, "oracle snorm16 vs numpy IEEE division")


def test_scene_flatten_matches_oracle(ctx, oracle):
    src = synth.displaced_sphere_scene(subdivisions=4, width=64, height=64)
    pos_o, attrs_o = oracle.flatten(src)
    tr = np.zeros(3)
    ctx.call("pk_configure", 16, 16, 256)
    ctx.call("pk_scene_flatten", ptr(src.pos), ptr(src.normal), ptr(src.tangent), ptr(src.uv), src.pos.shape[0],
             ptr(src.tris), src.tris.shape[0], 1.0, ptr(tr))
    pos = np.zeros_like(pos_o)
    attrs = np.zeros_like(attrs_o)
    ctx.call("pk_scene_download", ptr(pos), ptr(attrs))
    assert np.array_equal(pos.view(np.uint64), pos_o.view(np.uint64))
    assert np.array_equal(attrs, attrs_o)


def test_scene_flatten_quantizer_known_answers(ctx):
    """The GPU scene tables against the reference-derived words of
    tests/golden/wgsl_quirks.json (typed-array stores of scene.js:104-118;
    UVs outside [0, 1] wrap modulo 2^16)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "wgsl_quirks.json")) as f:
        q = json.load(f)["quantizers"]
    uv = np.array([e["uv"] for e in q["uv"]] + [[0.0, 0.0]] * len(q["normal"]), np.float64)
    nrm = np.array([[0.0, 0.0, 1.0]] * len(q["uv"]) + [e["normal"] for e in q["normal"]], np.float64)
    n = uv.shape[0]
    pos = np.ascontiguousarray(np.arange(3 * n, dtype=np.float64).reshape(n, 3))
    tan = np.ascontiguousarray(np.tile([1.0, 0.0, 0.0, 1.0], (n, 1)))
    k3 = n - n % 3
    tris = np.zeros((k3 // 3, 4), np.int32)  # {i0, i1, i2, material}
    tris[:, :3] = np.arange(k3, dtype=np.int32).reshape(-1, 3)
    tr = np.zeros(3)
    ctx.call("pk_configure", 16, 16, 256)
    ctx.call("pk_scene_flatten", ptr(pos), ptr(nrm), ptr(tan), ptr(uv), n, ptr(tris), tris.shape[0], 1.0, ptr(tr))
    pos_d = np.zeros((n, 3), np.float64)
    attrs = np.zeros((n, 4), np.uint32)
    ctx.call("pk_scene_download", ptr(pos_d), ptr(attrs))
    k = len(q["uv"])
    assert [int(w) for w in attrs[:k, 3]] == [e["word"] for e in q["uv"]]
    assert [int(w) for w in attrs[k:, 2]] == [e["word"] for e in q["normal"]]


def test_env_black_texel_bin_known_answer(ctx):
    """The GPU env tables against the reference-derived bins, coordinates and
    pdf of tests/golden/wgsl_quirks.json (a black texel gets a bin of its
    own, env_sampler.js:74-95)."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "wgsl_quirks.json")) as f:
        q = json.load(f)["env_black_bin"]
    rgbe = np.ascontiguousarray(np.array(q["rgbe"], np.uint8))
    h, w = rgbe.shape[:2]
    ctx.call("pk_env_build", ptr(rgbe), w, h)
    ww, hh, nb = (np.zeros(1, np.uint32) for _ in range(3))
    ctx.call("pk_env_info", ptr(ww), ptr(hh), ptr(nb))
    assert int(nb[0]) == len(q["bins"])
    bins = np.zeros((len(q["bins"]), 2), np.int32)
    coords = np.zeros((w * h, 2), np.int32)
    pdf = np.zeros((h, w), np.float32)
    ctx.call("pk_env_download", ptr(bins), ptr(coords), ptr(pdf))
    assert bins.tolist() == q["bins"] and coords.tolist() == q["coords"]
    assert (pdf.view(np.uint32) == int(q["pdf_f32_bits"], 16)).all()


def test_materials_match_oracle(ctx, oracle):
    src = synth.displaced_sphere_scene(subdivisions=2, width=8, height=8)
    idx_o, layers_o = oracle.materials(src.materials)
    ctx.call("pk_materials_set", ptr(src.materials), src.materials.shape[0])
    nm, nl = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    ctx.call("pk_materials_download", ptr(nm), ptr(nl), None, None)
    idx = np.zeros((int(nm[0]), 4), np.int32)
    layers = np.zeros((int(nl[0]), 4), np.uint8)
    ctx.call("pk_materials_download", ptr(nm), ptr(nl), ptr(idx), ptr(layers))
    assert np.array_equal(idx, idx_o)
    assert np.array_equal(layers, layers_o)


@pytest.mark.parametrize("size", [(64, 32), (2048, 1024), "constant", "banded"])
def test_env_tables_match_oracle(ctx, oracle, size):
    """GPU env tables (radiance, stable descending sort, sequential bin walk,
    pdf) equal env_sampler.js's, including environments full of equal texels."""
    if size == "constant":
        w, h = 64, 32
        rgbe = np.zeros((h, w, 4), np.uint8)
        rgbe[...] = (255, 255, 255, 128)
    elif size == "banded":
        w, h = 300, 150
        rgbe = synth.rgbe_encode(synth.hdr_env(77, w, h, sun=500.0))
        rgbe[::3] = rgbe[0, 0]
    else:
        w, h = size
        rgbe = synth.rgbe_encode(synth.hdr_env(1234, w, h))
    env = oracle.Env(rgbe)
    ctx.call("pk_env_build", ptr(rgbe), w, h)
    ww, hh, nb = (np.zeros(1, np.uint32) for _ in range(3))
    ctx.call("pk_env_info", ptr(ww), ptr(hh), ptr(nb))
    assert int(nb[0]) == env.bins.shape[0]
    bins = np.zeros_like(env.bins)
    coords = np.zeros_like(env.coords)
    pdf = np.zeros_like(env.pdf)
    ctx.call("pk_env_download", ptr(bins), ptr(coords), ptr(pdf))
    assert np.array_equal(bins, env.bins)
    assert np.array_equal(coords, env.coords)
    assert_bits_equal(pdf, env.pdf, "pdf")


def _bvh_case(ctx, oracle, src):
    pos_o, _ = oracle.flatten(src)
    ref = oracle.BVH(pos_o, src.tris)
    tr = np.zeros(3)
    ctx.call("pk_configure", 16, 16, 256)
    ctx.call("pk_scene_flatten", ptr(src.pos), ptr(src.normal), ptr(src.tangent), ptr(src.uv), src.pos.shape[0],
             ptr(src.tris), src.tris.shape[0], 1.0, ptr(tr))
    ctx.call("pk_bvh_build", _lib.PK_BVH_SWEEP)
    nn, nt = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
    norm = np.zeros(4)
    ctx.call("pk_bvh_info", ptr(nn), ptr(nt), ptr(norm))
    assert int(nn[0]) == ref.n_nodes and int(nt[0]) == ref.n_leaf_tris
    nodes = np.zeros_like(ref.nodes)
    tris = np.zeros_like(ref.tris)
    verts = np.zeros_like(ref.verts)
    ctx.call("pk_bvh_download", ptr(nodes), ptr(tris), ptr(verts))
    assert np.array_equal(nodes[:, :2], ref.nodes[:, :2]), "topology / leaf words differ"
    assert np.array_equal(nodes, ref.nodes), "quantised boxes differ"
    assert np.array_equal(tris, ref.tris), "leaf triangle order differs"
    assert_bits_equal(verts, ref.verts, "normalised vertices")
    assert np.array_equal(norm[:3].view(np.uint64), ref.center.view(np.uint64))


def test_bvh_small_scene_matches_oracle(ctx, oracle):
    _bvh_case(ctx, oracle, synth.small_scene())


def test_bvh_single_triangle(ctx, oracle):
    src = synth.small_scene(n_boxes=0)
    src.tris = src.tris[:1].copy()
    _bvh_case(ctx, oracle, src)


def test_bvh_sphere_matches_oracle(ctx, oracle):
    _bvh_case(ctx, oracle, synth.displaced_sphere_scene(subdivisions=5, width=8, height=8))


def test_bvh_soup_matches_oracle(ctx, oracle):
    _bvh_case(ctx, oracle, synth.triangle_soup_scene(n_tris=200_000, width=8, height=8, env_size=(64, 32)))


@pytest.mark.slow
def test_bvh_full_sphere_matches_oracle(ctx, oracle):
    _bvh_case(ctx, oracle, synth.displaced_sphere_scene(subdivisions=8, width=8, height=8, env_size=(64, 32)))


@pytest.mark.parametrize("fn,lo,hi,div,signed", [(9, -128, 127, 127.0, True), (10, 0, 255, 255.0, False),
                                                 (11, 0, 65535, 65535.0, False),
                                                 (12, -32768, 32767, 32767.0, True)])
def test_integer_decodes_all_values(ctx, fn, lo, hi, div, signed):
    """snorm8, unorm8, unorm16 and snorm16 decode with a reciprocal product and
    one FMA; each must equal the IEEE quotient (max(v / d, -1) when signed)
    for every value of its domain."""
    v = np.arange(lo, hi + 1, dtype=np.int32)
    got = np.zeros(v.size, np.float32)
    ctx.call("pk_math_eval", fn, ptr(v.view(np.float32)), None, ptr(got), v.size)
    want = v.astype(np.float32) / np.float32(div)
    if signed:
        want = np.maximum(want, np.float32(-1.0))
    assert_bits_equal(got, want, f"decode fn {fn}")
