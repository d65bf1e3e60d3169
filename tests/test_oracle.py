"""Pins the CPU oracle.

The reference ships no tests or golden vectors for this path and cannot run
here (JavaScript + WGSL on WebGPU), so parity is pinned three ways:
  * known answers computed by hand from the reference formulas;
  * a second, independent restatement in plain Python of the integer/double
    algorithms (hash, WGSL packing, bvh.js sweep SAH + serialisation + packing,
    env_sampler.js tables) that must agree with the C++ oracle exactly;
  * accuracy of the oracle's definitions of the WGSL built-ins against the
    float64 functions of numpy (they are defined, not copied, so they are
    checked against mathematics).
"""
import collections
import math
import struct

import numpy as np
import pytest

from pike_gb300 import synth

M32 = 0xFFFFFFFF


# ---------------- hash (camera.wgsl:46-56) ----------------
def py_hash_stream(seed, n):
    out = []
    for _ in range(n):
        state = seed
        seed = (seed * 747796405 + 2891336453) & M32
        word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & M32
        out.append((word >> 22) ^ word)
    return out


def test_hash_matches_independent_restatement(oracle):
    for seed in (1, 0xDEADBEEF, (5 * 1973 + 7 * 9277 + 3 * 26699) | 1):
        assert list(oracle.hash_stream(seed, 64)) == py_hash_stream(seed, 64)


def test_hash_known_answer(oracle):
    # permute(1): state 1 -> (1 >> 4) ^ 1 = 1 -> 277803737 -> (277803737 >> 22) ^ 277803737
    assert int(oracle.hash_stream(1, 1)[0]) == ((277803737 >> 22) ^ 277803737)


# ---------------- math definitions vs float64 ----------------
def ulp_err(got, want):
    got = got.astype(np.float64)
    spacing = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    return np.abs(got - want) / spacing


@pytest.mark.parametrize("name,lo,hi,fn,tol", [
    ("sin", -100.0, 100.0, np.sin, 2.0),
    ("cos", -100.0, 100.0, np.cos, 2.0),
    ("exp2", -126.0, 127.0, np.exp2, 2.0),
    ("log2", 1e-30, 1e30, np.log2, 3.0),
    ("acos", -1.0, 1.0, np.arccos, 4.0),
])
def test_math_accuracy(oracle, name, lo, hi, fn, tol):
    rng = np.random.default_rng(3)
    x = rng.uniform(lo, hi, 100_000).astype(np.float32)
    if name == "log2":
        x = np.exp2(rng.uniform(-100, 100, 100_000)).astype(np.float32)
    got = oracle.math_fn(name, x)
    want = fn(x.astype(np.float64))
    mask = np.abs(want) > 1e-30
    if name in ("sin", "cos"):  # absolute error near zeros of the function
        assert np.max(np.abs(got - want)) < 2e-7
    else:
        assert np.max(ulp_err(got[mask], want[mask])) <= tol


def test_atan2_and_pow_accuracy(oracle):
    rng = np.random.default_rng(4)
    y = rng.uniform(-5, 5, 100_000).astype(np.float32)
    x = rng.uniform(-5, 5, 100_000).astype(np.float32)
    got = oracle.math_fn("atan2", y, x)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.max(ulp_err(got, want)) <= 3.0
    b = rng.uniform(0, 1, 100_000).astype(np.float32)
    e = np.float32(1.0 / 2.4)
    got = oracle.math_fn("pow", b, np.full_like(b, e))
    want = np.power(b.astype(np.float64), float(e))
    m = want > 1e-30
    assert np.max(ulp_err(got[m], want[m])) <= 8.0  # pow = exp2(y log2 x): error grows with |y log2 x|


def test_math_special_values(oracle):
    f = oracle.math_fn
    x = np.array([0.0, -0.0, np.inf, -np.inf, np.nan], np.float32)
    assert np.isnan(f("sin", x)[2:]).all() and f("sin", x)[0] == 0.0
    assert f("exp2", np.array([0.0, 1.0, -1.0, 10.0, 200.0, -200.0], np.float32)).tolist() == [1.0, 2.0, 0.5, 1024.0, np.inf, 0.0]
    assert f("log2", np.array([1.0, 2.0, 0.5, 1024.0, 0.0], np.float32)).tolist() == [0.0, 1.0, -1.0, 10.0, -np.inf]
    # pow(2, k) = exp2(k * log2(2)) is exact for integers (shade_miss.wgsl:42 decodes RGBE with it)
    k = np.arange(-126, 128, dtype=np.float32)
    assert np.array_equal(f("pow", np.full_like(k, 2.0), k), np.exp2(k.astype(np.float64)).astype(np.float32))
    a = f("atan2", np.array([0.0, 0.0, -0.0, 1.0], np.float32), np.array([1.0, -1.0, -1.0, 0.0], np.float32))
    assert a[0] == 0.0 and a[1] == np.float32(math.pi) and a[2] == -np.float32(math.pi) and a[3] == np.float32(math.pi / 2)


def test_snorm16_decode_fma_form_is_exact():
    """The device decodes snorm16 boxes as fma(fma(-q0, 32767, s), r, q0) with
    q0 = s * r and r = RN(1/32767); with exact rational arithmetic that equals
    the IEEE quotient s / 32767 for all 65536 values."""
    from fractions import Fraction

    def rn32(q):
        c = np.float32(float(q))
        cands = [np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))]
        return min(cands, key=lambda v: (abs(Fraction(float(v)) - q), int(v.view(np.int32)) & 1))

    r = np.float32(1.0) / np.float32(32767.0)
    assert float(r).hex() == "0x1.0002000000000p-15"
    for s in range(-32768, 32768, 7):  # every 7th value here; the GPU test covers all of them
        sf = np.float32(s)
        q0 = sf * r
        e = rn32(Fraction(float(sf)) - Fraction(float(q0)) * 32767)
        q1 = rn32(Fraction(float(e)) * Fraction(float(r)) + Fraction(float(q0)))
        assert q1 == sf / np.float32(32767.0)


# ---------------- bvh.js + trace_pass.js packing, restated in Python ----------------
def js_toint16(v):
    if not math.isfinite(v):
        return 0
    m = int(math.trunc(v)) % 65536
    return m - 65536 if m >= 32768 else m


def py_build_bvh(pos, tris):
    T = len(tris)
    boxes = []
    for t in tris:
        mn, mx = [math.inf] * 3, [-math.inf] * 3
        for k in range(3):
            v = pos[t[k]]
            mn = [min(v[i], mn[i]) for i in range(3)]
            mx = [max(v[i], mx[i]) for i in range(3)]
        boxes.append((mn, mx))
    cent = [[(b[0][a] + b[1][a]) * 0.5 for a in range(3)] for b in boxes]

    def area(mn, mx):
        xl, yl, zl = (max(mx[i] - mn[i], 0.0) for i in range(3))
        return (xl * yl + xl * zl + yl * zl) * 2

    def union(acc, b):
        return ([min(acc[0][i], b[0][i]) for i in range(3)], [max(acc[1][i], b[1][i]) for i in range(3)])

    empty = ([math.inf] * 3, [-math.inf] * 3)
    lists = [sorted(range(T), key=lambda r, a=a: cent[r][a]) for a in range(3)]

    def build(L):
        n = len(L[0])
        bounds = empty
        for r in L[0]:
            bounds = union(bounds, boxes[r])
        psa = area(*bounds)
        best = (math.inf, -1, -1)
        for a in range(3):
            refs = L[a]
            f, b = empty, empty
            af, ab = [], []
            for i in range(n):
                f = union(f, boxes[refs[i]])
                b = union(b, boxes[refs[n - 1 - i]])
                af.append(area(*f))
                ab.append(area(*b))
            for i in range(n):
                cost = 0.5 + (af[i] / psa) * (i + 1) + (ab[n - 1 - i] / psa) * (n - 1 - i)
                if cost < best[0]:
                    best = (cost, i, a)
        cost, idx, axis = best
        node = {"bounds": bounds}
        if cost > n:
            node["leaf"] = list(L[axis])
            return node
        left = set(L[axis][: idx + 1])
        Ls, Rs = [None] * 3, [None] * 3
        for a in range(3):
            Ls[a] = [r for r in L[a] if r in left]
            Rs[a] = [r for r in L[a] if r not in left]
        node["left"], node["right"] = build(Ls), build(Rs)
        return node

    root = build(lists)
    order = []
    q = collections.deque([(root, -1)])
    while q:
        nd, parent = q.popleft()
        me = len(order)
        order.append([nd, parent, -1])
        if "leaf" not in nd:
            q.append((nd["left"], me))
            q.append((nd["right"], me))
    for i, e in enumerate(order):
        if e[1] >= 0 and i % 2 == 1:
            order[e[1]][2] = i
    rmn, rmx = root["bounds"]
    span = [rmx[i] - rmn[i] for i in range(3)]
    longest = max(span)
    center = [rmn[i] + span[i] * 0.5 for i in range(3)]

    def norm(v):
        return [(v[i] - center[i]) * (2 / longest) for i in range(3)]

    def q2(a, b):
        s0 = js_toint16(a * (32767 if a > 0 else 32768))
        s1 = js_toint16(b * (32767 if b > 0 else 32768))
        return struct.unpack("<i", struct.pack("<hh", s0, s1))[0]

    nodes, leaf_tris, tri_index = [], [], 0
    for nd, _, left in order:
        mn, mx = norm(nd["bounds"][0]), norm(nd["bounds"][1])
        if "leaf" in nd:
            word = struct.unpack("<i", struct.pack("<I", ((len(nd["leaf"]) << 24) | tri_index) & M32))[0]
            tri_index += len(nd["leaf"])
            leaf_tris.extend(nd["leaf"])
            head = [-1, word]
        else:
            head = [left, -1]
        nodes.append(head + [q2(mx[0], mn[0]), q2(mx[1], mn[1]), q2(mx[2], mn[2])])
    verts = [[float(np.float32(c)) for c in norm(p)] for p in pos]
    return np.array(nodes, np.int32), np.array([list(tris[t]) for t in leaf_tris], np.int32), np.array(verts, np.float32)


def _small_random_scene(n_tris, seed):
    s = synth.Rng(seed).stream()
    c = s.uniform(3 * n_tris, -5, 5).reshape(n_tris, 3)
    d = s.uniform(9 * n_tris, -0.6, 0.6).reshape(n_tris, 3, 3)
    pos = (c[:, None, :] + d).reshape(-1, 3)
    tris = np.concatenate([np.arange(3 * n_tris).reshape(-1, 3), np.zeros((n_tris, 1), int)], axis=1).astype(np.int32)
    return pos, tris


@pytest.mark.parametrize("n,seed", [(1, 1), (2, 2), (7, 3), (40, 4), (150, 5)])
def test_bvh_matches_python_restatement(oracle, n, seed):
    pos, tris = _small_random_scene(n, seed)
    b = oracle.BVH(pos, tris)
    nodes, ltris, verts = py_build_bvh(pos.tolist(), tris.tolist())
    assert np.array_equal(b.nodes, nodes)
    assert np.array_equal(b.tris, ltris)
    assert np.array_equal(b.verts[:, :3], verts)


def test_bvh_small_scene_matches_python_restatement(oracle):
    src = synth.small_scene()
    pos, _ = oracle.flatten(src)
    b = oracle.BVH(pos, src.tris)
    nodes, ltris, _ = py_build_bvh(pos.tolist(), src.tris.tolist())
    assert np.array_equal(b.nodes, nodes) and np.array_equal(b.tris, ltris)


def test_bvh_two_separated_triangles_known_answer(oracle):
    # two unit triangles far apart on x: the root splits them; two leaves of one triangle
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [10, 0, 0], [11, 0, 0], [10, 1, 0]], float)
    tris = np.array([[0, 1, 2, 0], [3, 4, 5, 0]], np.int32)
    b = oracle.BVH(pos, tris)
    assert b.n_nodes == 3
    assert b.nodes[0, 0] == 1 and b.nodes[0, 1] == -1
    assert b.nodes[1, 0] == -1 and b.nodes[1, 1] == (1 << 24) | 0
    assert b.nodes[2, 0] == -1 and b.nodes[2, 1] == (1 << 24) | 1
    # root box spans x in [0, 11]: normalised to [-1, 1] -> snorm16 max 32767, min -32768
    assert b.nodes[0, 2] == struct.unpack("<i", struct.pack("<hh", 32767, -32768))[0]


def test_bvh_coincident_triangles_make_one_leaf(oracle):
    """bvh.js:137 makes a leaf when the best split costs more than the
    triangle count.  Two copies of one triangle: every box equals the
    parent's, so both candidates cost 0.5 + 1*1 + 1*1 = 2.5 (i = 0) and
    0.5 + 1*2 + 0 = 2.5 (i = 1), both above 2: one leaf of two triangles, in
    input order."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    tris = np.array([[0, 1, 2, 0], [3, 4, 5, 0]], np.int32)
    b = oracle.BVH(pos, tris)
    assert b.n_nodes == 1
    assert b.nodes[0, 0] == -1 and b.nodes[0, 1] == (2 << 24) | 0


def test_bvh_cost_tie_goes_to_x(oracle):
    """bvh.js:194-207 keeps a candidate only when it is strictly cheaper, axes
    in order x, y, z.  Two unit right triangles offset by (5, 5, 0): the
    candidate right box areasBack[n - 1 - i] still holds ref i (the right
    side of split i is refs[i..n-1]), so split 0 costs 0.5 + 2/72 + 72/72 on
    every axis (z included, where both centroids are 0 and the stable sort
    keeps input order) and split 1 costs 2.5; the first, x, wins: the root's
    left child is the triangle at the smaller x."""
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [5, 5, 0], [6, 5, 0], [5, 6, 0]], float)
    tris = np.array([[3, 4, 5, 0], [0, 1, 2, 0]], np.int32)
    b = oracle.BVH(pos, tris)
    assert b.n_nodes == 3
    assert b.nodes[0, 0] == 1 and b.nodes[0, 1] == -1
    # left child: the triangle with the smaller x centroid (input index 1),
    # leaf-ordered first; right child: input index 0
    assert b.nodes[1, 1] == (1 << 24) | 0 and b.nodes[2, 1] == (1 << 24) | 1
    assert [int(v) for v in b.tris[:, 0]] == [0, 3]


# ---------------- env_sampler.js, restated in Python ----------------
def py_env_tables(rgbe):
    h, w = rgbe.shape[:2]
    rad = []
    total, brightest = 0.0, 0.0
    for y in range(h):
        for x in range(w):
            r, g, b, a = (int(v) for v in rgbe[y, x])
            v = math.ldexp(1.0, a - 128) * (0.2126 * r + 0.7152 * g + 0.0722 * b) / 255.0
            brightest = max(v, brightest)
            total += v
            rad.append((v, x, y))
    order = sorted(range(len(rad)), key=lambda i: -rad[i][0])
    nb = min(256, max(32, 2 * math.ceil(total / brightest)))
    size = total / nb
    hist, cur = [], 0.0
    for i, k in enumerate(order):
        if cur >= size:
            hist.append((hist[-1][1] if hist else 0, i))
            cur = 0.0
        cur += rad[k][0]
    hist.append((hist[-1][1], len(order)))
    pdf = np.zeros((h, w), np.float32)
    for h0, h1 in hist:
        for i in range(h0, h1):
            _, x, y = rad[order[i]]
            pdf[y, x] = (1 / len(hist)) * (len(order) / (h1 - h0)) * (1 / (math.pi * math.pi * 2))
    coords = np.array([[rad[k][1], rad[k][2]] for k in order], np.int32)
    return np.array(hist, np.int32), coords, pdf


@pytest.mark.parametrize("w,h,seed", [(16, 8, 1), (64, 32, 2)])
def test_env_tables_match_python_restatement(oracle, w, h, seed):
    rgbe = synth.rgbe_encode(synth.hdr_env(seed, w, h, sun=50.0))
    e = oracle.Env(rgbe)
    bins, coords, pdf = py_env_tables(rgbe)
    assert np.array_equal(e.bins, bins)
    assert np.array_equal(e.coords, coords)
    assert np.array_equal(e.pdf.view(np.uint32), pdf.view(np.uint32))


def test_constant_env_tables(oracle):
    rgbe = np.zeros((32, 64, 4), np.uint8)
    rgbe[...] = (255, 255, 255, 128)
    e = oracle.Env(rgbe)
    # every texel has the same radiance: 256 bins of (nearly) equal counts, uniform pdf
    assert e.bins.shape[0] in (256, 257)
    assert np.allclose(e.pdf, 1.0 / (2 * math.pi ** 2), rtol=0.2)


def test_black_env_is_rejected(oracle):
    with pytest.raises(RuntimeError):
        oracle.Env(np.zeros((4, 8, 4), np.uint8))


# ---------------- attribute quantisation (scene.js:104-118) ----------------
def test_flatten_known_answers(oracle):
    src = synth.small_scene(n_boxes=0)
    pos, attrs = oracle.flatten(src)
    # ground: normal +y -> bytes (0, 127, 0, 0); tangent +x -> (127, 0, 0, 0)
    assert attrs[0, 2] == 127 << 8 and attrs[0, 0] == 127
    # bitangent = normalize(cross(n, t)) = cross(+y, +x) = -z -> byte -128 -> 0x80 in byte 2
    assert attrs[0, 1] == 0x80 << 16
    # uv (0,0) -> 0; uv (1,1) -> 32767 | 32767 << 16
    assert attrs[0, 3] == 0 and attrs[2, 3] == (32767 | (32767 << 16))
    assert np.array_equal(pos, src.pos)


def test_materials_known_answers(oracle):
    mats = np.array([[0.5, 0.5, 0.5, 1.0, 1.0, 0.0, 0, 0, 0], [0.5, 0.5, 0.5, 1.0, 0.25, 1.0, 0, 0, 0]])
    idx, layers = oracle.materials(mats)
    # layers: diffuse, metRough0, normal, emissive, metRough1 (diffuse and normal/emissive shared)
    assert idx.tolist() == [[0, 1, 2, 3], [0, 4, 2, 3]]
    assert layers.tolist() == [[128, 128, 128, 255], [0, 255, 0, 255], [128, 128, 255, 255], [0, 0, 0, 255],
                               [0, 64, 255, 255]]


# ---------------- traversal known answers ----------------
def test_moller_trumbore_known_answer(oracle):
    pos = np.array([[-1, -1, 0], [1, -1, 0], [-1, 1, 0]], float)
    tris = np.array([[0, 1, 2, 0]], np.int32)
    b = oracle.BVH(pos, tris)
    r = oracle.Renderer(4, 4)
    attrs = np.zeros((3, 4), np.uint32)
    r.set_scene(b, attrs, np.zeros((1, 4), np.int32), np.full((1, 4), 255, np.uint8))
    # normalised frame: the triangle spans [-1,1]^2 at z = 0; rays straight down -z from z = 2
    rays = np.array([[-0.5, -0.5, 2.0, 0, 0, 0, -1.0, 0],
                     [0.5, 0.5, 2.0, 0, 0, 0, -1.0, 0],     # outside the hypotenuse
                     [-0.5, -0.5, -2.0, 0, 0, 0, -1.0, 0]],  # behind the origin
                    np.float32)
    out = r.trace_rays(rays)
    t = out[:, 0].view(np.float32)
    assert t[0] == 2.0 and out[0, 1] == 0
    # barycentrics u = v = 0.25 -> pack2x16unorm = floor(0.5 + 65535 * 0.25) = 16384
    assert out[0, 2] == (16384 | (16384 << 16))
    assert out[1, 1] == 0xFFFFFFFF and out[2, 1] == 0xFFFFFFFF
    any_hit = r.trace_rays(rays, any_hit=True)
    assert any_hit[0, 1] == 0 and any_hit[1, 1] == 0xFFFFFFFF
