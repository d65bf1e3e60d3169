"""glTF + texture ingestion on the CPU: the vector.js matrix helpers against
the reference's own known answers, the loader's behaviour (including its
quirks), the texture packer, and the flattened arrays against the oracle."""
import json
import math
import os

import numpy as np
import pytest

from pike_gb300 import atlas, gltf
from pike_gb300.scene import Scene
from pike_gb300.scene_loader import build_scene_arrays

from gltf_fixtures import GltfBuilder, U16, demo_scene, quat


def close(a, b, tol=0.001):
    """Vec.eq (vector.js:37-47): same length and every component within 0.001."""
    return len(a) == len(b) and all(abs(x - y) <= tol for x, y in zip(a, b))


# ---- vector.js test() (vector.js:284-360): the reference's own known answers
Q45 = [0.3826834, 0, 0, 0.9238795]


def test_vector_known_answers():
    V = gltf
    m = V.compose_trs([1, 1, 1], [0, 0, 0, 1], [3, 3, 3])
    assert close(V.mat_vec_multiply(m, [0, 1, 0]), [1, 4, 1])
    m = V.compose_trs([0, 0, 0], Q45, [1, 1, 1])
    assert close(V.mat_vec_multiply(m, [0, 0.707, -0.707]), [0, 1, 0])
    r = V.compose_trs([0, 0, 0], Q45, [1, 1, 1])
    assert close(r, V.transpose_matrix(V.invert_matrix(r)))
    r = V.compose_trs([1, 1, 1], Q45, [3, 3, 3])
    assert close(r, V.invert_matrix(V.invert_matrix(r)))
    tr = V.compose_trs([1, 1, 1], [0, 0, 0, 1], [1, 1, 1])
    sc = V.compose_trs([0, 0, 0], [0, 0, 0, 1], [3, 3, 3])
    assert close(V.mat_multiply(tr, sc), V.compose_trs([1, 1, 1], [0, 0, 0, 1], [3, 3, 3]))
    rot = V.compose_trs([0, 0, 0], Q45, [1, 1, 1])
    assert close(V.mat_multiply(tr, rot), V.compose_trs([1, 1, 1], Q45, [1, 1, 1]))
    assert close(V.mat_multiply(tr, V.mat_multiply(rot, sc)), V.compose_trs([1, 1, 1], Q45, [3, 3, 3]))


def test_vector_helpers_match_numpy():
    rng = np.random.default_rng(3)
    for _ in range(20):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        t, s = rng.normal(size=3), rng.uniform(0.5, 2, size=3)
        m = gltf.compose_trs(t, q, s)
        M = np.array(m).reshape(4, 4).T  # column-major
        assert np.allclose(np.array(gltf.invert_matrix(m)).reshape(4, 4).T, np.linalg.inv(M), atol=1e-12)
        v = rng.normal(size=(5, 3))
        got = gltf.mat_vec_multiply_rows(m, v)
        want = (M @ np.concatenate([v, np.ones((5, 1))], 1).T).T[:, :3]
        assert np.allclose(got, want, atol=1e-12)
        assert np.array_equal(got[0], np.array(gltf.mat_vec_multiply(m, v[0].tolist())))
        # rotateArbitrary applies the transpose of the matrix it lists: a rotation by -angle
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = float(rng.uniform(-3, 3))
        r = gltf.rotate_arbitrary_rows(v, axis, ang)
        m2 = gltf.compose_trs([0, 0, 0], list(axis * math.sin(-ang / 2)) + [math.cos(-ang / 2)], [1, 1, 1])
        assert np.allclose(r, gltf.mat_vec_multiply_rows(m2, v), atol=1e-12)


# ---- loader
@pytest.fixture(scope="module")
def demo(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("gltf"))
    return d, demo_scene(d)


def test_loader_node_hierarchy_and_attributes(demo):
    d, _ = demo
    g = gltf.GLTFLoader().load(os.path.join(d, "room.gltf"))
    assert [m.name for m in g.meshes] == ["floor", "box", "pyramid", "hidden", "mixed"]
    with open(os.path.join(d, "room.gltf")) as f:
        man = json.load(f)
    nodes = man["nodes"]
    root = nodes[-1]
    R = np.array(gltf.compose_trs(root["translation"], root["rotation"], [1, 1, 1])).reshape(4, 4).T
    box = g.meshes[1]
    nb = nodes[1]
    B = R @ np.array(gltf.compose_trs(nb["translation"], nb["rotation"], [1, 1, 1])).reshape(4, 4).T
    assert np.allclose(np.array(box.matrix).reshape(4, 4).T, B, atol=1e-15)
    prim = box.primitives[0]
    p_local = prim._values(prim.desc["attributes"]["POSITION"], 0, prim.attributeCount())
    p = prim.positions(0, prim.attributeCount())
    assert np.allclose(p, (B @ np.c_[p_local, np.ones(len(p_local))].T).T[:, :3], atol=1e-12)
    # normals through transpose(inverse(M)) and fallback tangents (no TANGENT accessor)
    n = prim.normals(prim.attributeCount())
    t = prim.tangents(prim.attributeCount(), n)
    assert t.shape[1] == 3 and np.isfinite(t).all()
    # an explicit node matrix is used as given (pyramid)
    assert np.allclose(np.array(g.meshes[2].matrix).reshape(4, 4).T,
                       R @ np.array(nodes[2]["matrix"]).reshape(4, 4).T, atol=1e-15)


def test_computed_normals_share_one_running_mean(demo):
    """gltf_loader.js:239 fills the array with one object: every vertex gets the
    normalised mean of all face normals of consecutive position triples."""
    d, _ = demo
    g = gltf.GLTFLoader().load(os.path.join(d, "room.gltf"))
    prim = g.meshes[2].primitives[0]
    n = prim.attributeCount()
    p = prim.positions(0, n)
    faces = [np.cross(p[i + 1] - p[i], p[i + 2] - p[i]) for i in range(0, n, 3)]
    mean = np.mean(faces, 0)
    want = mean / np.linalg.norm(mean)
    assert np.allclose(prim.shared_normal, want, atol=1e-12)
    normals = prim.normals(n)
    assert np.allclose(normals, normals[0], atol=0) and np.all(normals == normals[0])
    assert np.allclose(prim.uvs(n), 0.5)  # no TEXCOORD_0


def test_scene_load_tables(demo):
    d, path = demo
    sc = Scene.load(path)
    # floor 2 + box 12 + pyramid 2 + the kept primitive of "mixed" 1 + lamp 80
    assert sc.numTriangles == 97
    assert sc.skipped == 2  # the "hidden" mesh and the "skipme" primitive
    # one material per primitive; layers deduplicated by colour key and image source
    # (the lamp's metal/rough colour [0, 0, 0] has the key of the black emission layer 3)
    assert sc.material_index.tolist() == [[0, 1, 2, 3], [4, 5, 6, 3], [7, 8, 2, 3], [7, 8, 2, 3], [9, 3, 2, 10]]
    assert sc.atlas.shape == (11, 32, 32, 4)  # res = min(atlasRes 64, tallest texture 32)
    assert np.all(sc.atlas[2] == np.array([128, 128, 255, 255], np.uint8))  # the [0.5, 0.5, 1] normal colour
    assert np.all(sc.atlas[3] == np.array([0, 0, 0, 255], np.uint8))
    assert np.all(sc.atlas[1] == np.array([0, 204, 0, 255], np.uint8))  # [0, roughness 0.8, metal 0]
    assert sc.indices[:, 3].tolist() == [0] * 2 + [1] * 12 + [2] * 2 + [3] + [4] * 80
    assert sc.env is not None and sc.env.shape == (64, 128, 4)
    assert len(sc.lights) == 1  # the emissive lamp


def test_glb_matches_gltf(tmp_path):
    g = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.5]], np.float32)
    m = g.material(name="m", pbrMetallicRoughness={"baseColorFactor": [0.5, 0.5, 0.5, 1]})
    nrm = np.tile([0, 0, 1], (4, 1)).astype(np.float32)
    me = g.mesh("q", [g.primitive(pos, [0, 1, 2, 1, 3, 2], m, nrm, uv=pos[:, :2]),
                      g.primitive(pos, [0, 1, 2, 1, 3, 2], m, uv=pos[:, :2])])
    g.m["scenes"][0]["nodes"] = [g.node(mesh=me, translation=[1, 2, 3], rotation=quat([0, 1, 0], 0.7))]
    g.write_gltf(str(tmp_path / "a.gltf"))
    g.write_glb(str(tmp_path / "a.glb"))
    ga = gltf.GLTFLoader().load(str(tmp_path / "a.gltf"))
    gb = gltf.GLTFLoader().load(str(tmp_path / "a.glb"))
    # The second primitive has no NORMAL: _computeNormals reads positions 0..5 of a
    # 4-position view, the DataView read throws and the primitive is dropped.
    assert len(ga.meshes[0].primitives) == len(gb.meshes[0].primitives) == 1
    pa, pb = ga.meshes[0].primitives[0], gb.meshes[0].primitives[0]
    assert np.array_equal(pa.positions(0, 4), pb.positions(0, 4))
    assert np.array_equal(pa.normals(4), pb.normals(4))


def test_missing_materials_array_drops_primitives(tmp_path):
    """materialDescAt throws inside the primitive constructor, which the mesh
    constructor swallows (gltf_loader.js:351-357)."""
    g = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    me = g.mesh("t", [g.primitive(pos, [0, 1, 2], None)])
    g.m["scenes"][0]["nodes"] = [g.node(mesh=me)]
    del g.m["materials"]
    g.write_gltf(str(tmp_path / "t.gltf"))
    loaded = gltf.GLTFLoader().load(str(tmp_path / "t.gltf"))
    assert loaded.meshes[0].primitives == [] and loaded.meshes[0].dropped == 1
    with open(tmp_path / "s.json", "w") as f:
        json.dump({"props": [{"uri": "t.gltf"}]}, f)
    with pytest.raises(gltf.GLTFError):
        Scene.load(str(tmp_path / "s.json"))


def test_primitive_without_material_fails_the_load(tmp_path):
    """material.hasEmissive() on an undefined desc throws in scene.js:137."""
    g = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    g.material(name="unused")
    prim = g.primitive(pos, [0, 1, 2], 0)
    del prim["material"]
    g.m["scenes"][0]["nodes"] = [g.node(mesh=g.mesh("t", [prim]))]
    g.write_gltf(str(tmp_path / "t.gltf"))
    with pytest.raises(gltf.GLTFError):
        build_scene_arrays({"props": [{"uri": "t.gltf"}]}, str(tmp_path))


def test_jpeg_images_are_rejected(tmp_path):
    g = GltfBuilder()
    with open(tmp_path / "x.jpg", "wb") as f:
        f.write(b"\xff\xd8\xff\xe0" + b"\0" * 16)
    g.image_uri("x.jpg")
    g.write_gltf(str(tmp_path / "j.gltf"))
    with pytest.raises(gltf.GLTFError, match="JPEG"):
        gltf.GLTFLoader().load(str(tmp_path / "j.gltf"))


def test_fallback_tangent_quirk_and_fix(tmp_path, oracle):
    """normalize(cross(+y, +y)) is NaN (gltf_loader.js:275); the quantiser
    stores NaN as 0.  fix_tangents substitutes +x."""
    g = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    nrm = np.tile([0, 1, 0], (3, 1)).astype(np.float32)
    m = g.material(name="m")
    g.m["scenes"][0]["nodes"] = [g.node(mesh=g.mesh("t", [g.primitive(pos, [0, 2, 1], m, nrm)]))]
    g.write_gltf(str(tmp_path / "t.gltf"))
    for fix in (False, True):
        a = build_scene_arrays({"props": [{"uri": "t.gltf"}]}, str(tmp_path), fix_tangents=fix)
        assert np.isnan(a["tangent"][:, :3]).any() != fix
        _, attrs = oracle.flatten_tbn(a["pos"], a["normal"], a["tangent"], a["bnormal"], a["btangent"], a["uv"])
        assert (attrs[:, 0] == 0).all() != fix


def test_flatten_tbn_equals_flatten_without_rotations(oracle):
    from pike_gb300 import synth
    src = synth.small_scene(width=8, height=8)
    pos, attrs = oracle.flatten(src)
    pos2, attrs2 = oracle.flatten_tbn(src.pos, src.normal, src.tangent, src.normal, src.tangent, src.uv)
    assert np.array_equal(attrs, attrs2)
    assert np.array_equal(pos, pos2)


# ---- texture packer
def test_packer_index_zero_quirk():
    """`if (this.imageKeys[src])` misses the image stored at index 0
    (texture_packer.js:87-88): it is pushed again, later lookups find the copy."""
    p = atlas.TexturePacker(16)
    img = atlas.AtlasImage(np.zeros((4, 4, 4), np.uint8), "a.png")
    other = atlas.AtlasImage(np.zeros((8, 8, 4), np.uint8), "b.png")
    assert p.addTexture(img, True) == 0
    assert p.addColor([0.5, 0.5, 1]) == 1
    assert p.addTexture(other) == 2
    assert p.addTexture(other) == 2
    assert p.addTexture(img) == 3  # index 0 is falsy
    assert p.addTexture(img) == 3
    assert p.addColor([0.5, 0.5, 1]) == 1
    assert p.addColor([0.5, 0.5, 1.0, 1]) == 4  # a different key ("0.5 0.5 1 1")
    assert p.getResolution() == [8, 8, 5]  # min(atlasRes, tallest texture)
    assert img.corrected is False  # the second addTexture re-set the shared flag


def test_draw_texture_identity_and_srgb():
    rng = np.random.default_rng(5)
    px = rng.integers(0, 256, (16, 16, 4), dtype=np.uint8)
    img = atlas.AtlasImage(px, "x")
    assert np.array_equal(atlas.draw_texture(img, 16), px)  # texel centres hit exactly
    img.corrected = True
    out = atlas.draw_texture(img, 16)
    assert np.array_equal(out[..., 3], px[..., 3])
    assert np.array_equal(out[..., :3], atlas.unorm8(atlas.SRGB_TO_LINEAR[px[..., :3]]))
    assert atlas.SRGB_TO_LINEAR[0] == 0.0 and atlas.SRGB_TO_LINEAR[255] == 1.0


def test_draw_texture_bilinear_wrap_and_clamp():
    """Magnifying 2x2 -> 4x4: S repeats (column 0 mixes with column 1 across the
    edge), T clamps (row 0 keeps the first row)."""
    px = np.zeros((2, 2, 4), np.uint8)
    px[0, 0, 0], px[0, 1, 0], px[1, 0, 0], px[1, 1, 0] = 0, 200, 40, 240
    out = atlas.draw_texture(atlas.AtlasImage(px, "w"), 4)[..., 0].astype(float)
    # u = 0.125 -> x = -0.25: 0.25 * texel(-1 -> column 1) + 0.75 * column 0
    # v = 0.125 -> y = -0.25: clamped rows, both row 0
    assert out[0, 0] == np.floor((0.75 * 0 + 0.25 * 200) + 0.5)
    assert out[0, 3] == np.floor((0.25 * 0 + 0.75 * 200) + 0.5)
    assert out[3, 0] == np.floor((0.75 * 40 + 0.25 * 240) + 0.5)
    # v = 0.375 -> y = 0.25: 0.75 row 0 + 0.25 row 1
    want = 0.75 * (0.75 * 0 + 0.25 * 200) + 0.25 * (0.75 * 40 + 0.25 * 240)
    assert out[1, 0] == np.floor(want + 0.5)


def test_draw_color_rounding():
    c = atlas.draw_color([0.5, 1.2, -1, 0.3], 2)
    assert c.shape == (2, 2, 4) and (c[..., 3] == 255).all()
    assert c[0, 0, :3].tolist() == [128, 255, 0]
