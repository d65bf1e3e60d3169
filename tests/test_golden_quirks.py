"""Reference-derived known answers (tests/golden/wgsl_quirks.json, made by
tests/golden/make_wgsl_quirks.py from the reference's source text and the
WGSL / JavaScript rules, not from the oracle) checked against the oracle:
rand() returning exactly 1.0 (camera.wgsl:54-56), the NaN fallback tangent
of a +y normal stored as 0 (gltf_loader.js:275, scene.js:104-111), the
environment rotation undone between sampleEnv and envPdf (shade_hit.wgsl:
202-227), the typed-array quantisers of the scene tables, UVs outside
[0, 1] wrapping modulo 2^16 (scene.js:104-118), and a black texel given a
luminance bin of its own (env_sampler.js:74-95)."""
import json
import os

import numpy as np

from gltf_fixtures import GltfBuilder
from pike_gb300.scene_loader import build_scene_arrays

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "wgsl_quirks.json")) as f:
    Q = json.load(f)


def test_rand_returns_one(oracle):
    q = Q["rand_one"]
    seed = (q["px"] * 1973 + q["py"] * 9277 + q["samples"] * 26699) & 0xFFFFFFFF | 1
    first = int(oracle.hash_stream(seed, 1)[0])       # seed = hash(): the output becomes the state
    jitter, jy = (int(v) for v in oracle.hash_stream(first, 2))
    assert first == q["state"] and jitter == q["hash"]
    assert np.float32(np.float32(jitter) / np.float32(4294967296.0)).view(np.uint32) == int(q["rand_f32_bits"], 16)
    # the oracle's camera ray of that pixel: jitter x = 1.0 puts it on the
    # pixel's right edge.  Pinhole camera at the origin looking down +z,
    # fov pi/3, no lens: dir = normalize(-t ux, t uy, 1), t = tan(pi/6).
    W, H = q["px"] + 1, q["py"] + 1
    r = oracle.Renderer(W, H, batch=128, threads=1)
    state = {"pos": [0.0, 0.0, 0.0], "dir": [0.0, 0.0, 1.0], "fov": float(np.pi / 3), "focalDepth": 0.5,
             "apertureSize": 0.0, "distortion": 0.0, "bokeh": 0.5, "invocationOffset": q["py"] * W + q["px"]}
    r.set_camera(state)
    r.set_render_state(q["samples"])
    r.clear_rays()
    r.camera()
    ray = r.rays(0, 1)[0]
    jyf = float(np.float32(np.float32(jy) / np.float32(4294967296.0)))
    ux = (2.0 * ((q["px"] + 1.0) / W) - 1.0) * (W / H)
    uy = -(2.0 * ((q["py"] + jyf) / H) - 1.0)
    t = np.tan(np.pi / 6)
    want = np.array([-t * ux, t * uy, 1.0])
    want /= np.linalg.norm(want)
    assert np.allclose(ray[4:7], want, atol=2e-6), (ray[4:7], want)
    assert ray[11].view(np.uint32) == q["py"] * W + q["px"]  # the pixel index rides in tp.w


def test_nan_fallback_tangent_words(tmp_path, oracle):
    q = Q["nan_tangent"]
    g = GltfBuilder()
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    nrm = np.tile(np.array(q["normal"], np.float32), (3, 1))
    m = g.material(name="m")
    g.m["scenes"][0]["nodes"] = [g.node(mesh=g.mesh("t", [g.primitive(pos, [0, 2, 1], m, nrm)]))]
    g.write_gltf(str(tmp_path / "t.gltf"))
    a = build_scene_arrays({"props": [{"uri": "t.gltf"}]}, str(tmp_path))
    _, attrs = oracle.flatten_tbn(a["pos"], a["normal"], a["tangent"], a["bnormal"], a["btangent"], a["uv"])
    assert (attrs[:, 0] == q["tangent_word"]).all()
    assert (attrs[:, 1] == q["bitangent_word"]).all()
    assert (attrs[:, 2] == q["normal_word"]).all()


def test_env_theta_roundtrip(oracle):
    q = Q["env_theta_roundtrip"]
    w, h = q["w"], q["h"]
    r = oracle.Renderer(4, 4, threads=1)
    rgbe = np.full((h, w, 4), 128, np.uint8)
    r.set_env(oracle.Env(rgbe))
    r.set_render_state(0, q["theta"])
    d, texel = r.env_roundtrip(*q["texel"])
    assert np.allclose(d, q["direction"], atol=1e-6), (d, q["direction"])
    assert list(texel) == q["pdf_texel"]


def test_scene_table_quantizers(oracle):
    from types import SimpleNamespace
    q = Q["quantizers"]
    uv = np.array([e["uv"] for e in q["uv"]], np.float64)
    n = uv.shape[0]
    src = SimpleNamespace(pos=np.zeros((n, 3)), normal=np.tile([0.0, 0.0, 1.0], (n, 1)),
                          tangent=np.tile([1.0, 0.0, 0.0, 1.0], (n, 1)), uv=uv)
    _, attrs = oracle.flatten(src)
    assert [int(w) for w in attrs[:, 3]] == [e["word"] for e in q["uv"]]
    nrm = np.array([e["normal"] for e in q["normal"]], np.float64)
    m = nrm.shape[0]
    src = SimpleNamespace(pos=np.zeros((m, 3)), normal=nrm, tangent=np.tile([1.0, 0.0, 0.0, 1.0], (m, 1)),
                          uv=np.zeros((m, 2)))
    _, attrs = oracle.flatten(src)
    assert [int(w) for w in attrs[:, 2]] == [e["word"] for e in q["normal"]]


def test_env_black_texel_bin(oracle):
    q = Q["env_black_bin"]
    env = oracle.Env(np.array(q["rgbe"], np.uint8))
    assert env.bins.tolist() == q["bins"]
    assert env.coords.tolist() == q["coords"]
    assert (env.pdf.view(np.uint32) == int(q["pdf_f32_bits"], 16)).all()
