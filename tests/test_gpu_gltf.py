"""glTF scenes end to end on the GPU: Scene.load -> pk_scene_flatten_tbn ->
GPU BVH -> textured atlas -> frames, bit for bit against the oracle fed the
same loaded arrays."""
import numpy as np
import pytest

from pike_gb300.passes import GPUDevice
from pike_gb300.renderer import PikeRenderer
from pike_gb300.scene import Scene

from gltf_fixtures import demo_scene
from helpers import assert_bits_equal_nan

pytestmark = pytest.mark.gpu

CAMERA = dict(pos=[0.0, 0.45, 1.7], dir=[0.0, -0.3304, -0.9438], fov=1.0, focalDepth=0.5, apertureSize=0.0,
              distortion=0.0, bokeh=0.5, invocationOffset=0)


@pytest.fixture(scope="module")
def scene_dir(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("gltf_gpu"))
    return demo_scene(d)


@pytest.fixture(scope="module")
def scene(scene_dir):
    return Scene.load(scene_dir)


def oracle_renderer(oracle, sc: Scene, width: int, height: int, camera: dict):
    pos, attrs = oracle.flatten_tbn(sc.pos, sc.normal, sc.tangent, sc.bnormal, sc.btangent, sc.uv)
    bvh = oracle.BVH(pos, sc.indices)
    r = oracle.Renderer(width, height, threads=8)
    n_layers = sc.atlas.shape[0]
    r.set_scene(bvh, attrs, np.ascontiguousarray(sc.material_index, np.int32), np.zeros((n_layers, 4), np.uint8))
    r.set_atlas(sc.atlas)
    r.set_env(oracle.Env(sc.env))
    r.set_camera(camera)
    return r, pos, attrs


def test_flatten_tbn_matches_oracle(oracle, pk_built, scene):
    dev = GPUDevice(0)
    scene.createBuffers(dev)
    pos, attrs = scene.downloadAttributes(dev)
    _, want_pos, want_attrs = oracle_renderer(oracle, scene, 8, 8, CAMERA)
    assert np.array_equal(attrs, want_attrs)
    assert np.array_equal(pos.view(np.uint64), want_pos.view(np.uint64))


@pytest.mark.parametrize("fused,fix", [(True, False), (False, False), (True, True)])
def test_gltf_scene_frames_match_oracle(oracle, pk_built, scene_dir, fused, fix):
    """The lamp's +-y vertex normals get the reference's NaN fallback tangent
    unless fix_tangents is set: NaN shading then reaches the same pixels on
    both sides."""
    scene = Scene.load(scene_dir, fix_tangents=fix)
    w, h, bounces = 160, 120, 4
    r = PikeRenderer(scene, (w, h), CAMERA, device=GPUDevice(0), num_bounces=bounces, fused=fused)
    r.initWebGpu()
    for _ in range(2):
        r.tick()
    acc = r.accumulation()
    o, _, _ = oracle_renderer(oracle, scene, w, h, CAMERA)
    o.set_render_state(0)
    for _ in range(2):
        o.tick(bounces)
    assert_bits_equal_nan(acc, o.accum(), f"glTF scene accumulation (fused={fused}, fix_tangents={fix})")
    assert r.counters()["err"] == 0
    if fix:
        assert np.isfinite(acc).all()
