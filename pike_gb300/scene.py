"""Scene and environment objects of the pass API (render/scene.js, render/env_sampler.js).

``Scene`` holds the glTF-level inputs of ``Scene._createBuffers``
(render/scene.js:120-181): per-vertex positions, normals, signed tangents and
uvs, triangles ``{i0, i1, i2, matId}`` and materials, either as constant
factors (synthetic scenes) or as an atlas index table plus packed layers
(``Scene.load`` of a scene description with glTF props).  Its
``createBuffers(device)`` flattens them on the GPU (pk_scene_flatten /
pk_scene_flatten_tbn), which quantises the attributes exactly as scene.js
does.  ``EnvironmentGenerator`` holds an RGBE equirect image and builds the
luminance histogram, sorted texel coordinates and pdf of
render/env_sampler.js through pk_env_build.
"""
from __future__ import annotations

import json
import os

import numpy as np

from ._lib import ptr

# pike.js:33-45 and the CameraController ray of pike.js:65-70
DEFAULT_CAMERA = dict(pos=[0.0, 0.0, 2.0], dir=[0.0, 0.0, -1.0], fov=1.0, focalDepth=0.5, apertureSize=0.0,
                      distortion=0.0, bokeh=0.5, invocationOffset=0)


class Scene:
    def __init__(self, pos, normal, tangent, uv, tris, materials, env_rgbe=None, scale: float = 1.0,
                 translate=(0.0, 0.0, 0.0), name: str = "scene"):
        self.name = name
        self.pos = np.ascontiguousarray(pos, np.float64)
        self.normal = np.ascontiguousarray(normal, np.float64)
        self.tangent = np.ascontiguousarray(tangent, np.float64)
        self.uv = np.ascontiguousarray(uv, np.float64)
        self.indices = np.ascontiguousarray(tris, np.int32)
        self.materials = np.ascontiguousarray(materials, np.float64)
        self.env = None if env_rgbe is None else np.ascontiguousarray(env_rgbe, np.uint8)
        self.scale = float(scale)
        self.translate = np.asarray(translate, np.float64)
        self.lights = []  # emissive boxes; unused by the shaders (shade_hit.wgsl:229-237)
        # set by Scene.load: bitangent sources, atlas index table and layers
        self.bnormal = None
        self.btangent = None
        self.material_index = None
        self.atlas = None
        self.camera = dict(DEFAULT_CAMERA)

    @classmethod
    def from_source(cls, src) -> "Scene":
        """A Scene from a pike_gb300.synth.SceneSource."""
        return cls(src.pos, src.normal, src.tangent, src.uv, src.tris, src.materials, src.env_rgbe, name=src.name)

    @property
    def numVertices(self) -> int:
        return int(self.pos.shape[0])

    @property
    def numTriangles(self) -> int:
        return int(self.indices.shape[0])

    @classmethod
    def load(cls, path: str, fix_tangents: bool = False) -> "Scene":
        """Scene.load (scene.js:17-41) of a scene description file: glTF props,
        their transforms and skip lists, the environment image and atlasRes.
        ``fix_tangents`` replaces the NaN fallback tangent of +-y normals
        (gltf_loader.js:275) with +x; it departs from the reference."""
        from .envmap import load_env
        with open(path, "r") as f:
            desc = json.load(f)
        base = os.path.dirname(os.path.abspath(path))
        from .scene_loader import build_scene_arrays
        arrays = build_scene_arrays(desc, base, fix_tangents=fix_tangents)
        env = None
        if desc.get("environment"):
            env = load_env(os.path.join(base, desc["environment"]))
        sc = cls(arrays["pos"], arrays["normal"], arrays["tangent"], arrays["uv"], arrays["tris"],
                 np.zeros((arrays["material_index"].shape[0], 9)), env,
                 name=os.path.splitext(os.path.basename(path))[0])
        sc.bnormal = arrays["bnormal"]
        sc.btangent = arrays["btangent"]
        sc.material_index = arrays["material_index"]
        sc.atlas = arrays["atlas"]
        sc.lights = arrays["lights"]
        sc.skipped = arrays["skipped"]
        return sc

    def createBuffers(self, device):
        """Scene._createBuffers on the GPU: quantised attributes + flat tables."""
        if self.bnormal is not None:
            device.ctx.call("pk_scene_flatten_tbn", ptr(self.pos), ptr(self.normal), ptr(self.tangent),
                            ptr(self.bnormal), ptr(self.btangent), ptr(self.uv), self.numVertices, ptr(self.indices),
                            self.numTriangles)
            return
        device.ctx.call("pk_scene_flatten", ptr(self.pos), ptr(self.normal), ptr(self.tangent), ptr(self.uv),
                        self.numVertices, ptr(self.indices), self.numTriangles, self.scale, ptr(self.translate))

    def uploadMaterials(self, device):
        """The material index table and atlas of ShadeHitPass (shade_hit_pass.js:58-81)."""
        if self.material_index is None:
            mats = np.ascontiguousarray(self.materials, np.float64)
            device.ctx.call("pk_materials_set", ptr(mats), mats.shape[0])
            return
        idx = np.ascontiguousarray(self.material_index, np.int32)
        atlas = np.ascontiguousarray(self.atlas, np.uint8)
        n_layers, res = int(atlas.shape[0]), int(atlas.shape[1])
        device.ctx.call("pk_materials_upload", ptr(idx), idx.shape[0], ptr(np.zeros((n_layers, 4), np.uint8)),
                        n_layers)
        device.ctx.call("pk_atlas_upload", ptr(atlas), res, n_layers)

    def downloadAttributes(self, device):
        pos = np.zeros((self.numVertices, 3), np.float64)
        attrs = np.zeros((self.numVertices, 4), np.uint32)
        device.ctx.call("pk_scene_download", ptr(pos), ptr(attrs))
        return pos, attrs


class EnvironmentGenerator:
    """env_sampler.js:8-29: importance tables of an RGBE-in-rgba8 equirect image."""

    def __init__(self, img: np.ndarray):
        self.img = np.ascontiguousarray(img, np.uint8)
        self.height, self.width = self.img.shape[:2]
        self.device = None

    @classmethod
    def fromFile(cls, path: str) -> "EnvironmentGenerator":
        """An RGBE PNG (what the reference loads) or a Radiance .hdr file."""
        from .envmap import load_env
        return cls(load_env(path))

    def upload(self, device):
        device.ctx.call("pk_env_build", ptr(self.img), self.width, self.height)
        self.device = device

    def tables(self):
        """(bins (nb,2) i32, coords (N,2) i32, pdf (h,w) f32) as built on the device."""
        ctx = self.device.ctx
        w, h, nb = (np.zeros(1, np.uint32) for _ in range(3))
        ctx.call("pk_env_info", ptr(w), ptr(h), ptr(nb))
        bins = np.zeros((int(nb[0]), 2), np.int32)
        coords = np.zeros((self.width * self.height, 2), np.int32)
        pdf = np.zeros((self.height, self.width), np.float32)
        ctx.call("pk_env_download", ptr(bins), ptr(coords), ptr(pdf))
        return bins, coords, pdf

    # env_sampler.js accessors
    def createHistogramBuffer(self):
        return self.tables()[0]

    def createEnvCoordBuffer(self):
        return self.tables()[1]

    def createPdfTexture(self, device=None):
        return self.tables()[2]
