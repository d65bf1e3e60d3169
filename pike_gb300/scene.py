"""Scene and environment objects of the pass API (render/scene.js, render/env_sampler.js).

``Scene`` holds the glTF-level inputs of ``Scene._createBuffers``
(render/scene.js:120-181): per-vertex positions, normals, signed tangents and
uvs, triangles ``{i0, i1, i2, matId}`` and material factors.  Its
``createBuffers(device)`` flattens them on the GPU (pk_scene_flatten), which
quantises the attributes exactly as scene.js does.  ``EnvironmentGenerator``
holds an RGBE equirect image and builds the luminance histogram, sorted texel
coordinates and pdf of render/env_sampler.js through pk_env_build.
"""
from __future__ import annotations

import numpy as np

from ._lib import ptr


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

    def createBuffers(self, device):
        """Scene._createBuffers on the GPU: quantised attributes + flat tables."""
        device.ctx.call("pk_scene_flatten", ptr(self.pos), ptr(self.normal), ptr(self.tangent), ptr(self.uv),
                        self.numVertices, ptr(self.indices), self.numTriangles, self.scale, ptr(self.translate))

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
