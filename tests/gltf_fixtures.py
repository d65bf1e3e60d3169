"""Writers for the small glTF scenes the ingestion tests load (no glTF assets
ship with the reference).  ``demo_scene(dir)`` writes a scene description with
two props: a ``.gltf`` (external .bin and PNG images) and a ``.glb`` (embedded
image), covering node TRS/matrix hierarchies, textured and constant
materials, a primitive without NORMAL, a primitive without TEXCOORD_0,
u16/u32 indices and the skip lists."""
from __future__ import annotations

import json
import math
import os
import struct

import numpy as np

from pike_gb300 import synth
from pike_gb300.envmap import write_hdr
from pike_gb300.image import encode_png

FLOAT, U16, U32 = 5126, 5123, 5125


class GltfBuilder:
    def __init__(self):
        self.bin = bytearray()
        self.m = {"asset": {"version": "2.0"}, "buffers": [], "bufferViews": [], "accessors": [], "meshes": [],
                  "nodes": [], "scenes": [{"nodes": []}], "scene": 0, "materials": [], "images": []}

    def _view(self, data: bytes) -> int:
        while len(self.bin) % 4:
            self.bin.append(0)
        self.m["bufferViews"].append({"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)})
        self.bin += data
        return len(self.m["bufferViews"]) - 1

    def accessor(self, arr: np.ndarray, comp: int) -> int:
        arr = np.asarray(arr)
        typ = {1: "SCALAR", 2: "VEC2", 3: "VEC3", 4: "VEC4"}[1 if arr.ndim == 1 else arr.shape[1]]
        dt = {FLOAT: "<f4", U16: "<u2", U32: "<u4"}[comp]
        v = self._view(np.ascontiguousarray(arr, dt).tobytes())
        acc = {"bufferView": v, "componentType": comp, "count": int(arr.shape[0]), "type": typ}
        if comp == FLOAT and typ == "VEC3":
            acc["min"] = arr.min(0).tolist()
            acc["max"] = arr.max(0).tolist()
        self.m["accessors"].append(acc)
        return len(self.m["accessors"]) - 1

    def mesh(self, name: str, prims: list) -> int:
        self.m["meshes"].append({"name": name, "primitives": prims})
        return len(self.m["meshes"]) - 1

    def primitive(self, pos, idx, material, normal=None, tangent=None, uv=None, idx_comp=U16) -> dict:
        attrs = {"POSITION": self.accessor(pos, FLOAT)}
        if normal is not None:
            attrs["NORMAL"] = self.accessor(normal, FLOAT)
        if tangent is not None:
            attrs["TANGENT"] = self.accessor(tangent, FLOAT)
        if uv is not None:
            attrs["TEXCOORD_0"] = self.accessor(uv, FLOAT)
        return {"attributes": attrs, "indices": self.accessor(np.asarray(idx).reshape(-1), idx_comp),
                "material": material, "mode": 4}

    def node(self, **kw) -> int:
        self.m["nodes"].append(kw)
        return len(self.m["nodes"]) - 1

    def material(self, **kw) -> int:
        self.m["materials"].append(kw)
        return len(self.m["materials"]) - 1

    def image_uri(self, uri: str) -> int:
        self.m["images"].append({"uri": uri})
        return len(self.m["images"]) - 1

    def image_embedded(self, png: bytes) -> int:
        self.m["images"].append({"bufferView": self._view(png), "mimeType": "image/png"})
        return len(self.m["images"]) - 1

    def write_gltf(self, path: str):
        binname = os.path.splitext(os.path.basename(path))[0] + ".bin"
        self.m["buffers"] = [{"uri": binname, "byteLength": len(self.bin)}]
        with open(os.path.join(os.path.dirname(path), binname), "wb") as f:
            f.write(bytes(self.bin))
        with open(path, "w") as f:
            json.dump(self.m, f)

    def write_glb(self, path: str):
        self.m["buffers"] = [{"byteLength": len(self.bin)}]
        js = json.dumps(self.m).encode()
        js += b" " * (-len(js) % 4)
        bn = bytes(self.bin) + b"\0" * (-len(self.bin) % 4)
        total = 12 + 8 + len(js) + 8 + len(bn)
        with open(path, "wb") as f:
            f.write(struct.pack("<4sII", b"glTF", 2, total))
            f.write(struct.pack("<II", len(js), 0x4E4F534A) + js)
            f.write(struct.pack("<II", len(bn), 0x004E4942) + bn)


def quat(axis, angle):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    s = math.sin(angle / 2)
    return [float(a[0] * s), float(a[1] * s), float(a[2] * s), float(math.cos(angle / 2))]


def checker(n: int, cells: int, c0, c1) -> np.ndarray:
    y, x = np.mgrid[0:n, 0:n]
    m = ((x * cells // n) + (y * cells // n)) % 2
    return np.where(m[..., None] == 0, np.array(c0, np.uint8), np.array(c1, np.uint8)).astype(np.uint8)


def box(lo, hi):
    p, n, t, uv, q = synth._box_faces(lo, hi)
    return p, n, t, uv, synth._quads_to_tris(q)


def demo_scene(d: str, atlas_res: int = 64, env_size=(128, 64)) -> str:
    """Writes the demo scene into directory d; returns the scene description path."""
    rng = np.random.default_rng(1234)
    # ---- room.gltf: floor (textured), box (normal + metal/rough maps), pyramid (no NORMAL, no uv)
    g = GltfBuilder()
    with open(os.path.join(d, "checker.png"), "wb") as f:
        f.write(encode_png(checker(32, 8, (230, 220, 200), (40, 60, 90))))
    nrm = np.stack([rng.integers(100, 156, (16, 16)), rng.integers(100, 156, (16, 16)),
                    np.full((16, 16), 250), np.full((16, 16), 255)], -1).astype(np.uint8)
    with open(os.path.join(d, "normal.png"), "wb") as f:
        f.write(encode_png(nrm))
    mr = np.stack([np.zeros((8, 8)), rng.integers(20, 250, (8, 8)), rng.integers(0, 255, (8, 8))], -1).astype(np.uint8)
    with open(os.path.join(d, "metal_rough.png"), "wb") as f:
        f.write(encode_png(mr))
    i_checker = g.image_uri("checker.png")
    i_normal = g.image_uri("normal.png")
    i_mr = g.image_uri("metal_rough.png")
    m_floor = g.material(name="floor", pbrMetallicRoughness={"baseColorTexture": {"index": i_checker},
                                                             "roughnessFactor": 0.8})
    m_box = g.material(name="box", normalTexture={"index": i_normal},
                       pbrMetallicRoughness={"baseColorFactor": [0.9, 0.35, 0.2, 1.0],
                                             "metallicRoughnessTexture": {"index": i_mr}})
    m_pyr = g.material(name="pyramid", pbrMetallicRoughness={"baseColorFactor": [0.2, 0.7, 0.3, 1.0],
                                                             "metallicFactor": 0.0, "roughnessFactor": 0.5})
    m_skip = g.material(name="skipme", pbrMetallicRoughness={"baseColorFactor": [1, 0, 1, 1]})
    # floor: a 2x2 quad in xz with explicit tangents
    fp = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
    fn = np.tile([0, 1, 0], (4, 1)).astype(np.float32)
    ft = np.tile([1, 0, 0, 1], (4, 1)).astype(np.float32)
    fuv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    floor = g.mesh("floor", [g.primitive(fp, [0, 2, 1, 0, 3, 2], m_floor, fn, ft, fuv)])
    # box: normals from faces, no TANGENT (fallback tangents), u32 indices
    bp, bn, _, buv, bt = box((-0.3, 0.0, -0.3), (0.3, 0.6, 0.3))
    bx = g.mesh("box", [g.primitive(bp.astype(np.float32), bt[:, :3], m_box, bn.astype(np.float32), None,
                                    buv.astype(np.float32), idx_comp=U32)])
    # pyramid: no NORMAL (shared running-mean normal), no TEXCOORD_0
    pp = np.array([[-0.2, 0, -0.2], [0.2, 0, -0.2], [0.0, 0.35, 0.0], [0.2, 0, 0.2], [-0.2, 0, 0.2], [0.0, 0.35, 0.0]],
                  np.float32)
    pyr = g.mesh("pyramid", [g.primitive(pp, [0, 1, 2, 3, 4, 5], m_pyr)])
    hidden = g.mesh("hidden", [g.primitive(fp, [0, 1, 2], m_floor, fn, ft, fuv)])
    skipped = g.mesh("mixed", [g.primitive(fp * 0.1, [0, 1, 2], m_skip, fn, ft, fuv),
                               g.primitive(fp * 0.2 + 0.5, [0, 2, 1], m_pyr, fn, ft, fuv)])
    n_floor = g.node(mesh=floor, scale=[2.0, 1.0, 2.0])
    n_box = g.node(mesh=bx, translation=[0.4, 0.0, -0.2], rotation=quat([0, 0, 1], 0.35))
    mtx = np.eye(4)
    mtx[:3, 3] = [-0.5, 0.0, 0.3]
    n_pyr = g.node(mesh=pyr, matrix=mtx.T.reshape(-1).tolist())
    n_hidden = g.node(mesh=hidden)
    n_mixed = g.node(mesh=skipped, translation=[0.0, 0.01, 0.0])
    root = g.node(children=[n_floor, n_box, n_pyr, n_hidden, n_mixed], translation=[0.0, -0.3, 0.0],
                  rotation=quat([1, 0, 0], 0.05))
    g.m["scenes"][0]["nodes"] = [root]
    g.write_gltf(os.path.join(d, "room.gltf"))
    # ---- lamp.glb: an emissive, textured icosphere with an embedded image
    h = GltfBuilder()
    ip, ifc = synth.icosphere(1)
    ip = ip / np.linalg.norm(ip, axis=1, keepdims=True)
    iuv = np.stack([0.5 + np.arctan2(ip[:, 0], ip[:, 2]) / (2 * np.pi), 0.5 - np.arcsin(ip[:, 1]) / np.pi], 1)
    # the image's bufferView comes after the accessors' views: the loader looks up
    # accessors[bufferView] for strides (gltf_loader.js:325), which must exist
    m_lamp = h.material(name="lamp", emissiveFactor=[1.0, 0.9, 0.7],
                        pbrMetallicRoughness={"baseColorTexture": {"index": 0}})
    lamp = h.mesh("lamp", [h.primitive(ip.astype(np.float32), ifc, m_lamp, ip.astype(np.float32), None,
                                       iuv.astype(np.float32))])
    h.image_embedded(encode_png(checker(8, 2, (255, 200, 120), (120, 160, 255))))
    h.m["scenes"][0]["nodes"] = [h.node(mesh=lamp)]
    h.write_glb(os.path.join(d, "lamp.glb"))
    # ---- environment and scene description
    env = synth.rgbe_encode(synth.hdr_env(77, env_size[0], env_size[1], sigma=1.0, sun=2000.0))
    with open(os.path.join(d, "sky.hdr"), "wb") as f:
        f.write(write_hdr(env))
    desc = {"props": [{"uri": "room.gltf",
                       "transforms": {"rotate": [{"axis": [0, 1, 0], "angle": 0.4}], "scale": 1.0,
                                      "translate": [0, 0, 0]},
                       "skipMeshes": ["hidden"], "skipMaterials": ["skipme"]},
                      {"uri": "lamp.glb",
                       "transforms": {"rotate": [], "scale": 0.15, "translate": [-0.2, 0.45, -0.1]}}],
             "environment": "sky.hdr", "atlasRes": atlas_res}
    path = os.path.join(d, "scene.json")
    with open(path, "w") as f:
        json.dump(desc, f)
    return path
