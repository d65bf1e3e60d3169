"""glTF 2.0 ingestion: GLTFLoader (render/util/gltf_loader.js:28-370) and the
matrix helpers it uses (render/util/vector.js:1-150).

The loader keeps the reference's behaviour, including what it gets wrong,
because the flattened scene (and so every rendered bit) depends on it:

* accessor strides come from ``accessors[bufferView].byteStride``
  (gltf_loader.js:325), which is never set, so every accessor is read tightly
  packed and a bufferView's ``byteStride`` is ignored;
* a texture reference's ``index`` addresses ``images`` directly, not
  ``textures`` (:137-138, :148-150, :163-166, :171-173);
* without NORMAL, one shared ``{n, count}`` object receives every face normal
  (``new Array(n).fill({...})``, :239), so every vertex gets the normalised
  running mean of all face normals, where the faces are taken from consecutive
  position triples (``positionAt(i)``, not ``indexAt(i)``, :293-297);
* normals and tangents go through ``transpose(invert(M))`` with the vector
  padded by w = 1 (:253-266, vector.js:66-78), so a 4-component TANGENT's w
  picks up the inverse's translation; the fallback tangent
  ``normalize(cross(n, [0, 1, 0]))`` is NaN for n = +-y (:268-279) unless the
  caller asks for ``fix_tangents`` (not the reference's behaviour);
* errors inside a primitive's constructor drop the primitive (:351-357);
  errors elsewhere fail the load (:class:`GLTFError`).

Scalar arithmetic is IEEE double in the reference's operation order; the
per-vertex loops are numpy expressions with that order, which gives the same
doubles.  Images are decoded to rgba8 (PNG: pike_gb300.image.decode_png).
Beyond the reference: ``.glb`` containers, ``data:`` URIs, images stored in
buffer views, and a missing ``scene`` index (scene 0).
"""
from __future__ import annotations

import base64
import json
import math
import os
import struct

import numpy as np

from .atlas import AtlasImage

INT16, UINT16, UINT32, FLOAT32 = 5122, 5123, 5125, 5126
STRIDE = {INT16: 2, UINT16: 2, UINT32: 4, FLOAT32: 4}
_DTYPE = {INT16: "<i2", UINT16: "<u2", UINT32: "<u4", FLOAT32: "<f4"}
TRIANGLES = 4
ELEMENT_COUNT = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4}


class GLTFError(RuntimeError):
    """What makes the reference's scene load throw."""


class _JsError(Exception):
    """A TypeError/RangeError/Error the reference would raise at this point."""


# ---------------------------------------------------------------- vector.js
def vec_dot(v1, v2) -> float:
    res = 0.0
    for a, b in zip(v1, v2):
        res += a * b
    return res


def mat_vec_multiply(mat, v) -> list:
    """Vec.matVecMultiply (vector.js:66-78): column-major M * [v, pad to (0,0,0,1)]."""
    padded = [0.0, 0.0, 0.0, 1.0]
    padded[:len(v)] = list(v)
    res = [vec_dot([mat[4 * j + i] for j in range(4)], padded) for i in range(4)]
    return res[:len(v)]


def mat_vec_multiply_rows(mat, v: np.ndarray) -> np.ndarray:
    """mat_vec_multiply over rows of v (N, k), same operation order."""
    n, k = v.shape
    pad = np.zeros((n, 4), np.float64)
    pad[:, 3] = 1.0
    pad[:, :k] = v
    out = np.empty((n, 4), np.float64)
    for i in range(4):
        r = np.zeros(n, np.float64)
        for j in range(4):
            r = r + float(mat[4 * j + i]) * pad[:, j]
        out[:, i] = r
    return out[:, :k]


def mat_multiply(m1, m2) -> list:
    """Vec.matMultiply (vector.js:53-64): m1 * m2, column-major."""
    res = []
    for i in range(4):
        res.extend(mat_vec_multiply(m1, [m2[4 * i + j] for j in range(4)]))
    return res


def compose_trs(t, q, s) -> list:
    """Vec.composeTRSMatrix (vector.js:81-106)."""
    x, y, z, w = (float(c) for c in q)
    x2, y2, z2 = x + x, y + y, z + z
    xx, xy, xz = x * x2, x * y2, x * z2
    yy, yz, zz = y * y2, y * z2, z * z2
    wx, wy, wz = w * x2, w * y2, w * z2
    sx, sy, sz = (float(c) for c in s)
    return [(1 - (yy + zz)) * sx, (xy + wz) * sx, (xz - wy) * sx, 0.0,
            (xy - wz) * sy, (1 - (xx + zz)) * sy, (yz + wx) * sy, 0.0,
            (xz + wy) * sz, (yz - wx) * sz, (1 - (xx + yy)) * sz, 0.0,
            float(t[0]), float(t[1]), float(t[2]), 1.0]


def transpose_matrix(mm) -> list:
    """Vec.transposeMatrix (vector.js:109-119)."""
    m = [float(v) for v in mm]
    for a, b in ((1, 4), (2, 8), (6, 9), (3, 12), (7, 13), (11, 14)):
        m[a], m[b] = m[b], m[a]
    return m


def invert_matrix(mm) -> list:
    """Vec.invertMatrix (vector.js:122-149), with its term order."""
    m = [float(v) for v in mm]
    n11, n21, n31, n41, n12, n22, n32, n42, n13, n23, n33, n43, n14, n24, n34, n44 = m
    t11 = n23 * n34 * n42 - n24 * n33 * n42 + n24 * n32 * n43 - n22 * n34 * n43 - n23 * n32 * n44 + n22 * n33 * n44
    t12 = n14 * n33 * n42 - n13 * n34 * n42 - n14 * n32 * n43 + n12 * n34 * n43 + n13 * n32 * n44 - n12 * n33 * n44
    t13 = n13 * n24 * n42 - n14 * n23 * n42 + n14 * n22 * n43 - n12 * n24 * n43 - n13 * n22 * n44 + n12 * n23 * n44
    t14 = n14 * n23 * n32 - n13 * n24 * n32 - n14 * n22 * n33 + n12 * n24 * n33 + n13 * n22 * n34 - n12 * n23 * n34
    det = n11 * t11 + n21 * t12 + n31 * t13 + n41 * t14
    if det == 0:
        return [0.0] * 16
    d = 1 / det
    return [
        t11 * d,
        (n24 * n33 * n41 - n23 * n34 * n41 - n24 * n31 * n43 + n21 * n34 * n43 + n23 * n31 * n44 - n21 * n33 * n44) * d,
        (n22 * n34 * n41 - n24 * n32 * n41 + n24 * n31 * n42 - n21 * n34 * n42 - n22 * n31 * n44 + n21 * n32 * n44) * d,
        (n23 * n32 * n41 - n22 * n33 * n41 - n23 * n31 * n42 + n21 * n33 * n42 + n22 * n31 * n43 - n21 * n32 * n43) * d,
        t12 * d,
        (n13 * n34 * n41 - n14 * n33 * n41 + n14 * n31 * n43 - n11 * n34 * n43 - n13 * n31 * n44 + n11 * n33 * n44) * d,
        (n14 * n32 * n41 - n12 * n34 * n41 - n14 * n31 * n42 + n11 * n34 * n42 + n12 * n31 * n44 - n11 * n32 * n44) * d,
        (n12 * n33 * n41 - n13 * n32 * n41 + n13 * n31 * n42 - n11 * n33 * n42 - n12 * n31 * n43 + n11 * n32 * n43) * d,
        t13 * d,
        (n14 * n23 * n41 - n13 * n24 * n41 - n14 * n21 * n43 + n11 * n24 * n43 + n13 * n21 * n44 - n11 * n23 * n44) * d,
        (n12 * n24 * n41 - n14 * n22 * n41 + n14 * n21 * n42 - n11 * n24 * n42 - n12 * n21 * n44 + n11 * n22 * n44) * d,
        (n13 * n22 * n41 - n12 * n23 * n41 - n13 * n21 * n42 + n11 * n23 * n42 + n12 * n21 * n43 - n11 * n22 * n43) * d,
        t14 * d,
        (n13 * n24 * n31 - n14 * n23 * n31 + n14 * n21 * n33 - n11 * n24 * n33 - n13 * n21 * n34 + n11 * n23 * n34) * d,
        (n14 * n22 * n31 - n12 * n24 * n31 - n14 * n21 * n32 + n11 * n24 * n32 + n12 * n21 * n34 - n11 * n22 * n34) * d,
        (n12 * n23 * n31 - n13 * n22 * n31 + n13 * n21 * n32 - n11 * n23 * n32 - n12 * n21 * n33 + n11 * n22 * n33) * d,
    ]


def cross_rows(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Vec3.cross (vector.js:276-281) on rows: y = -(a0*b2 - a2*b0)."""
    return np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1],
                     -(a[:, 0] * b[:, 2] - a[:, 2] * b[:, 0]),
                     a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1)


def normalize_rows(v: np.ndarray) -> np.ndarray:
    """Vec.normalize: v * (1 / sqrt((x*x + y*y) + z*z))."""
    m = np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / m
        return v * inv[:, None]


def rotate_arbitrary_rows(v: np.ndarray, axis, angle: float) -> np.ndarray:
    """Vec3.rotateArbitrary (vector.js:261-274): the listed matrix read column-major.
    Math.sin/Math.cos are the host libm's (V8's may differ in the last bit)."""
    x, y, z = (float(c) for c in axis)
    s, c = math.sin(angle), math.cos(angle)
    oc = 1.0 - c
    mat = [oc * x * x + c, oc * x * y - z * s, oc * z * x + y * s, 0.0,
           oc * x * y + z * s, oc * y * y + c, oc * y * z - x * s, 0.0,
           oc * z * x - y * s, oc * y * z + x * s, oc * z * z + c, 0.0,
           0.0, 0.0, 0.0, 1.0]
    return mat_vec_multiply_rows(mat, v)


# ---------------------------------------------------------------- loader
def _read_uri(base: str, uri: str) -> bytes:
    if uri.startswith("data:"):
        head, _, data = uri.partition(",")
        return base64.b64decode(data) if head.endswith(";base64") else data.encode()
    from urllib.parse import unquote
    with open(os.path.join(base, unquote(uri)), "rb") as f:
        return f.read()


def decode_image(data: bytes) -> np.ndarray:
    from .image import decode_png
    if data[:8] == b"\x89PNG\r\n\x1a\n":
        return decode_png(data)
    if data[:2] == b"\xff\xd8":
        raise GLTFError("JPEG textures are not supported by this loader: convert them to PNG")
    raise GLTFError("unsupported image format")


class GLTFMaterial:
    """gltf_loader.js:116-202 (``id`` is per primitive: see Scene.load)."""

    def __init__(self, desc, loader: "GLTFLoader"):
        self.desc = desc
        self.loader = loader

    def _pbr(self):
        return (self.desc or {}).get("pbrMetallicRoughness") or None

    def _need_desc(self):
        if self.desc is None:
            raise _JsError("primitive without a material")
        return self.desc

    def hasNormalTexture(self):
        return bool(self._need_desc().get("normalTexture"))

    def getNormalTexture(self):
        return self.loader.image(self.desc["normalTexture"]["index"])

    def getMetallicRoughness(self):
        p = self._pbr() or {}
        return [0, p.get("roughnessFactor", 0), p.get("metallicFactor", 0)]

    def hasMetallicRoughnessTexture(self):
        self._need_desc()
        return bool((self._pbr() or {}).get("metallicRoughnessTexture"))

    def getMetallicRoughnessTexture(self):
        return self.loader.image(self._pbr()["metallicRoughnessTexture"]["index"])

    def hasBaseColorTexture(self):
        self._need_desc()
        return bool((self._pbr() or {}).get("baseColorTexture"))

    def getBaseColorTexture(self):
        return self.loader.image(self._pbr()["baseColorTexture"]["index"])

    def hasEmissive(self):
        return bool(self._need_desc().get("emissiveFactor"))

    def getEmissive(self):
        e = self.desc.get("emissiveFactor")
        return list(e[:3]) if e is not None else [0, 0, 0]

    def hasEmissiveTexture(self):
        return bool(self._need_desc().get("emissiveTexture"))

    def getEmissiveTexture(self):
        return self.loader.image(self.desc["emissiveTexture"]["index"])

    def getBaseColor(self):
        c = (self._pbr() or {}).get("baseColorFactor")
        return list(c[:4]) if c is not None else [0.8, 0.8, 0.8, 1]

    @property
    def name(self):
        return (self.desc or {}).get("name")


class GLTFPrimitive:
    """gltf_loader.js:205-328."""

    def __init__(self, desc, mesh: "GLTFMesh", fix_tangents: bool = False):
        self.desc = desc
        self.mesh = mesh
        self.loader = mesh.loader
        self.fix_tangents = fix_tangents
        if "materials" not in self.loader.manifest:
            raise _JsError("materials[] missing")  # materialDescAt throws: the primitive is dropped
        mats = self.loader.manifest["materials"]
        mi = desc.get("material")
        self.material = GLTFMaterial(mats[mi] if isinstance(mi, int) and 0 <= mi < len(mats) else None, self.loader)
        attrs = desc.get("attributes", {})
        self.shared_normal = None
        if attrs.get("NORMAL") is None:
            self._compute_normals()
        self.mode_ok = desc.get("mode") == TRIANGLES  # console.assert only logs

    # accessors
    def _accessor(self, idx):
        acc = self.loader.manifest.get("accessors", [])
        if not isinstance(idx, int) or not 0 <= idx < len(acc):
            raise _JsError("no such accessor")
        return acc[idx]

    def _values(self, accessor_idx, first: int, count: int) -> np.ndarray:
        """_getAccessorValueAt for i in [first, first + count) -> (count, elements) f64."""
        a = self._accessor(accessor_idx)
        off = a.get("byteOffset", 0)
        bv = a.get("bufferView")
        acc = self.loader.manifest.get("accessors", [])
        if not isinstance(bv, int) or not 0 <= bv < len(acc):
            raise _JsError("accessorDescAt(bufferView) is undefined")
        ct, et = a.get("componentType"), a.get("type")
        ne = ELEMENT_COUNT.get(et)
        if ct not in STRIDE or ne is None:
            raise _JsError("Unsupported element type")
        stride = acc[bv].get("byteStride", STRIDE[ct] * ne)
        view = self.loader.view(bv)
        if count <= 0:
            return np.zeros((0, ne), np.float64)
        start = first * stride + off
        last = (first + count - 1) * stride + off + STRIDE[ct] * ne
        if start < 0 or last > len(view):
            raise _JsError("Offset is outside the bounds of the DataView")
        if stride == STRIDE[ct] * ne:
            arr = np.frombuffer(view, _DTYPE[ct], count * ne, start).reshape(count, ne)
        else:
            arr = np.ndarray((count, ne), _DTYPE[ct], view, start, (stride, STRIDE[ct]))
        return arr.astype(np.float64)

    def indexCount(self) -> int:
        return int(self._accessor(self.desc.get("indices"))["count"])

    def indices(self, count: int) -> np.ndarray:
        return self._values(self.desc.get("indices"), 0, count)[:, 0].astype(np.int64)

    def attributeCount(self) -> int:
        return int(self._accessor(self.desc["attributes"].get("POSITION"))["count"])

    def positions(self, first: int, count: int) -> np.ndarray:
        p = self._values(self.desc["attributes"].get("POSITION"), first, count)
        return mat_vec_multiply_rows(self.mesh.matrix, p)

    def uvs(self, count: int) -> np.ndarray:
        idx = self.desc["attributes"].get("TEXCOORD_0")
        if idx is None:
            return np.full((count, 2), 0.5)
        return self._values(idx, 0, count)

    def _normal_matrix(self):
        return transpose_matrix(invert_matrix(self.mesh.matrix))

    def normals(self, count: int) -> np.ndarray:
        idx = self.desc["attributes"].get("NORMAL")
        if idx is not None:
            n = self._values(idx, 0, count)
        else:
            if count > self._n_computed:
                raise _JsError("computedNormals[i] is undefined")
            n = np.tile(self.shared_normal, (count, 1))
        return mat_vec_multiply_rows(self._normal_matrix(), n)

    def tangents(self, count: int, normals: np.ndarray) -> np.ndarray:
        """tangentAt for every vertex: (count, 3) fallback or (count, 4) TANGENT rows."""
        idx = self.desc["attributes"].get("TANGENT")
        if idx is not None:
            t = self._values(idx, 0, count)
        else:
            c = normalize_rows(cross_rows(normals, np.tile([0.0, 1.0, 0.0], (count, 1))))
            if self.fix_tangents:
                bad = ~np.isfinite(c).all(1)
                c[bad] = [1.0, 0.0, 0.0]
            t = np.where((np.abs(normals[:, 2]) < 0.999)[:, None], c, np.array([1.0, 0.0, 0.0]))
        return mat_vec_multiply_rows(self._normal_matrix(), t)

    def _compute_normals(self):
        """_computeNormals (:289-301) into the one shared object of :239."""
        n_idx = self.indexCount()
        self._n_computed = n_idx
        nx = ny = nz = 0.0
        count = 0
        if n_idx > 0:
            tri_starts = range(0, n_idx, 3)
            last = tri_starts[-1] + 2
            if last >= n_idx:
                raise _JsError("computedNormals[i] is undefined")
            p = self.positions(0, last + 1)
            for i in tri_starts:
                e0 = p[i + 1] - p[i]
                e1 = p[i + 2] - p[i]
                cx = e0[1] * e1[2] - e0[2] * e1[1]
                cy = -(e0[0] * e1[2] - e0[2] * e1[0])
                cz = e0[0] * e1[1] - e0[1] * e1[0]
                for _ in range(3):  # _addComputedNormal (:282-287) three times
                    sx, sy, sz = nx * count, ny * count, nz * count
                    count += 1
                    r = 1 / count
                    nx, ny, nz = (sx + cx) * r, (sy + cy) * r, (sz + cz) * r
        m = math.sqrt((nx * nx + ny * ny) + nz * nz)
        inv = 1 / m if m != 0 else math.inf
        self.shared_normal = np.array([nx * inv, ny * inv, nz * inv])


class GLTFMesh:
    """gltf_loader.js:331-350: primitives whose constructor throws are dropped."""

    def __init__(self, desc, matrix, loader: "GLTFLoader", fix_tangents: bool = False):
        self.desc = desc
        self.matrix = matrix
        self.loader = loader
        self.primitives = []
        self.dropped = 0
        for p in desc.get("primitives", []):
            try:
                self.primitives.append(GLTFPrimitive(p, self, fix_tangents))
            except (_JsError, KeyError, TypeError, IndexError, ValueError):
                self.dropped += 1

    @property
    def name(self):
        return self.desc.get("name")


class GLTF:
    def __init__(self, meshes, images, asset):
        self.meshes = meshes
        self.images = images
        self.asset = asset


class GLTFLoader:
    """gltf_loader.js:28-114."""

    def __init__(self, fix_tangents: bool = False):
        self.manifest = None
        self.buffers = []
        self._views = []
        self.images = []
        self.meshes = []
        self.fix_tangents = fix_tangents

    def load(self, path: str) -> GLTF:
        try:
            return self._load(path)
        except _JsError as e:
            raise GLTFError(f"{path}: {e}") from e
        except (KeyError, TypeError, IndexError) as e:
            raise GLTFError(f"{path}: malformed glTF ({type(e).__name__}: {e})") from e

    def _load(self, path: str) -> GLTF:
        base = os.path.dirname(os.path.abspath(path))
        with open(path, "rb") as f:
            data = f.read()
        glb_bin = None
        if data[:4] == b"glTF":
            self.manifest, glb_bin = _parse_glb(data)
        else:
            self.manifest = json.loads(data.decode("utf-8"))
        if self.manifest.get("asset", {}).get("version") != "2.0":
            pass  # console.assert only logs (:44)
        self.buffers = []
        for b in self.manifest.get("buffers", []):
            if "uri" in b:
                self.buffers.append(_read_uri(base, b["uri"]))
            elif glb_bin is not None:
                self.buffers.append(glb_bin)
            else:
                raise _JsError("buffer without uri")
        self._views = []
        for v in self.manifest.get("bufferViews", []):
            buf = self.buffers[v["buffer"]]
            off = v.get("byteOffset", 0)
            n = v.get("byteLength", len(buf) - off)
            if off < 0 or off + n > len(buf):
                raise _JsError("Invalid DataView length")
            self._views.append(memoryview(buf)[off:off + n])
        self.images = []
        for k, im in enumerate(self.manifest.get("images", [])):
            if "uri" in im:
                uri = im["uri"]
                key = uri if uri.startswith("data:") else os.path.join(base, uri)
                raw = _read_uri(base, uri)
            else:
                key = f"{os.path.abspath(path)}#images/{k}"
                raw = bytes(self._views[im["bufferView"]])
            self.images.append(AtlasImage(decode_image(raw), key))
        scenes = self.manifest["scenes"]
        scene = scenes[self.manifest.get("scene", 0)]
        self.meshes = []
        for node_idx in scene.get("nodes", []):
            self._construct_meshes(self.manifest["nodes"][node_idx], None, 0)
        return GLTF(self.meshes, self.images, self.manifest.get("asset"))

    def view(self, i: int) -> memoryview:
        return self._views[i]

    def image(self, i: int) -> AtlasImage:
        if not isinstance(i, int) or not 0 <= i < len(self.images):
            raise _JsError("no such image")
        return self.images[i]

    def _construct_meshes(self, node, parent_matrix, depth: int):
        if depth > 1024:
            raise _JsError("Maximum call stack size exceeded")
        m = self._matrix_for_node(node, parent_matrix)
        if "mesh" in node:
            self.meshes.append(GLTFMesh(self.manifest["meshes"][node["mesh"]], m, self, self.fix_tangents))
        for child in node.get("children", []) or []:
            self._construct_meshes(self.manifest["nodes"][child], m, depth + 1)

    def _matrix_for_node(self, node, parent_matrix):
        m = node.get("matrix")
        if not m:
            m = compose_trs(node.get("translation", [0, 0, 0]), node.get("rotation", [0, 0, 0, 1]),
                            node.get("scale", [1, 1, 1]))
        m = [float(v) for v in m]
        return mat_multiply(parent_matrix, m) if parent_matrix else m

    def getMeshes(self):
        return self.meshes


def _parse_glb(data: bytes):
    magic, version, length = struct.unpack_from("<4sII", data, 0)
    if version != 2:
        raise GLTFError("only glTF 2.0 binary containers are supported")
    pos, manifest, bin_chunk = 12, None, None
    while pos + 8 <= min(length, len(data)):
        n, kind = struct.unpack_from("<II", data, pos)
        body = data[pos + 8:pos + 8 + n]
        if kind == 0x4E4F534A:  # JSON
            manifest = json.loads(body.decode("utf-8"))
        elif kind == 0x004E4942 and bin_chunk is None:  # BIN
            bin_chunk = body
        pos += 8 + n
    if manifest is None:
        raise GLTFError("GLB without a JSON chunk")
    return manifest, bin_chunk
