"""Scene._createBuffers and _createSceneMaterial (render/scene.js:43-181) over
loaded glTF groups: the per-vertex arrays pk_scene_flatten_tbn quantises, the
triangle table, the material index table and the packed atlas.

Per vertex, in the reference's order (scene.js:155-169):
  pos       = rotations(positionAt(i)) * scale + translate
  normal    = rotations(normalAt(i)) * 1 + 0
  tangent   = rotations(tangentAt(i).xyz) * 1 + 0
  bitangent = normalize(cross(normalAt(i), tangentAt(i)) * (tangentAt(i)[3] || 1))
The bitangent uses the vectors before the prop's rotations; both forms are
handed to the GPU flattener, which quantises
normalize(tangent)/bitangent/normalize(normal) to snorm8x4 and uv to
snorm16x2.

Materials: ``materialIds`` is keyed by ``GLTFMaterial.id``, a fresh
``Math.round(Math.random() * 10000)`` per primitive (gltf_loader.js:118), so
every primitive gets its own material unless two random ids collide; this
restatement gives every primitive its own material (the collision-free
outcome).  Colours and textures are still deduplicated by the packer.
"""
from __future__ import annotations

import os

import numpy as np

from .atlas import TexturePacker
from .gltf import GLTFError, GLTFLoader, _JsError, rotate_arbitrary_rows


def _rotations(v: np.ndarray, transforms) -> np.ndarray:
    for r in transforms.get("rotate", []):
        v = rotate_arbitrary_rows(v, r["axis"], float(r["angle"]))
    return v


def _apply_vector_transforms(v: np.ndarray, transforms, rotation_only: bool = False) -> np.ndarray:
    """scene.js:77-80."""
    r = _rotations(v, transforms)
    s = 1.0 if rotation_only else float(transforms.get("scale", 1.0))
    t = np.zeros(3) if rotation_only else np.asarray(transforms.get("translate", [0.0, 0.0, 0.0]), np.float64)
    return r * s + t


def _scene_material(m, packer: TexturePacker):
    """scene.js:43-70: {diffMap, metRoughMap, normMap, emitMap}."""
    diff = packer.addTexture(m.getBaseColorTexture(), True) if m.hasBaseColorTexture() else \
        packer.addColor(m.getBaseColor())
    mr = packer.addTexture(m.getMetallicRoughnessTexture()) if m.hasMetallicRoughnessTexture() else \
        packer.addColor(m.getMetallicRoughness())
    nm = packer.addTexture(m.getNormalTexture()) if m.hasNormalTexture() else packer.addColor([0.5, 0.5, 1])
    em = packer.addTexture(m.getEmissiveTexture(), True) if m.hasEmissiveTexture() else \
        packer.addColor(m.getEmissive())
    return [diff, mr, nm, em]


def build_scene_arrays(desc: dict, base: str, fix_tangents: bool = False) -> dict:
    props = desc.get("props", [])
    groups = []
    for prop in props:
        g = GLTFLoader(fix_tangents).load(os.path.join(base, prop["uri"]))
        g.transforms = prop.get("transforms") or {"rotate": [], "scale": 1.0, "translate": [0.0, 0.0, 0.0]}
        g.skipMaterials = set(prop.get("skipMaterials") or [])
        g.skipMeshes = set(prop.get("skipMeshes") or [])
        groups.append(g)
    packer = TexturePacker(desc.get("atlasRes", 1024))
    P, N, T, BN, BT, UV, TRIS, MATS, lights = [], [], [], [], [], [], [], [], []
    offset = 0
    skipped = 0
    try:
        for g in groups:
            for mesh in g.meshes:
                if mesh.name in g.skipMeshes:
                    skipped += 1
                    continue
                for prim in mesh.primitives:
                    name = prim.material.name
                    if name is not None and name in g.skipMaterials:
                        skipped += 1
                        continue
                    emissive = prim.material.hasEmissive()
                    mat_id = len(MATS)
                    MATS.append(_scene_material(prim.material, packer))
                    n_idx = prim.indexCount()
                    n_read = -(-n_idx // 3) * 3
                    idx = prim.indices(n_read)
                    tris = np.empty((n_read // 3, 4), np.int64)
                    tris[:, 0] = offset + idx[0::3]
                    tris[:, 1] = offset + idx[1::3]
                    tris[:, 2] = offset + idx[2::3]
                    tris[:, 3] = mat_id
                    TRIS.append(tris)
                    n = prim.attributeCount()
                    offset += n
                    pos = _apply_vector_transforms(prim.positions(0, n), g.transforms)
                    n0 = prim.normals(n)
                    t0 = prim.tangents(n, n0)
                    nrm = _apply_vector_transforms(n0, g.transforms, True)
                    tan = _apply_vector_transforms(t0[:, :3], g.transforms, True)
                    bt = np.ones((n, 4))
                    bt[:, :3] = t0[:, :3]
                    if t0.shape[1] == 4:
                        bt[:, 3] = t0[:, 3]
                    P.append(pos)
                    N.append(nrm)
                    T.append(np.concatenate([tan, np.zeros((n, 1))], 1))
                    BN.append(n0)
                    BT.append(bt)
                    UV.append(prim.uvs(n))
                    if emissive and n:
                        lights.append((pos.min(0), pos.max(0)))
    except _JsError as e:
        raise GLTFError(str(e)) from e
    if not TRIS:
        raise GLTFError("the scene has no triangles")
    res, _, n_layers = packer.getResolution()
    atlas = packer.getPixels()
    tris = np.concatenate(TRIS)
    n_verts = offset
    if tris[:, :3].min() < 0 or tris[:, :3].max() >= n_verts:
        raise GLTFError("triangle index outside the scene's vertices")
    return dict(pos=np.concatenate(P), normal=np.concatenate(N), tangent=np.concatenate(T),
                bnormal=np.concatenate(BN), btangent=np.concatenate(BT), uv=np.concatenate(UV),
                tris=tris.astype(np.int32), material_index=np.asarray(MATS, np.int32).reshape(-1, 4), atlas=atlas,
                lights=lights, skipped=skipped)
