"""Seeded synthetic scenes for Pike's wavefront path (no scene assets ship with
the reference: its scene/, environment/ and asset_packs/ folders are
git-ignored, see .gitignore:2-5 of the reference).

Every generator returns a :class:`SceneSource`: glTF-like per-vertex arrays
(positions, normals, signed tangents, uvs), triangles ``{i0, i1, i2, matId}``,
per-material factors, an environment map and a camera in world units.  These
are the inputs of ``Scene._createBuffers`` (render/scene.js:120-181) after the
glTF loader has run, with identity node matrices and transforms.

Randomness is counter-based (splitmix64 of seed, stream and index) and all
arithmetic is plain IEEE double (no libm transcendentals: ``_exp`` below is a
Cody-Waite reduction plus Taylor series), so the same seed yields the same
bytes on x86 and on Arm.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)

SEED_BASE = 0x50494B45  # "PIKE"


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = x + np.uint64(0x9E3779B97F4A7C15)
    z = x
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


class Rng:
    """Counter-based generator: value i of stream s is splitmix64(splitmix64(key(s)) ^ i)."""

    def __init__(self, seed: int):
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self._stream = 0

    def stream(self) -> "_Stream":
        s = _Stream(self.seed, self._stream)
        self._stream += 1
        return s


class _Stream:
    def __init__(self, seed: int, stream: int):
        key = _splitmix64(np.array([seed ^ (stream * 0xD1B54A32D192ED03 & 0xFFFFFFFFFFFFFFFF)], dtype=np.uint64))[0]
        self.key = np.uint64(key)
        self.ctr = 0

    def u64(self, n: int) -> np.ndarray:
        idx = np.arange(self.ctr, self.ctr + n, dtype=np.uint64)
        self.ctr += n
        with np.errstate(over="ignore"):
            return _splitmix64(idx ^ self.key)

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + u * (hi - lo)

    def normal_approx(self, n: int) -> np.ndarray:
        """Irwin-Hall(12) - 6: a unit-variance, zero-mean bell curve from 12 uniforms."""
        u = self.uniform(12 * n).reshape(n, 12)
        s = u[:, 0].copy()
        for k in range(1, 12):
            s = s + u[:, k]
        return s - 6.0


_LN2_HI = 6.93147180369123816490e-01
_LN2_LO = 1.90821492927058770002e-10
_INV_LN2 = 1.44269504088896338700e00


def _exp(x: np.ndarray) -> np.ndarray:
    """exp(x) in IEEE double with only + - * and ldexp (Cody-Waite + Taylor to x^13)."""
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x * _INV_LN2 + 0.5)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.full_like(r, 1.0 / math.factorial(13))
    for n in range(12, 0, -1):
        p = (1.0 / math.factorial(n)) + r * p
    p = 1.0 + r * p
    return np.ldexp(p, k.astype(np.int64))


@dataclasses.dataclass
class SceneSource:
    name: str
    pos: np.ndarray        # (V,3) f64
    normal: np.ndarray     # (V,3) f64
    tangent: np.ndarray    # (V,4) f64, w = handedness
    uv: np.ndarray         # (V,2) f64
    tris: np.ndarray       # (T,4) i32: i0, i1, i2, matId
    materials: np.ndarray  # (M,9) f64: base r,g,b,a, roughness, metallic, emissive r,g,b
    env_rgbe: np.ndarray   # (h,w,4) u8, RGBE with rgb/255 * 2^(e-128)
    env_hdr: np.ndarray | None  # (h,w,3) f32 source radiance, when the scene defines one
    cam_pos: tuple
    cam_target: tuple
    fov: float             # radians, vertical
    width: int
    height: int
    spp: int
    bounces: int

    @property
    def n_tris(self) -> int:
        return int(self.tris.shape[0])

    def root_bounds(self):
        used = np.unique(self.tris[:, :3].reshape(-1))
        p = self.pos[used]
        return p.min(axis=0), p.max(axis=0)

    def normalizer(self):
        """trace_pass.js:202-211 #makeNormalizer over the root box: returns (center, scale)."""
        mn, mx = self.root_bounds()
        span = mx - mn
        longest = max(span[0], span[1], span[2])
        center = mn + span * 0.5
        return center, 2.0 / longest

    def camera_state(self, invocation_offset: int = 0, focal_depth: float = 0.5, aperture: float = 0.0,
                     distortion: float = 0.0, bokeh: float = 0.5):
        """CameraStateStuct fields (structs.js:235-249) in the normalised frame the passes render in."""
        center, s = self.normalizer()
        p = (np.asarray(self.cam_pos, dtype=np.float64) - center) * s
        d = np.asarray(self.cam_target, dtype=np.float64) - np.asarray(self.cam_pos, dtype=np.float64)
        d = d / math.sqrt(float(d @ d))
        return dict(pos=[float(np.float32(v)) for v in p], dir=[float(np.float32(v)) for v in d],
                    fov=float(np.float32(self.fov)), focalDepth=focal_depth, apertureSize=aperture,
                    distortion=distortion, bokeh=bokeh, invocationOffset=invocation_offset)


def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    """Encode linear radiance as RGBE8 for the decode rgb/255 * 2^(e-128) used by
    env_sampler.js:43-48 and shade_miss.wgsl:42."""
    rgb = np.asarray(rgb, dtype=np.float64)
    m = rgb.max(axis=-1)
    out = np.zeros(rgb.shape[:-1] + (4,), dtype=np.uint8)
    ok = m > 1e-30
    f, e = np.frexp(np.where(ok, m, 1.0))
    e = np.clip(e, -128, 127)
    scale = np.ldexp(np.ones_like(m), -e) * 255.0
    mant = np.floor(rgb * scale[..., None] + 0.5)
    mant = np.clip(mant, 0, 255)
    out[..., :3] = np.where(ok[..., None], mant, 0).astype(np.uint8)
    out[..., 3] = np.where(ok, e + 128, 0).astype(np.uint8)
    return out


def _box_faces(lo, hi, inward=False, skip=()):
    """Quads of an axis-aligned box: returns (pos, normal, tangent, uv, quads) for the faces not skipped."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    faces = {
        "+x": ([(x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)], (1, 0, 0), (0, 0, 1)),
        "-x": ([(x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)], (-1, 0, 0), (0, 0, 1)),
        "+y": ([(x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)], (0, 1, 0), (1, 0, 0)),
        "-y": ([(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)], (0, -1, 0), (1, 0, 0)),
        "+z": ([(x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)], (0, 0, 1), (1, 0, 0)),
        "-z": ([(x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)], (0, 0, -1), (1, 0, 0)),
    }
    P, N, Tg, UV, Q = [], [], [], [], []
    for key in ("+x", "-x", "+y", "-y", "+z", "-z"):
        if key in skip:
            continue
        verts, n, t = faces[key]
        if inward:
            n = tuple(-c for c in n)
        base = len(P)
        P.extend(verts)
        N.extend([n] * 4)
        Tg.extend([t + (1.0,)] * 4)
        UV.extend([(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)])
        Q.append((base, base + 1, base + 2, base + 3))
    return (np.array(P, float), np.array(N, float), np.array(Tg, float), np.array(UV, float), np.array(Q, np.int64))


def _quads_to_tris(q: np.ndarray) -> np.ndarray:
    return np.concatenate([q[:, [0, 1, 2]], q[:, [0, 2, 3]]], axis=1).reshape(-1, 3)


def small_scene(seed_index: int = 0, width: int = 256, height: int = 256, spp: int = 4, bounces: int = 4,
                n_boxes: int = 64) -> SceneSource:
    """40x40 ground quad + 64 boxes (770 triangles for 64 boxes), Lambert albedo U[0.2,0.8],
    constant white environment of radiance 1, pinhole camera at (0,8,-20) looking at the
    origin with a 60 degree vertical field of view."""
    rng = Rng(SEED_BASE + seed_index)
    s_box, s_col = rng.stream(), rng.stream()
    P, N, Tg, UV, T, M = [], [], [], [], [], []
    g = 20.0
    P.append(np.array([(-g, 0, -g), (g, 0, -g), (g, 0, g), (-g, 0, g)], float))
    N.append(np.array([(0, 1, 0)] * 4, float))
    Tg.append(np.array([(1, 0, 0, 1)] * 4, float))
    UV.append(np.array([(0, 0), (1, 0), (1, 1), (0, 1)], float))
    T.append(np.concatenate([_quads_to_tris(np.array([[0, 1, 2, 3]])), np.zeros((2, 1), np.int64)], axis=1))
    cols = s_col.uniform(3 * (n_boxes + 1), 0.2, 0.8).reshape(-1, 3)
    M.append([cols[0, 0], cols[0, 1], cols[0, 2], 1.0, 1.0, 0.0, 0.0, 0.0, 0.0])
    r = s_box.uniform(5 * n_boxes).reshape(n_boxes, 5)
    base = 4
    for b in range(n_boxes):
        cx, cz = -10.0 + 20.0 * r[b, 0], -10.0 + 20.0 * r[b, 1]
        sx, sy, sz = 0.2 + 1.8 * r[b, 2], 0.2 + 1.8 * r[b, 3], 0.2 + 1.8 * r[b, 4]
        p, n, t, uv, q = _box_faces((cx - sx / 2, 0.0, cz - sz / 2), (cx + sx / 2, sy, cz + sz / 2))
        P.append(p); N.append(n); Tg.append(t); UV.append(uv)
        tr = _quads_to_tris(q) + base
        T.append(np.concatenate([tr, np.full((tr.shape[0], 1), b + 1, np.int64)], axis=1))
        M.append([cols[b + 1, 0], cols[b + 1, 1], cols[b + 1, 2], 1.0, 1.0, 0.0, 0.0, 0.0, 0.0])
        base += p.shape[0]
    env = np.zeros((32, 64, 4), np.uint8)
    env[...] = (255, 255, 255, 128)
    return SceneSource(
        name=f"ground+{n_boxes}boxes", pos=np.concatenate(P), normal=np.concatenate(N), tangent=np.concatenate(Tg),
        uv=np.concatenate(UV), tris=np.concatenate(T).astype(np.int32), materials=np.array(M, np.float64),
        env_rgbe=env, env_hdr=np.ones((32, 64, 3), np.float32), cam_pos=(0.0, 8.0, -20.0), cam_target=(0.0, 0.0, 0.0),
        fov=math.pi / 3, width=width, height=height, spp=spp, bounces=bounces)


def icosphere(subdivisions: int):
    """Unit icosphere: (verts (V,3) f64, faces (F,3) i64).  Each face is replaced by its four
    children in place, so face i's ancestors are i >> 2, i >> 4, ..."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], float)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    v = v / np.sqrt((v * v).sum(axis=1))[:, None]
    for _ in range(subdivisions):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])  # (3F,2): edges 01, 12, 20
        lo, hi = np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1])
        key = lo * np.int64(1 << 32) + hi
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = (uniq >> np.int64(32)), (uniq & np.int64(0xFFFFFFFF))
        mid = v[a] + v[b]
        mid = mid / np.sqrt((mid * mid).sum(axis=1))[:, None]
        v = np.concatenate([v, mid])
        F = f.shape[0]
        m01, m12, m20 = nv + inv[:F], nv + inv[F:2 * F], nv + inv[2 * F:]
        children = np.stack([
            np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=1)
        f = children.reshape(-1, 3)
    return v, f


def _value_noise(p: np.ndarray, stream_seed: int, freq: float) -> np.ndarray:
    """Trilinear value noise in [-1, 1] with smoothstep weights on an integer lattice."""
    q = p * freq
    i0 = np.floor(q)
    fr = q - i0
    w = fr * fr * (3.0 - 2.0 * fr)
    i0 = i0.astype(np.int64)

    def lattice(ix, iy, iz):
        h = (ix.astype(np.uint64) * np.uint64(0x9E3779B1) ^ iy.astype(np.uint64) * np.uint64(0x85EBCA77)
             ^ iz.astype(np.uint64) * np.uint64(0xC2B2AE3D) ^ np.uint64(stream_seed))
        with np.errstate(over="ignore"):
            h = _splitmix64(h)
        return (h >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0

    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1.0 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out = out + wx * wy * wz * lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def _vertex_normals(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    a, b, c = pos[faces[:, 0]], pos[faces[:, 1]], pos[faces[:, 2]]
    fn = np.cross(b - a, c - a)
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    return n / np.sqrt((n * n).sum(axis=1))[:, None]


def _tangents(n: np.ndarray) -> np.ndarray:
    """A unit tangent perpendicular to each normal (cross with +y, +x near the poles), w = 1."""
    up = np.where(np.abs(n[:, 1:2]) < 0.999, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(n, up)
    t = t / np.sqrt((t * t).sum(axis=1))[:, None]
    return np.concatenate([t, np.ones((n.shape[0], 1))], axis=1)


def hdr_env(seed: int, width: int = 2048, height: int = 1024, sigma: float = 1.5, sun: float = 1.0e4):
    """Equirect radiance: log-normal(0, sigma) grey texels plus a 4x4-texel sun of radiance `sun`."""
    s = Rng(seed).stream()
    z = s.normal_approx(width * height)
    L = _exp(sigma * z).reshape(height, width)
    sy, sx = height // 4, width // 4
    L[sy:sy + 4, sx:sx + 4] = sun
    return np.repeat(L[..., None], 3, axis=2).astype(np.float32)


def displaced_sphere_scene(subdivisions: int = 8, width: int = 1920, height: int = 1080, spp: int = 64,
                           bounces: int = 8, n_groups: int = 256, seed_index: int = 1,
                           env_size=(2048, 1024)) -> SceneSource:
    """Icosphere subdivided `subdivisions` times (20*4^s triangles; 1,310,720 at s=8), radius 1.5,
    displaced radially by value noise of amplitude 0.05, inside an open 10x10x10 box (10 triangles,
    open towards +y); 256 face groups with GGX roughness U[0.05,1], metallic Bernoulli(0.5),
    albedo U[0.1,0.9]; log-normal HDR environment with a sun."""
    rng = Rng(SEED_BASE + seed_index)
    s_noise, s_mat = rng.stream(), rng.stream()
    v, f = icosphere(subdivisions)
    noise = _value_noise(v, int(s_noise.u64(1)[0]), 4.0)
    R = 1.5
    pos = v * (R * (1.0 + 0.05 * noise))[:, None]
    nrm = _vertex_normals(pos, f)
    tan = _tangents(nrm)
    uv = np.full((pos.shape[0], 2), 0.5)
    F = f.shape[0]
    group = (np.arange(F, dtype=np.int64) * n_groups) // F
    tris = np.concatenate([f, group[:, None]], axis=1)
    m = s_mat.uniform(5 * n_groups).reshape(n_groups, 5)
    mats = np.zeros((n_groups + 1, 9))
    mats[:n_groups, 0:3] = 0.1 + 0.8 * m[:, 0:3]
    mats[:n_groups, 3] = 1.0
    mats[:n_groups, 4] = 0.05 + 0.95 * m[:, 3]
    mats[:n_groups, 5] = (m[:, 4] < 0.5).astype(np.float64)
    mats[n_groups] = [0.7, 0.7, 0.7, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0]
    bp, bn, bt, buv, bq = _box_faces((-5.0, -5.0, -5.0), (5.0, 5.0, 5.0), inward=True, skip=("+y",))
    btr = _quads_to_tris(bq) + pos.shape[0]
    tris = np.concatenate([tris, np.concatenate([btr, np.full((btr.shape[0], 1), n_groups)], axis=1)])
    ew, eh = env_size
    hdr = hdr_env(SEED_BASE + 100 + seed_index, ew, eh)
    return SceneSource(
        name=f"icosphere{subdivisions}+openbox", pos=np.concatenate([pos, bp]), normal=np.concatenate([nrm, bn]),
        tangent=np.concatenate([tan, bt]), uv=np.concatenate([uv, buv]), tris=tris.astype(np.int32), materials=mats,
        env_rgbe=rgbe_encode(hdr), env_hdr=hdr, cam_pos=(0.0, 1.5, -4.5), cam_target=(0.0, 0.0, 0.0),
        fov=math.pi / 3, width=width, height=height, spp=spp, bounces=bounces)


def triangle_soup_scene(n_tris: int = 8_388_608, width: int = 1920, height: int = 1080, spp: int = 16,
                        bounces: int = 4, seed_index: int = 2, env_size=(2048, 1024)) -> SceneSource:
    """Triangle soup: centroids uniform in a 100^3 cube, edge scale log-uniform in [0.01, 1]."""
    rng = Rng(SEED_BASE + seed_index)
    s_c, s_e, s_s = rng.stream(), rng.stream(), rng.stream()
    c = s_c.uniform(3 * n_tris, -50.0, 50.0).reshape(n_tris, 3)
    size = _exp(s_s.uniform(n_tris, -4.605170185988091, 0.0))
    d = s_e.uniform(6 * n_tris, -1.0, 1.0).reshape(n_tris, 2, 3)
    d = d / np.maximum(np.sqrt((d * d).sum(axis=2)), 1e-9)[..., None]
    a, b = d[:, 0] * size[:, None], d[:, 1] * size[:, None]
    pos = np.stack([c + a, c + b, c - a - b], axis=1).reshape(-1, 3)
    fn = np.cross(b - a, -a - b - a)
    fn = fn / np.maximum(np.sqrt((fn * fn).sum(axis=1)), 1e-30)[:, None]
    nrm = np.repeat(fn, 3, axis=0)
    tan = _tangents(nrm)
    uv = np.full((pos.shape[0], 2), 0.5)
    idx = np.arange(3 * n_tris, dtype=np.int64).reshape(n_tris, 3)
    tris = np.concatenate([idx, np.zeros((n_tris, 1), np.int64)], axis=1).astype(np.int32)
    mats = np.array([[0.6, 0.6, 0.6, 1.0, 0.5, 0.0, 0.0, 0.0, 0.0]])
    ew, eh = env_size
    hdr = hdr_env(SEED_BASE + 100 + 1, ew, eh)
    return SceneSource(
        name=f"soup{n_tris}", pos=pos, normal=nrm, tangent=tan, uv=uv, tris=tris, materials=mats,
        env_rgbe=rgbe_encode(hdr), env_hdr=hdr, cam_pos=(0.0, 0.0, -120.0), cam_target=(0.0, 0.0, 0.0),
        fov=math.pi / 3, width=width, height=height, spp=spp, bounces=bounces)
