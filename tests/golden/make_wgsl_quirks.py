"""Generates tests/golden/wgsl_quirks.json: reference-derived known answers
for three behaviours of the reference path, worked out from the reference's
own source text and the WGSL / JavaScript language rules, not from the
oracle (the oracle is what the fixtures check).

1. rand() == 1.0 (render/shader/camera.wgsl:46-56): rand() is
   f32(hash()) / 4294967296.0.  A u32 above 2^32 - 128 is not representable in
   binary32 and converts to 2^32 (round to nearest), so rand() returns exactly
   1.0.  The search below runs the hash of camera.wgsl:46-52 (as numpy u32
   arithmetic) over camera seeds (px*1973 + py*9277 + samples*26699) | 1
   (camera.wgsl:86-87) and records the first pixel whose jitter-x draw is 1.0.
2. The missing-tangent fallback for a +y normal (render/util/gltf_loader.js:
   268-276): normalize(cross(n, (0,1,0))) with n = (0,1,0) is 0/0 = NaN per
   component; scene.js _quantizeVec3ToInt (scene.js:104-111) stores each
   component into an Int8Array, and ToInt8(NaN) = 0, so the tangent and the
   bitangent words are 0; the normal (0,1,0) stores bytes {0, 127, 0, 0}.
5. A black texel gets a luminance bin of its own (render/env_sampler.js:
   74-95): the histogram walk closes a bin before adding the next texel and
   pushes the last bin after the loop, so with every lit texel above binSize
   each texel ends up alone in a bin and the black one is sampled as often
   as any other (worked example in env_black_bin below).
4. The typed-array quantisers of the scene tables (render/scene.js:104-118):
   UV pairs go through Int16Array (ToInt16: truncation, then wrap modulo
   2^16), so UVs outside [0, 1] wrap; normals through Int8Array after
   Vec3.normalize.  The expected words follow the ECMAScript conversions
   (js_toint below), not the oracle.
3. The environment rotation theta in sampleEnv and envPdf
   (render/shader/shade_hit.wgsl:202-227): sampleEnv puts texel (cx, cy) at
   azimuth u = -theta + (cx + 0.5)/W, and envPdf reads u' = (1 + theta +
   atan2(z, x)/2pi) % 1 = (cx + 0.5)/W again, so the pdf of a sampled
   direction is its own texel's (the signs undo each other).  Worked example
   W x H = 8 x 4, theta = 0.25, texel (3, 1): u = 0.1875, v = 0.375, both
   angles 3pi/8; direction (cos(3pi/8) sin(3pi/8), cos(3pi/8), sin^2(3pi/8)).

Run: python tests/golden/make_wgsl_quirks.py
"""
import json
import math
import os

import numpy as np


def _hash(state):
    s = state.astype(np.uint32)
    nxt = (s * np.uint32(747796405) + np.uint32(2891336453)).astype(np.uint32)
    word = (((s >> ((s >> np.uint32(28)) + np.uint32(4))) ^ s) * np.uint32(277803737)).astype(np.uint32)
    return ((word >> np.uint32(22)) ^ word).astype(np.uint32), nxt


def rand_one():
    W = 4096
    py, px = np.meshgrid(np.arange(W, dtype=np.uint32), np.arange(W, dtype=np.uint32), indexing="ij")
    for samples in range(8):
        seed = ((px * np.uint32(1973) + py * np.uint32(9277) + np.uint32(samples * 26699)) | np.uint32(1))
        first, _ = _hash(seed)           # seed = hash(): the state becomes this output
        jitter, _ = _hash(first)         # rand() #1, the jitter x of createPrimaryRay
        hit = np.argwhere(jitter >= np.uint32(0xFFFFFF80))
        if len(hit):
            y, x = (int(v) for v in hit[0])
            return {"px": x, "py": y, "samples": samples, "state": int(first[y, x]),
                    "hash": int(jitter[y, x]), "rand_f32_bits": "0x3f800000",
                    "why": "u32 >= 2^32 - 128 rounds to 2^32 in binary32; / 2^32 = 1.0"}
    raise RuntimeError("no seed found")


def js_toint(x: float, bits: int) -> int:
    """ECMAScript ToInt8 / ToInt16 (the conversion a typed-array store
    applies): NaN and infinities give 0; otherwise truncate toward zero and
    wrap modulo 2^bits into [-2^(bits-1), 2^(bits-1))."""
    if x != x or x in (math.inf, -math.inf):
        return 0
    i = int(math.copysign(math.floor(abs(x)), x))
    i %= 1 << bits
    return i - (1 << bits) if i >= 1 << (bits - 1) else i


def uv_word(u: float, v: float) -> int:
    """scene.js:113-118 _quantizeVec2ToInt: Int16Array{u * (u > 0 ? 32767 :
    32768), v * ...} read back as one little-endian u32."""
    a = js_toint(u * (32767 if u > 0 else 32768), 16)
    b = js_toint(v * (32767 if v > 0 else 32768), 16)
    return (a & 0xFFFF) | ((b & 0xFFFF) << 16)


def normal_word(n) -> int:
    """scene.js:104-111 _quantizeVec3ToInt of Vec3.normalize(n): Int8Array
    bytes n_i * (n_i > 0 ? 127 : 128), the fourth byte 0."""
    m = math.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
    k = 1.0 / m
    w = 0
    for i in range(3):
        c = n[i] * k
        w |= (js_toint(c * (127 if c > 0 else 128), 8) & 0xFF) << (8 * i)
    return w


def quantizers():
    """UVs outside [0, 1] wrap: 1.5 * 32767 = 49150.5 truncates to 49150,
    which Int16 stores as 49150 - 65536 = -16386 (a repeating texture's UV
    decodes near -0.5); -1.5 * 32768 = -49152 stores as 16384."""
    uvs = [[0.5, 0.25], [1.0, 0.0], [1.5, 2.25], [-0.25, -1.5], [3.0, -0.0], [1e-5, 0.999999]]
    normals = [[0.0, 0.0, -1.0], [0.6, 0.8, 0.0], [-0.6, -0.8, 0.0], [0.0, 2.0, 0.0]]
    return {"uv": [{"uv": uv, "word": uv_word(*uv)} for uv in uvs],
            "normal": [{"normal": n, "word": normal_word(n)} for n in normals],
            "why": "typed-array stores truncate toward zero and wrap modulo 2^16 / 2^8"}


def env_black_bin():
    """env_sampler.js:59-95 on a 4 x 2 map of white texels with exponents
    128 + k (radiance 2^k v, v = luma(255,255,255)/255) and one black texel.
    The sort (b.rad - a.rad; Array.prototype.sort is stable) orders equal
    radiances row-major.  numBins = max(32, 2 ceil(19v / 8v)) = 32, so
    binSize = 19v/32 < v: every texel with light closes a bin at the next
    step, and the closing push after the loop gives the black texel a bin of
    its own.  Eight one-texel bins: every texel, the black one included, has
    pdf (1/8) (8/1) / (2 pi^2)."""
    ks = [[0, 0, 1, 1], [2, None, 0, 3]]
    rgbe = [[[255, 255, 255, 128 + k] if k is not None else [0, 0, 0, 128] for k in row] for row in ks]
    order = [(3, 1), (0, 1), (2, 0), (3, 0), (0, 0), (1, 0), (2, 1), (1, 1)]
    pdf = (1.0 / 8.0) * (8.0 / 1.0) * (1.0 / (math.pi * math.pi * 2.0))
    return {"rgbe": rgbe, "bins": [[i, i + 1] for i in range(8)], "coords": [list(c) for c in order],
            "pdf_f32_bits": "0x%08x" % int(np.float32(pdf).view(np.uint32)),
            "why": "the bin walk closes bins before adding; the last bin is pushed unconditionally"}


def main():
    c, s = math.cos(3 * math.pi / 8), math.sin(3 * math.pi / 8)
    out = {
        "rand_one": rand_one(),
        "nan_tangent": {"normal": [0.0, 1.0, 0.0], "tangent_word": 0, "bitangent_word": 0,
                        "normal_word": 0x00007F00,
                        "why": "normalize(cross(+y, +y)) = NaN; Int8Array stores NaN as 0"},
        "env_theta_roundtrip": {"w": 8, "h": 4, "theta": 0.25, "texel": [3, 1], "u": 0.1875, "v": 0.375,
                                "direction": [c * s, c, s * s], "pdf_texel": [3, 1],
                                "why": "sampleEnv subtracts theta, envPdf adds it back"},
        "quantizers": quantizers(),
        "env_black_bin": env_black_bin(),
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "wgsl_quirks.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(path)


if __name__ == "__main__":
    main()
