"""Environment-map ingestion.

The reference loads its environment as an image whose RGBA bytes hold RGBE
(render/scene.js:38, env_sampler.js:43-48: radiance = rgb/255 * 2^(a-128));
`load_env` reads such a PNG, or a Radiance .hdr file, whose RGBE bytes are
used the same way (the reference's own .hdr loader, render/util/hdr_loader.js,
is an unfinished stub with an empty RLE decoder and is not called).
"""
from __future__ import annotations

import re

import numpy as np

from .image import decode_png


def read_hdr(data: bytes) -> np.ndarray:
    """Radiance RGBE (.hdr / .pic) -> (H, W, 4) uint8 RGBE bytes, top row first.
    Supports flat scanlines and both run-length encodings."""
    if not (data.startswith(b"#?RADIANCE") or data.startswith(b"#?RGBE")):
        raise ValueError("not a Radiance file")
    end = data.index(b"\n\n")
    header = data[:end].decode("ascii", "replace")
    fmt = re.search(r"FORMAT=(\S+)", header)
    if fmt and fmt.group(1) != "32-bit_rle_rgbe":
        raise ValueError(f"unsupported format {fmt.group(1)}")
    nl = data.index(b"\n", end + 2)
    m = re.match(r"([-+])Y (\d+) ([-+])X (\d+)", data[end + 2:nl].decode("ascii"))
    if not m:
        raise ValueError("unsupported resolution line")
    h, w = int(m.group(2)), int(m.group(4))
    pos = nl + 1
    out = np.zeros((h, w, 4), np.uint8)
    buf = memoryview(data)
    for y in range(h):
        if 8 <= w < 32768 and data[pos] == 2 and data[pos + 1] == 2 and (data[pos + 2] & 0x80) == 0:
            if (data[pos + 2] << 8 | data[pos + 3]) != w:
                raise ValueError("scanline width mismatch")
            pos += 4
            for ch in range(4):
                x = 0
                while x < w:
                    count = data[pos]
                    pos += 1
                    if count > 128:
                        count -= 128
                        out[y, x:x + count, ch] = data[pos]
                        pos += 1
                    else:
                        out[y, x:x + count, ch] = np.frombuffer(buf[pos:pos + count], np.uint8)
                        pos += count
                    x += count
        else:
            x, shift = 0, 0
            while x < w:
                px = np.frombuffer(buf[pos:pos + 4], np.uint8)
                pos += 4
                if px[0] == 1 and px[1] == 1 and px[2] == 1:  # old-style run of the previous pixel
                    n = int(px[3]) << shift
                    out[y, x:x + n] = out[y, x - 1]
                    x += n
                    shift += 8
                else:
                    out[y, x] = px
                    x += 1
                    shift = 0
    if m.group(1) == "+":
        out = out[::-1]
    if m.group(3) == "-":
        out = out[:, ::-1]
    return np.ascontiguousarray(out)


def write_hdr(img_rgbe: np.ndarray, rle: bool = True) -> bytes:
    """(H, W, 4) RGBE bytes -> Radiance file bytes (new-style RLE when possible)."""
    h, w = img_rgbe.shape[:2]
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        row = img_rgbe[y]
        if not rle or not 8 <= w < 32768:
            out += row.tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 0xFF])
        for ch in range(4):
            v = row[:, ch]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and v[x + run] == v[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, int(v[x])])
                    x += run
                    continue
                start = x
                while x < w and x - start < 128:
                    if x + 2 < w and v[x] == v[x + 1] == v[x + 2]:
                        break
                    x += 1
                out += bytes([x - start]) + v[start:x].tobytes()
    return bytes(out)


def load_env(path: str) -> np.ndarray:
    """An environment file -> (H, W, 4) uint8 RGBE bytes for pk_env_build."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] == b"\x89PNG\r\n\x1a\n":
        img = decode_png(data)
        if img.shape[2] != 4:
            raise ValueError("an RGBE environment PNG needs an alpha channel (the exponent)")
        return img
    return read_hdr(data)
