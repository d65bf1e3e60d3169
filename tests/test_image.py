"""Headless PNG output of the display buffer."""
import zlib

import numpy as np

from pike_gb300.image import decode_png, encode_png


def test_png_round_trip_rgba_and_rgb():
    rng = np.random.default_rng(0)
    for c in (3, 4):
        img = rng.integers(0, 256, (17, 23, c), dtype=np.uint8)
        data = encode_png(img)
        assert data[:8] == b"\x89PNG\r\n\x1a\n"
        assert np.array_equal(decode_png(data), img)


def test_png_decoder_handles_all_filters():
    # hand-built 2x2 RGB image whose rows use filters 1 (sub) and 4 (paeth)
    import struct
    rows = [bytes([1, 10, 20, 30, 5, 5, 5]), bytes([4, 1, 2, 3, 4, 5, 6])]
    raw = b"".join(rows)

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 2, 2, 8, 2, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
    img = decode_png(data)
    assert img[0, 0].tolist() == [10, 20, 30] and img[0, 1].tolist() == [15, 25, 35]
    # row 1, pixel 0: paeth(a=0, b=up, c=0) = up
    assert img[1, 0].tolist() == [11, 22, 33]
