"""Environment ingestion: RGBE PNG (the reference's format) and Radiance .hdr."""
import numpy as np

from pike_gb300 import synth
from pike_gb300.envmap import load_env, read_hdr, write_hdr
from pike_gb300.image import encode_png


def _env(w=64, h=32, seed=3):
    e = synth.rgbe_encode(synth.hdr_env(seed, w, h, sun=80.0))
    e[3:7, 10:40] = e[3, 10]  # runs for the RLE paths
    return e


def test_hdr_rle_round_trip(tmp_path):
    e = _env()
    for rle in (True, False):
        data = write_hdr(e, rle=rle)
        assert np.array_equal(read_hdr(data), e)
        p = tmp_path / f"env_{rle}.hdr"
        p.write_bytes(data)
        assert np.array_equal(load_env(str(p)), e)


def test_hdr_orientation_flags():
    e = _env(16, 8)
    data = write_hdr(e, rle=False).replace(b"-Y 8 +X 16", b"+Y 8 -X 16")
    assert np.array_equal(read_hdr(data), e[::-1, ::-1])


def test_hdr_old_style_runs():
    row = np.array([[10, 20, 30, 130], [1, 1, 1, 3], [5, 6, 7, 128]], np.uint8)
    data = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X 5\n" + row.tobytes()
    img = read_hdr(data)
    assert img[0, :4].tolist() == [[10, 20, 30, 130]] * 4 and img[0, 4].tolist() == [5, 6, 7, 128]


def test_rgbe_png(tmp_path):
    e = _env()
    p = tmp_path / "env.png"
    p.write_bytes(encode_png(e))
    assert np.array_equal(load_env(str(p)), e)
