"""The oracle's FP64 companion (om_render64.h): every contribution of the
FP32 passes recomputed in FP64 along the same light paths.  The FP32 result
is unchanged by tracking, agrees with the FP64 evaluation to the stated
relative error, and the converged image lies inside the 3-sigma Monte Carlo
band of the FP64 render."""
import numpy as np

from pike_gb300 import synth


def fp64_stats(a32: np.ndarray, a64: np.ndarray, sd: np.ndarray, frames: int) -> dict:
    d = np.abs(a32 - a64)
    lit = a64 > 1e-6
    rel = d[lit] / a64[lit]
    band = 3.0 * sd / np.sqrt(frames)
    noisy = sd > 0
    # pixels without Monte Carlo noise (a constant estimate) must agree to rounding
    inside = np.where(noisy, d <= band, d <= 1e-6 * np.maximum(np.abs(a64), 1e-30))
    return {"rel_median": float(np.median(rel)), "rel_p99": float(np.percentile(rel, 99)),
            "rel_max": float(rel.max()), "band_fraction_max": float((d[noisy] / band[noisy]).max()),
            "inside_3sigma": float(inside.mean())}


def test_fp64_companion_small_scene(oracle):
    src = synth.small_scene(width=128, height=128)  # 770 triangles, 4 bounces
    frames = 16
    plain = oracle.Prepared(src, threads=8).r
    plain.set_render_state(0)
    P = oracle.Prepared(src, threads=8)
    R = P.r
    R.set_track64(True)
    R.set_render_state(0)
    for _ in range(frames):
        plain.tick(4)
        R.tick(4)
    a32 = R.accum()
    assert np.array_equal(a32.view(np.uint32), plain.accum().view(np.uint32))  # tracking changes nothing
    assert R.frames64() == frames
    s = fp64_stats(a32[..., :3].astype(np.float64), R.accum64()[..., :3], R.std64()[..., :3], frames)
    assert s["rel_median"] < 1e-6 and s["rel_p99"] < 1e-5 and s["rel_max"] < 1e-4, s
    assert s["inside_3sigma"] == 1.0, s
