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


def test_fp64_outliers_are_texel_flips_and_the_pole(oracle):
    """Where the FP32 passes and their FP64 evaluation differ by more than 1e-4
    per pixel, the cause is a texel choice, not arithmetic conditioning.  envPdf
    (shade_hit.wgsl:202-210) computes u = (1 + theta + atan2/2pi) mod 1 in
    binary32, so u moves in steps of 2^-23.  A direction within half a step of
    a texel boundary then gets the neighbouring pdf texel, and the bounce's MIS
    weight changes by the ratio of the two texels.  When the FP64 evaluation
    takes its texel indices from the FP32 lookups, all but one value fall
    below 1e-4.  That one (2.5e-4) is a bounce 1.3 degrees from the pole,
    where envPdf's 1/sin(acos y) scales the direction's binary32 rounding by
    1/(2(1 - |y|))."""
    src = synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256))
    frames, bounces = 16, 8
    rel, img = {}, {}
    for share in (False, True):
        R = oracle.Prepared(src, threads=8).r
        R.set_track64(True, share_texels=share)
        R.set_render_state(0)
        for _ in range(frames):
            R.tick(bounces)
        a32, a64 = R.accum(), R.accum64()[..., :3]
        img[share] = a32
        d = np.abs(a32[..., :3].astype(np.float64) - a64)
        rel[share] = np.where(a64 > 1e-6, d / np.maximum(a64, 1e-300), 0.0)
    assert np.array_equal(img[False].view(np.uint32), img[True].view(np.uint32))  # the FP32 image is untouched
    independent, shared = rel[False], rel[True]
    assert (independent > 1e-4).sum() >= 10 and independent.max() > 1e-3  # the texel flips
    assert (shared > 1e-4).sum() <= 2 and shared.max() < 5e-4, (int((shared > 1e-4).sum()), float(shared.max()))
    assert np.median(shared[shared > 0]) < 1e-6


def paired_band(R, F, frames: int, bounces: int, scale: float = 1.0):
    """Renders `frames` frames with the FP32 oracle R and the independent FP64
    renderer F (same seeds) and returns the paired statistics of the per-frame
    difference d = max(c32, 0) * scale - max(c64, 0): per pixel, the fraction
    inside |mean d| <= 3 se(d) + 1e-5 |a64| (se = sd / sqrt(frames); the 1e-5
    floor is rounding for pixels whose paths never diverge), and the image
    z-score of the mean difference over all pixels."""
    s1 = s2 = 0.0
    for _ in range(frames):
        R.tick(bounces)
        F.tick(bounces)
        d = np.maximum(R.color()[..., :3].astype(np.float64), 0.0) * scale - np.maximum(F.color()[..., :3], 0.0)
        s1 = s1 + d
        s2 = s2 + d * d
    m = s1 / frames
    se = np.sqrt(np.maximum(s2 / frames - m * m, 0.0) * frames / (frames - 1)) / np.sqrt(frames)
    a64 = F.accum()[..., :3]
    inside = float((np.abs(m) <= 3.0 * se + 1e-5 * np.abs(a64)).mean())
    SE = np.sqrt((se ** 2).sum()) / m.size
    return inside, float(m.mean() / SE) if SE > 0 else 0.0


def test_independent_fp64_render_band(oracle):
    """The FP32 reference path against the reference path rendered in binary64
    end to end (om_render_f64.h: its own hits, queues and branches from the
    same seeds).  Paths diverge where an FP32 decision flips, so pixels differ
    by Monte Carlo amounts; the paired 3-sigma band of the per-frame
    differences holds at every pixel and the image-level mean difference is
    within 4 standard errors.  The test has power: the same statistics on the
    FP32 image scaled by 1.002 fail."""
    cases = [(synth.small_scene(width=128, height=128), 32, 4),
             (synth.displaced_sphere_scene(subdivisions=6, width=160, height=90, env_size=(512, 256)), 32, 8)]
    for src, frames, bounces in cases:
        stats = {}
        for scale in (1.0, 1.002):
            R = oracle.Prepared(src, threads=8).r
            R.set_render_state(0)
            F = R.render64()
            stats[scale] = paired_band(R, F, frames, bounces, scale)
        inside, z = stats[1.0]
        assert inside == 1.0 and abs(z) < 4.0, stats
        inside_b, z_b = stats[1.002]
        assert inside_b < 0.9 and z_b > 4.0, stats
