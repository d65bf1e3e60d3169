"""TexturePacker (render/util/texture_packer.js:55-136): material maps to atlas layers.

The reference draws every layer with WebGL2 (``WebGLTextureWriter``,
texture_packer.js:230-336) and reads it back with ``readPixels``.  No graphics
API exists here, so this module restates what that draw computes:

* ``drawColor`` (:274-279): ``gl.clearColor(r, g, b, 1)`` fills the layer; the
  float to unorm8 conversion is ``floor(clamp(c, 0, 1) * 255 + 0.5)`` and the
  alpha is forced to 255.
* ``drawTexture`` (:293-309): a full-viewport quad samples the image with
  ``texture()``: LINEAR min/mag filters without mipmaps, S wrap REPEAT, T wrap
  CLAMP_TO_EDGE (:245-249).  Fragment (i, j) samples at ``((i + .5) / res,
  (j + .5) / res)``; the filter is the GL bilinear rule around ``u * w - .5``.
  ``corrected`` images are uploaded as SRGB8_ALPHA8, so their colour channels
  are decoded to linear (GL sRGB EOTF) before filtering; alpha stays linear.
  The framebuffer is plain RGBA8: the filtered value is re-quantised with the
  rule above.  Row 0 of ``readPixels`` is the bottom of the framebuffer, where
  ``texCoord.y`` is 0, which samples the image's first row: layers keep the
  image's row order.

Arithmetic is IEEE double throughout, so the packed bytes are the same on any
host.  A GPU's fixed-point filter weights can differ from this by one unorm8
step on some texels; the shading kernels consume the packed bytes as given.
"""
from __future__ import annotations

import math

import numpy as np


def unorm8(c) -> np.ndarray:
    """float -> unorm8 of an RGBA8 colour buffer: floor(clamp(c, 0, 1) * 255 + 0.5); NaN -> 0."""
    x = np.asarray(c, np.float64)
    x = np.where(np.isnan(x), 0.0, np.clip(x, 0.0, 1.0))
    return np.floor(x * 255.0 + 0.5).astype(np.uint8)


def _srgb_to_linear_table() -> np.ndarray:
    cs = np.arange(256, dtype=np.float64) / 255.0
    out = np.empty(256, np.float64)
    for i, c in enumerate(cs):  # GL's sRGB EOTF
        out[i] = c / 12.92 if c <= 0.04045 else math.pow((c + 0.055) / 1.055, 2.4)
    return out


SRGB_TO_LINEAR = _srgb_to_linear_table()


class AtlasImage:
    """A decoded image as the loader hands it to the packer: rgba8 pixels, a
    source key (``currentSrc`` in the reference) and the mutable ``corrected``
    flag that ``addTexture`` sets (texture_packer.js:90)."""

    def __init__(self, pixels: np.ndarray, src: str):
        px = np.asarray(pixels, np.uint8)
        if px.ndim == 3 and px.shape[2] == 1:
            px = px[..., 0]
        if px.ndim == 2:
            px = np.stack([px, px, px, np.full_like(px, 255)], -1)
        elif px.shape[2] == 3:
            px = np.concatenate([px, np.full(px.shape[:2] + (1,), 255, np.uint8)], -1)
        elif px.shape[2] == 2:
            px = np.concatenate([px[..., :1], px[..., :1], px[..., :1], px[..., 1:2]], -1)
        self.pixels = np.ascontiguousarray(px)
        self.currentSrc = src
        self.corrected = False

    @property
    def height(self) -> int:
        return int(self.pixels.shape[0])

    @property
    def width(self) -> int:
        return int(self.pixels.shape[1])


def draw_color(color, res: int) -> np.ndarray:
    """WebGLTextureWriter.drawColor: the layer cleared to (r, g, b, 1)."""
    c = list(color) + [0.0] * max(0, 3 - len(color))
    px = np.empty((res, res, 4), np.uint8)
    px[..., :3] = unorm8([c[0], c[1], c[2]])
    px[..., 3] = 255
    return px


def draw_texture(image: AtlasImage, res: int) -> np.ndarray:
    """WebGLTextureWriter.drawTexture: the image resampled to res x res."""
    src = image.pixels.astype(np.float64)
    if image.corrected:
        src = np.concatenate([SRGB_TO_LINEAR[image.pixels[..., :3]], src[..., 3:4] / 255.0], -1)
    else:
        src = src / 255.0
    h, w = image.height, image.width
    t = (np.arange(res, dtype=np.float64) + 0.5) / res
    x = t * w - 0.5
    y = t * h - 0.5
    x0, y0 = np.floor(x), np.floor(y)
    a, b = x - x0, y - y0
    i0 = x0.astype(np.int64)
    j0 = y0.astype(np.int64)
    i_lo, i_hi = np.mod(i0, w), np.mod(i0 + 1, w)          # S: REPEAT
    j_lo, j_hi = np.clip(j0, 0, h - 1), np.clip(j0 + 1, 0, h - 1)  # T: CLAMP_TO_EDGE
    a = a[None, :, None]
    b = b[:, None, None]
    t00 = src[j_lo][:, i_lo]
    t10 = src[j_lo][:, i_hi]
    t01 = src[j_hi][:, i_lo]
    t11 = src[j_hi][:, i_hi]
    v = (1.0 - a) * (1.0 - b) * t00 + a * (1.0 - b) * t10 + (1.0 - a) * b * t01 + a * b * t11
    return unorm8(v)


def _color_key(color) -> str:
    """color.join(' ') with JS number formatting for the values a material holds."""
    def fmt(v):
        v = float(v)
        if math.isnan(v):
            return "NaN"
        if v == 0.0:
            return "0"
        if math.isinf(v):
            return "Infinity" if v > 0 else "-Infinity"
        if v == int(v) and abs(v) < 1e21:
            return str(int(v))
        return repr(v)
    return " ".join(fmt(v) for v in color)


class TexturePacker:
    """texture_packer.js:55-136 (the ImageLayer/reserveImages path is unused by
    scene.js: its call is commented out at scene.js:33)."""

    def __init__(self, atlasRes: int = 1024):
        self.res = int(atlasRes)
        self.imageSet: list = []
        self.imageKeys: dict = {}
        self.maxRes = 1

    def addTexture(self, image: AtlasImage, corrected: bool = False) -> int:
        key = image.currentSrc
        # `if (this.imageKeys[key])` is a truthiness test: an image stored at
        # index 0 is not found and is pushed again (texture_packer.js:87-88).
        if self.imageKeys.get(key):
            return self.imageKeys[key]
        self.maxRes = max(self.maxRes, image.height)
        image.corrected = bool(corrected)
        self.imageSet.append(image)
        self.imageKeys[key] = len(self.imageSet) - 1
        return self.imageKeys[key]

    def addColor(self, color) -> int:
        key = _color_key(color)
        if key in self.imageKeys:
            return self.imageKeys[key]
        self.imageSet.append(list(color))
        self.imageKeys[key] = len(self.imageSet) - 1
        return self.imageKeys[key]

    def getResolution(self):
        if self.maxRes < self.res:
            self.res = self.maxRes
        return [self.res, self.res, len(self.imageSet)]

    def getPixels(self) -> np.ndarray:
        """(layers, res, res, 4) uint8; call getResolution() first, as
        ShadeHitPass.createAtlasTetxure does (shade_hit_pass.js:58-60)."""
        out = np.empty((len(self.imageSet), self.res, self.res, 4), np.uint8)
        for i, img in enumerate(self.imageSet):
            out[i] = draw_color(img, self.res) if isinstance(img, list) else draw_texture(img, self.res)
        return out
