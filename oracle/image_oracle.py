"""Test infrastructure: a numpy restatement of the reference's display encoding
(PNGWriter.visualizedRGBA8Pixels, Sources/DenrimRendererKit/Image/PNGWriter.swift:35-178),
the checker for the device encoder (`dk_encode_rgba8`, `dk_session_read_rgba8`).

Only tests/ may import this module.  Every formula is evaluated in float32 in
the reference's operation order (numpy does not contract into FMAs); Swift's
`max(x, y)` / `min(x, y)` keep the first operand when the second is NaN, which
`np.fmax` / `np.fmin` do as well for these call sites.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32
BEAUTY, DEPTH, NORMAL, ALBEDO, MATERIAL_ID, OBJECT_ID, MOTION_VECTOR = range(7)


def _byte(v):  # UInt8(max(0, min(255, v)))
    return np.fmax(f32(0), np.fmin(f32(255), v)).astype(np.uint8)


def _gamma(v):  # pow(max(0, min(1, v)), 1 / 2.2)
    return np.power(np.fmax(f32(0), np.fmin(f32(1), v)), f32(1) / f32(2.2))


def tonemap(linear):  # :146-152 (inf / inf -> NaN -> min(1, NaN) = 1, as in Swift)
    exposed = np.fmax(f32(0), linear) * f32(0.8)
    with np.errstate(over="ignore", invalid="ignore"):
        mapped = (exposed * (f32(2.51) * exposed + f32(0.03))) / (exposed * (f32(2.43) * exposed + f32(0.59)) + f32(0.14))
    return _byte(_gamma(mapped) * f32(255))


def display_linear(linear):  # :153-156
    return _byte(_gamma(linear) * f32(255))


def alpha(a):  # :158-160
    return _byte(a * f32(255))


def signed(v):  # :176-178
    return _byte((v * f32(0.5) + f32(0.5)) * f32(255))


def color_for_id(ids):  # :162-174, wrapping 32-bit arithmetic
    h = ids.astype(np.uint32)
    h = h * np.uint32(747796405) + np.uint32(2891336453)
    h = np.right_shift(h, np.right_shift(h, np.uint32(28)) + np.uint32(4)) ^ h
    h = h * np.uint32(277803737)
    h = np.right_shift(h, np.uint32(22)) ^ h
    r = 64 + (h & 0x7F)
    g = 64 + ((h >> 8) & 0x7F)
    b = 64 + ((h >> 16) & 0x7F)
    return np.stack([r, g, b], -1).astype(np.uint8)


def visualized_rgba8(pixels: np.ndarray, kind: int) -> np.ndarray:
    """(h, w, 4) float32 output plane -> (h, w, 4) uint8, as the reference's PNG export."""
    px = np.ascontiguousarray(pixels, dtype=np.float32)
    out = np.zeros(px.shape[:-1] + (4,), np.uint8)
    r, g, b, a = px[..., 0], px[..., 1], px[..., 2], px[..., 3]
    if kind == BEAUTY:
        out[..., 0], out[..., 1], out[..., 2], out[..., 3] = tonemap(r), tonemap(g), tonemap(b), alpha(a)
    elif kind in (NORMAL, ALBEDO):
        out[..., 0], out[..., 1], out[..., 2] = display_linear(r), display_linear(g), display_linear(b)
        out[..., 3] = alpha(a) if kind == ALBEDO else 255
    elif kind == DEPTH:  # encodeDepthPixels (:83-116)
        valid = np.isfinite(r) & (r > 0)
        if not valid.any():
            return out
        lo, hi = r[valid].min(), r[valid].max()
        rng = f32(hi - lo)
        t = np.ones_like(r) if rng <= f32(np.finfo(np.float32).eps) else (r - lo) / rng
        d = _byte((f32(0.1) + t * f32(0.9)) * f32(255))
        out[..., 3] = 255
        for c in range(3):
            out[..., c] = np.where(valid, d, 0)
    elif kind in (MATERIAL_ID, OBJECT_ID):  # encodeIDPixels (:118-138); rounded() = nearest, ties away
        r64 = r.astype(np.float64)
        ids = np.sign(r64) * np.floor(np.abs(r64) + 0.5)
        pos = ids > 0
        col = color_for_id(np.where(pos, np.minimum(ids, 4294967040.0), 0).astype(np.uint64))
        for c in range(3):
            out[..., c] = np.where(pos, col[..., c], 0)
        out[..., 3] = 255
    else:  # encodeMotionVectorPixels (:140-158)
        mag = np.fmax(np.abs(r), np.abs(g))
        scale = np.fmax(f32(max(f32(0), np.nanmax(mag) if mag.size else f32(0))), f32(1))
        out[..., 0], out[..., 1] = signed(r / scale), signed(g / scale)
        out[..., 2], out[..., 3] = 128, 255
    return out
