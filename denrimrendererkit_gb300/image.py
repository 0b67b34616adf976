"""Displayed-image helpers around the device encoder (`RenderSession.rgba8`,
`RenderSession.write_png`, `dk_encode_rgba8`):

* `read_png` decodes an 8-bit RGBA PNG (the files `write_png` produces, or any
  non-interlaced 8-bit RGBA PNG) into a (height, width, 4) uint8 array;
* `image_metrics` and `alpha_metrics` restate the reference's render-test
  metrics (Tests/RenderReferenceTests/ImageMetrics.swift:55-118 and
  TransparentExportRenderTests.swift, AlphaMetricReader), which the reference
  compares against its stored baselines (ReferenceMetrics/*.json).

Both metric readers draw the decoded image into a premultiplied-alpha RGBA8
context first (CGImageAlphaInfo.premultipliedLast); for opaque pixels that is
the identity, otherwise each colour byte becomes round(c * a / 255).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def read_png(path: str) -> np.ndarray:
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, width, height = 8, b"", 0, 0
    while pos < len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + length]
        if zlib.crc32(kind + body) != struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])[0]:
            raise ValueError(f"bad CRC in {kind!r} chunk")
        if kind == b"IHDR":
            width, height, depth, color, _, _, interlace = struct.unpack(">IIBBBBB", body)
            if depth != 8 or color != 6 or interlace != 0:
                raise ValueError("only non-interlaced 8-bit RGBA PNGs are read")
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + length
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(height, width * 4 + 1)
    out = np.zeros((height, width * 4), np.int32)
    for y in range(height):  # the five PNG row filters
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        prev = out[y - 1] if y else np.zeros(width * 4, np.int32)
        if f == 0:
            out[y] = line
        elif f == 2:
            out[y] = (line + prev) & 0xFF
        else:
            row = np.zeros(width * 4, np.int32)
            for x in range(width * 4):
                a = row[x - 4] if x >= 4 else 0
                b = prev[x]
                c = prev[x - 4] if x >= 4 else 0
                if f == 1:
                    pred = a
                elif f == 3:
                    pred = (a + b) // 2
                else:  # Paeth
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                row[x] = (line[x] + pred) & 0xFF
            out[y] = row
    return out.reshape(height, width, 4).astype(np.uint8)


def _premultiplied(rgba: np.ndarray) -> np.ndarray:
    px = rgba.astype(np.int64)
    a = px[..., 3:4]
    rgb = np.where(a == 255, px[..., :3], (px[..., :3] * a + 127) // 255)
    return np.concatenate([rgb, a], axis=-1)


def image_metrics(rgba: np.ndarray) -> dict:
    """ImageMetricReader.metrics (ImageMetrics.swift:55-118) of a (h, w, 4) uint8 image."""
    h, w = rgba.shape[:2]
    px = _premultiplied(rgba)
    r, g, b = px[..., 0], px[..., 1], px[..., 2]
    bright = (r + g + b) / 3.0
    colors = np.unique(((r // 32) << 16) | ((g // 32) << 8) | (b // 32))
    xs = np.arange(w)[None, :]
    ys = np.arange(h)[:, None]
    center = (xs >= w * 3 // 8) & (xs <= w * 5 // 8)
    top = center & (ys < h // 4)
    bottom = center & (ys > h * 3 // 4)
    return {
        "width": w, "height": h,
        "averageBrightness": float(bright.sum() / (w * h)),
        "maxBrightness": float(bright.max()),
        "uniqueColorEstimate": int(colors.size),
        "topCenterMaxBrightness": float(bright[top].max()) if top.any() else 0.0,
        "bottomCenterMaxBrightness": float(bright[bottom].max()) if bottom.any() else 0.0,
    }


def alpha_metrics(rgba: np.ndarray) -> dict:
    """AlphaMetricReader.metrics (TransparentExportRenderTests.swift) of a (h, w, 4) uint8 image."""
    h, w = rgba.shape[:2]
    a = _premultiplied(rgba)[..., 3]
    return {"width": w, "height": h, "minAlpha": int(a.min()), "maxAlpha": int(a.max()),
            "transparentPixels": int((a < 8).sum()), "opaquePixels": int((a > 247).sum())}
