"""Headless surface images: the colour-mapped pressure textures of an
object's facets written as PNG files (the reference shows them through
EGL/OpenGL, src/ModelGl.cpp:222-341; here they leave as plain images).

``facet_textures`` splits the per-cell RGBA colours returned by
``api.get_surface_colours`` into one (numYpnts, numXpnts, 4) texture per facet;
``write_png`` writes an RGBA image with zlib only (no extra dependencies).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


def write_png(path, rgba):
    """Write an (h, w, 4) uint8 array (row 0 at the top) as an RGBA PNG."""
    a = np.ascontiguousarray(np.asarray(rgba, dtype=np.uint8))
    h, w, c = a.shape
    if c != 4:
        raise ValueError("expected RGBA")
    raw = b"".join(b"\x00" + a[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(path, "wb") as fh:
        fh.write(png)
    return path


def read_png_rgba(path):
    """Read back a PNG written by write_png (8-bit RGBA, no interlace)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[y * (4 * w + 1) + 1:(y + 1) * (4 * w + 1)] for y in range(h)]
    return np.frombuffer(b"".join(rows), dtype=np.uint8).reshape(h, w, 4)


def to_uint8(rgba):
    return (np.clip(np.asarray(rgba, np.float32), 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)


def facet_textures(layout_ints, rgba):
    """Per-facet textures from per-cell colours: texel (x, y) of facet f is
    cell y*numXpnts + x of that facet (the layout of the pressures)."""
    out, off = [], 0
    for nx, ny, _neg in np.asarray(layout_ints):
        n = int(nx) * int(ny)
        out.append(np.asarray(rgba[off:off + n]).reshape(int(ny), int(nx), 4))
        off += n
    return out


def atlas(textures, pad=2):
    """All facet textures side by side, texture row 0 at the image bottom (as
    a texture is drawn), on a transparent background."""
    if not textures:
        return np.zeros((1, 1, 4), np.uint8)
    h = max(t.shape[0] for t in textures)
    w = sum(t.shape[1] for t in textures) + pad * (len(textures) - 1)
    img = np.zeros((h, w, 4), np.uint8)
    x = 0
    for t in textures:
        t8 = to_uint8(t)[::-1]
        img[h - t8.shape[0]:, x:x + t8.shape[1]] = t8
        x += t8.shape[1] + pad
    return img


def save_object_png(api, object_type, idx, path):
    """Colour-map an object's surface (SoundVisualisationInit settings) to a PNG atlas."""
    ints, _ = api.get_fragment_layout(object_type, idx)
    rgba = api.get_surface_colours(object_type, idx)
    return write_png(path, atlas(facet_textures(ints, rgba)))
