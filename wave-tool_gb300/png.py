"""PNG heightmap loading: the part of stb_image the reference uses to read its
heightmap (src/render-engine.cpp:1308-1322: stbi_load forced to RGBA8 with
vertical flip on load, then a GL_RGBA8 texture).

`decode` inflates with the standard library's zlib and undoes the five
scanline filters; every colour type and bit depth of the PNG specification
is handled the way stb_image converts it to 8 bits per channel (grey of
depth 1/2/4 scaled to 0..255, palette indices looked up, 16-bit samples
keep their high byte), including Adam7 interlacing.  `load_heightmap` sends
the pixels to the GPU, where wt_heightmap_from_unorm8 flips rows and turns
channel 0 (red, or grey) into R32F texels c / 255.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

_SIGNATURE = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
# Adam7: (x0, y0, dx, dy) per pass
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


class PngError(ValueError):
    pass


def _unfilter(data: bytes, pos: int, width: int, height: int, bits_pp: int) -> tuple[np.ndarray, int]:
    """Scanlines of one (sub)image -> (height, row_bytes) uint8; returns the
    array and the position after it."""
    row_bytes = (width * bits_pp + 7) // 8
    bpp = max(1, bits_pp // 8)  # filter byte distance
    out = np.zeros((height, row_bytes), np.uint8)
    prev = bytearray(row_bytes)
    for r in range(height):
        if pos + 1 + row_bytes > len(data):
            raise PngError("truncated image data")
        f = data[pos]
        line = bytearray(data[pos + 1:pos + 1 + row_bytes])
        pos += 1 + row_bytes
        if f == 0:
            pass
        elif f == 1:
            for i in range(bpp, row_bytes):
                line[i] = (line[i] + line[i - bpp]) & 255
        elif f == 2:
            line = bytearray(((np.frombuffer(line, np.uint8).astype(np.uint16) +
                               np.frombuffer(prev, np.uint8)) & 255).astype(np.uint8).tobytes())
        elif f == 3:
            for i in range(row_bytes):
                a = line[i - bpp] if i >= bpp else 0
                line[i] = (line[i] + ((a + prev[i]) >> 1)) & 255
        elif f == 4:
            for i in range(row_bytes):
                a = line[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                line[i] = (line[i] + (a if pa <= pb and pa <= pc else (b if pb <= pc else c))) & 255
        else:
            raise PngError(f"unknown filter type {f}")
        out[r] = np.frombuffer(line, np.uint8)
        prev = line
    return out, pos


def _samples(rows: np.ndarray, width: int, depth: int, channels: int) -> np.ndarray:
    """Unfiltered rows -> (h, w, channels) samples (uint16 for depth 16)."""
    h = rows.shape[0]
    if depth == 8:
        return rows[:, :width * channels].reshape(h, width, channels)
    if depth == 16:
        return rows[:, :2 * width * channels].reshape(h, width * channels, 2).astype(np.uint16).dot(
            np.array([256, 1], np.uint16)).reshape(h, width, channels)
    bits = np.unpackbits(rows, axis=1)[:, :width * depth].reshape(h, width, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint8)
    return (bits * weights).sum(axis=2, dtype=np.uint8).reshape(h, width, 1)


def decode(data: bytes) -> np.ndarray:
    """PNG bytes -> (height, width, channels) uint8, top row first, channels
    as stored (1 grey, 2 grey+alpha, 3 RGB, 4 RGBA; palette images give RGB
    or RGBA).  Samples converted to 8 bits the way stb_image does."""
    if data[:8] != _SIGNATURE:
        raise PngError("not a PNG file")
    pos = 8
    ihdr = None
    idat = bytearray()
    palette = None
    trns = None
    while pos + 8 <= len(data):
        (length,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + length]
        if len(body) != length:
            raise PngError("truncated chunk")
        if zlib.crc32(kind + body) & 0xFFFFFFFF != struct.unpack(">I", data[pos + 8 + length:pos + 12 + length])[0]:
            raise PngError(f"CRC mismatch in {kind!r} chunk")
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + length
    if ihdr is None:
        raise PngError("missing IHDR")
    width, height, depth, ctype, comp, filt, interlace = ihdr
    if ctype not in _CHANNELS or comp != 0 or filt != 0 or interlace not in (0, 1):
        raise PngError(f"unsupported IHDR {ihdr}")
    if depth not in ((1, 2, 4, 8, 16) if ctype == 0 else (1, 2, 4, 8) if ctype == 3 else (8, 16)):
        raise PngError(f"bit depth {depth} invalid for colour type {ctype}")
    if width == 0 or height == 0:
        raise PngError("empty image")
    channels = _CHANNELS[ctype]
    raw = zlib.decompress(bytes(idat))
    bits_pp = depth * channels
    if interlace == 0:
        rows, _ = _unfilter(raw, 0, width, height, bits_pp)
        img = _samples(rows, width, depth, channels)
    else:
        img = np.zeros((height, width, channels), np.uint16 if depth == 16 else np.uint8)
        p = 0
        for x0, y0, dx, dy in _ADAM7:
            pw = (width - x0 + dx - 1) // dx if width > x0 else 0
            ph = (height - y0 + dy - 1) // dy if height > y0 else 0
            if pw == 0 or ph == 0:
                continue
            rows, p = _unfilter(raw, p, pw, ph, bits_pp)
            img[y0::dy, x0::dx] = _samples(rows, pw, depth, channels)
    if depth == 16:
        img = (img >> 8).astype(np.uint8)
    elif ctype == 0 and depth < 8:
        img = (img.astype(np.uint16) * (255 // ((1 << depth) - 1))).astype(np.uint8)
    if ctype == 3:
        if palette is None:
            raise PngError("palette image without PLTE")
        idx = img[..., 0]
        if idx.max(initial=0) >= len(palette):
            raise PngError("palette index out of range")
        rgb = palette[idx]
        if trns is not None:
            alpha = np.full(len(palette), 255, np.uint8)
            alpha[:len(trns)] = trns[:len(palette)]
            return np.ascontiguousarray(np.concatenate([rgb, alpha[idx][..., None]], axis=2))
        return np.ascontiguousarray(rgb)
    return np.ascontiguousarray(img)


def load_heightmap(path, sample_scale: float = 0.02, disp_scale: float = 1.0, wrap: int = 1,
                   flip_vertically: bool = True, stream=None):
    """A DeviceHeightmap from a PNG file, as src/render-engine.cpp:1308-1322
    and src/texture.cpp:54-71 set it up (flipped on load, GL_MIRRORED_REPEAT
    = wrap 1).  Defaults are the reference's sampler scales
    (heightmapSampleScale 0.02, heightmapDisplacementScale 1.0)."""
    from . import DeviceHeightmap, check, lib, stream_handle
    import torch
    img = decode(Path(path).read_bytes())
    h, w, ch = img.shape
    px = torch.from_numpy(img.reshape(-1)).to("cuda")
    texels = torch.empty((h, w), dtype=torch.float32, device="cuda")
    check(lib().wt_heightmap_from_unorm8(px.data_ptr(), w, h, ch, w * ch, int(bool(flip_vertically)),
                                         texels.data_ptr(), stream_handle(stream)))
    return DeviceHeightmap(texels, sample_scale, disp_scale, wrap)
