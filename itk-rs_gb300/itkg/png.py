"""PNG image I/O, the reference's src/io/png.rs (PNGImageIO analog): the
on-disk format of the blur example (examples/blur_png.rs) and its test
(tests/blur_png.rs).  Host code; the pixels go to the GPU through Image /
DeviceImage.

Readers (png.rs:25-68) return a 2-D Image at index (0, 0), spacing 1,
origin 0 (png.rs:205-212):
  read_gray8 / read_rgb8 / read_rgba8     8 bits per channel: 16-bit files are
      reduced to their high byte, 1/2/4-bit grayscale is scaled to 0..255
      (the png crate's EXPAND | STRIP_16, png.rs:139-143)
  read_gray16 / read_rgb16 / read_rgba16  16-bit files only (png.rs:163-185)
The file's own colour type must be the one asked for (png.rs:149-155):
a palette or grey+alpha file is refused by every reader, as in the reference.
Writers (png.rs:74-128) store 8- or 16-bit (big-endian) samples, non-interlaced.
Interlaced (Adam7) files and every scanline filter type are decoded.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

from . import Image, Region

__all__ = ["read_gray8", "read_gray16", "read_rgb8", "read_rgba8", "read_rgb16", "read_rgba16",
           "write_gray8", "write_gray16", "write_rgb8", "write_rgba8", "write_rgb16", "write_rgba16",
           "PngError"]

_SIG = b"\x89PNG\r\n\x1a\n"
GRAY, RGB, PALETTE, GRAY_ALPHA, RGBA = 0, 2, 3, 4, 6
_CHANNELS = {GRAY: 1, RGB: 3, PALETTE: 1, GRAY_ALPHA: 2, RGBA: 4}
_NAMES = {GRAY: "Grayscale", RGB: "Rgb", PALETTE: "Indexed", GRAY_ALPHA: "GrayscaleAlpha", RGBA: "Rgba"}
# Adam7 passes: (x start, y start, x step, y step)
_ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


class PngError(IOError):
    """A PNG that cannot be read as asked (io::ErrorKind::InvalidData in png.rs)."""


def _chunks(data: bytes):
    if data[:8] != _SIG:
        raise PngError("not a PNG file")
    pos = 8
    while pos + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if len(body) != n or pos + 12 + n > len(data):
            raise PngError("truncated chunk")
        (crc,) = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        if zlib.crc32(kind + body) & 0xFFFFFFFF != crc:
            raise PngError(f"CRC mismatch in {kind!r} chunk")
        yield kind, body
        pos += 12 + n
        if kind == b"IEND":
            return
    raise PngError("missing IEND chunk")


def _unfilter(raw: bytes, width: int, height: int, bpp: int, row_bytes: int) -> np.ndarray:
    """Undo the scanline filters (PNG spec: None, Sub, Up, Average, Paeth)."""
    out = np.zeros((height, row_bytes), dtype=np.uint8)
    prev = np.zeros(row_bytes, dtype=np.int32)
    pos = 0
    for y in range(height):
        ft = raw[pos]
        line = np.frombuffer(raw, dtype=np.uint8, count=row_bytes, offset=pos + 1).astype(np.int32)
        pos += 1 + row_bytes
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft in (1, 3, 4):
            cur = line.copy()
            for i in range(row_bytes):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                if ft == 1:
                    p = a
                elif ft == 3:
                    p = (a + b) >> 1
                else:
                    c = prev[i - bpp] if i >= bpp else 0
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[i] = (cur[i] + p) & 0xFF
        else:
            raise PngError(f"unknown filter type {ft}")
        out[y] = cur
        prev = cur
    return out


def _samples(rows: np.ndarray, width: int, channels: int, depth: int) -> np.ndarray:
    """Filtered-free scanlines -> (height, width, channels) samples (uint8 or uint16)."""
    h = rows.shape[0]
    if depth == 16:
        s = rows[:, :width * channels * 2].reshape(h, width * channels, 2).astype(np.uint16)
        return ((s[..., 0] << 8) | s[..., 1]).reshape(h, width, channels)
    if depth == 8:
        return rows[:, :width * channels].reshape(h, width, channels)
    bits = np.unpackbits(rows, axis=1)[:, :width * channels * depth].reshape(h, width * channels, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint8)
    return (bits * weights).sum(axis=2).astype(np.uint8).reshape(h, width, channels)


def _decode(path, want_color: int, sixteen: bool):
    data = open(path, "rb").read()
    ihdr, idat, trns = None, [], None
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
    if ihdr is None:
        raise PngError("missing IHDR chunk")
    width, height, depth, color, comp, filt, interlace = ihdr
    if comp != 0 or filt != 0 or color not in _CHANNELS:
        raise PngError("unsupported PNG header")
    if color != want_color:
        raise PngError(f"PNG color type mismatch: expected {_NAMES[want_color]}, got {_NAMES[color]}")
    if sixteen and depth != 16:
        raise PngError(f"expected 16-bit PNG, got {depth}-bit")
    if trns is not None:
        # the png crate's EXPAND would add an alpha channel the typed readers do not hold
        raise PngError("PNG with a tRNS chunk: its alpha channel does not fit the requested pixel type")
    ch = _CHANNELS[color]
    raw = zlib.decompress(b"".join(idat))
    bpp = max(1, ch * depth // 8)
    img = np.zeros((height, width, ch), dtype=np.uint16 if depth == 16 else np.uint8)
    passes = _ADAM7 if interlace == 1 else [(0, 0, 1, 1)]
    pos = 0
    for x0, y0, dx, dy in passes:
        pw = (width - x0 + dx - 1) // dx if width > x0 else 0
        ph = (height - y0 + dy - 1) // dy if height > y0 else 0
        if pw == 0 or ph == 0:
            continue
        row_bytes = (pw * ch * depth + 7) // 8
        n = ph * (1 + row_bytes)
        if pos + n > len(raw):
            raise PngError("truncated image data")
        rows = _unfilter(raw[pos:pos + n], pw, ph, bpp, row_bytes)
        img[y0::dy, x0::dx] = _samples(rows, pw, ch, depth)
        pos += n
    if not sixteen:
        if depth == 16:
            img = (img >> 8).astype(np.uint8)  # STRIP_16: the high byte
        elif depth < 8:
            img = (img.astype(np.uint16) * 255 // ((1 << depth) - 1)).astype(np.uint8)  # EXPAND
    return img


class Image16(Image):
    """Image<u16, 2> / Image<VecPixel<u16, N>, 2> on the host: u16 samples are
    storage the GPU filters do not take (the reference's u16 NumericPixel is
    not on the Gaussian path), so this image has no device dtype."""

    def __init__(self, data: np.ndarray, components: int = 1):
        self.data = np.ascontiguousarray(data, dtype=np.uint16)
        self.components = components
        spatial = self.data.shape[:-1] if components > 1 else self.data.shape
        self.region = Region((0,) * len(spatial), tuple(reversed(spatial)))
        self.spacing = (1.0,) * len(spatial)
        self.origin = (0.0,) * len(spatial)
        self.dtype = None


def _image(px: np.ndarray, comps: int) -> Image:
    """make_image (png.rs:205-212): index 0, spacing 1, origin 0."""
    arr = np.ascontiguousarray(px[..., 0] if comps == 1 else px)
    if px.dtype == np.uint16:
        return Image16(arr, comps)
    return Image(arr, index=(0, 0), spacing=(1.0, 1.0), origin=(0.0, 0.0), components=comps)


def read_gray8(path) -> Image:
    """png.rs:25-29"""
    return _image(_decode(path, GRAY, False), 1)


def read_gray16(path) -> Image:
    """png.rs:31-36 (numpy uint16 samples)"""
    return _image(_decode(path, GRAY, True), 1)


def read_rgb8(path) -> Image:
    """png.rs:38-43"""
    return _image(_decode(path, RGB, False), 3)


def read_rgba8(path) -> Image:
    """png.rs:45-50"""
    return _image(_decode(path, RGBA, False), 4)


def read_rgb16(path) -> Image:
    """png.rs:52-61"""
    return _image(_decode(path, RGB, True), 3)


def read_rgba16(path) -> Image:
    """png.rs:63-72"""
    return _image(_decode(path, RGBA, True), 4)


def _chunk(kind: bytes, body: bytes) -> bytes:
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _encode(path, px: np.ndarray, color: int, depth: int):
    h, w = px.shape[0], px.shape[1]
    samples = px.reshape(h, -1)
    if depth == 16:
        samples = samples.astype(">u2").view(np.uint8).reshape(h, -1)
    else:
        samples = samples.astype(np.uint8)
    rows = np.concatenate([np.zeros((h, 1), np.uint8), samples], axis=1)  # filter type 0 per row
    out = _SIG + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, 0))
    out += _chunk(b"IDAT", zlib.compress(rows.tobytes(), 6)) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(out)


def _pixels(image, comps: int, dtype) -> np.ndarray:
    a = np.asarray(image.data if hasattr(image, "data") else image)
    if a.ndim != (2 if comps == 1 else 3):
        raise ValueError("a 2-D image is required")
    return a.astype(dtype, copy=False)


def write_gray8(image, path):
    """png.rs:74-79"""
    _encode(path, _pixels(image, 1, np.uint8), GRAY, 8)


def write_gray16(image, path):
    """png.rs:81-87"""
    _encode(path, _pixels(image, 1, np.uint16), GRAY, 16)


def write_rgb8(image, path):
    """png.rs:89-95"""
    _encode(path, _pixels(image, 3, np.uint8), RGB, 8)


def write_rgba8(image, path):
    """png.rs:97-103"""
    _encode(path, _pixels(image, 4, np.uint8), RGBA, 8)


def write_rgb16(image, path):
    """png.rs:105-115"""
    _encode(path, _pixels(image, 3, np.uint16), RGB, 16)


def write_rgba16(image, path):
    """png.rs:117-127"""
    _encode(path, _pixels(image, 4, np.uint16), RGBA, 16)
