"""PNG I/O (itkg.png, the reference's src/io/png.rs): round trips of every
writer through its reader, the decoder against scanlines filtered and
interlaced here by hand, the png crate transformations the 8-bit readers
apply (16-bit high byte, low-bit-depth grey scaled to 0..255), and the
colour-type / bit-depth refusals."""
import struct
import zlib

import numpy as np
import pytest

itkg = pytest.importorskip("itkg")
from itkg import png  # noqa: E402


def _write_raw(path, w, h, depth, color, rows, interlace=0):
    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color, 0, 0, interlace))
    data += chunk(b"IDAT", zlib.compress(rows)) + chunk(b"IEND", b"")
    open(path, "wb").write(data)


def _filter(rows: np.ndarray, bpp: int, types) -> bytes:
    """Encode rows (h, row_bytes) uint8 with the given filter type per row."""
    out = bytearray()
    prev = np.zeros(rows.shape[1], np.int32)
    for y, ft in zip(range(rows.shape[0]), types):
        cur = rows[y].astype(np.int32)
        enc = np.zeros_like(cur)
        for i in range(len(cur)):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if ft == 0:
                p = 0
            elif ft == 1:
                p = a
            elif ft == 2:
                p = b
            elif ft == 3:
                p = (a + b) >> 1
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            enc[i] = (cur[i] - p) & 0xFF
        out.append(ft)
        out += bytes(enc.astype(np.uint8))
        prev = cur
    return bytes(out)


@pytest.mark.parametrize("name,shape,dtype", [("gray8", (7, 9), np.uint8), ("gray16", (5, 6), np.uint16),
                                              ("rgb8", (4, 5, 3), np.uint8), ("rgba8", (3, 4, 4), np.uint8),
                                              ("rgb16", (4, 3, 3), np.uint16), ("rgba16", (2, 5, 4), np.uint16)])
def test_round_trip(tmp_path, name, shape, dtype):
    rng = np.random.default_rng(3)
    a = rng.integers(0, np.iinfo(dtype).max + 1, shape).astype(dtype)
    p = tmp_path / f"{name}.png"
    getattr(png, f"write_{name}")(a, p)
    img = getattr(png, f"read_{name}")(p)
    assert img.region.index == (0, 0) and img.region.size == (shape[1], shape[0])
    assert img.spacing == (1.0, 1.0) and img.origin == (0.0, 0.0)
    assert img.data.dtype == dtype and np.array_equal(img.data, a)


def test_every_filter_type_and_adam7(tmp_path):
    rng = np.random.default_rng(5)
    a = rng.integers(0, 256, (11, 13, 3), dtype=np.uint8)
    rows = a.reshape(11, 13 * 3)
    p = tmp_path / "filters.png"
    _write_raw(p, 13, 11, 8, 2, _filter(rows, 3, [0, 1, 2, 3, 4, 4, 3, 2, 1, 0, 4]))
    assert np.array_equal(png.read_rgb8(p).data, a)
    # Adam7: each pass's sub-image filtered on its own
    g = rng.integers(0, 256, (10, 12), dtype=np.uint8)
    raw = b""
    for k, (x0, y0, dx, dy) in enumerate([(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4),
                                          (1, 0, 2, 2), (0, 1, 1, 2)]):
        sub = g[y0::dy, x0::dx]
        if sub.size:
            raw += _filter(sub, 1, [(k + y) % 5 for y in range(sub.shape[0])])
    p2 = tmp_path / "adam7.png"
    _write_raw(p2, 12, 10, 8, 0, raw, interlace=1)
    assert np.array_equal(png.read_gray8(p2).data, g)


def test_8bit_readers_transform(tmp_path):
    # 16-bit grey read as 8-bit keeps the high byte (STRIP_16)
    a = np.array([[0x1234, 0xFF00], [0x00FF, 0x8080]], np.uint16)
    p = tmp_path / "g16.png"
    png.write_gray16(a, p)
    assert np.array_equal(png.read_gray8(p).data, (a >> 8).astype(np.uint8))
    # 2-bit grey scaled to 0..255 (EXPAND)
    v = np.array([[0, 1, 2, 3, 3, 2, 1]], np.uint8)
    packed = np.packbits(np.unpackbits(v[:, :, None], axis=2)[:, :, 6:].reshape(1, -1), axis=1)
    p2 = tmp_path / "g2.png"
    _write_raw(p2, 7, 1, 2, 0, b"\x00" + packed.tobytes())
    assert list(png.read_gray8(p2).data[0]) == [0, 85, 170, 255, 255, 170, 85]


def test_refusals(tmp_path):
    p = tmp_path / "rgb.png"
    png.write_rgb8(np.zeros((2, 2, 3), np.uint8), p)
    with pytest.raises(png.PngError, match="color type mismatch"):
        png.read_gray8(p)
    p8 = tmp_path / "g8.png"
    png.write_gray8(np.zeros((2, 2), np.uint8), p8)
    with pytest.raises(png.PngError, match="16-bit"):
        png.read_gray16(p8)
    data = bytearray(open(p8, "rb").read())
    data[20] ^= 0xFF  # inside IHDR
    bad = tmp_path / "bad.png"
    open(bad, "wb").write(bytes(data))
    with pytest.raises(png.PngError, match="CRC"):
        png.read_gray8(bad)
