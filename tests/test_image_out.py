"""Output images of the headless renderer (ptw_write_image): PNG (checked
with Python's own zlib and a plain unfilter), baseline JPEG (decoded back,
PSNR and stream structure), lossless WebP (decoded by a small VP8L reader
written here from the format description) and PPM; code-length limits are
exercised with skewed value distributions."""
import struct
import zlib

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi


def smooth_image(h, w, seed=1):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    img = np.stack([128 + 100 * np.sin(x / 17 + c) * np.cos(y / 23 - c) for c in range(3)], -1)
    return np.clip(img + rng.normal(0, 4, img.shape), 0, 255).astype(np.uint8)


def skewed_image(h, w):
    """red values with Fibonacci-like frequencies (an unlimited Huffman code would be deeper than 16)"""
    vals, fib = [], [1, 1]
    while len(fib) < 26:
        fib.append(fib[-1] + fib[-2])
    for v, f in enumerate(fib):
        vals += [v] * f
    vals = np.array(vals[: h * w] + [0] * max(0, h * w - len(vals)), np.uint8)
    img = np.zeros((h, w, 3), np.uint8)
    img[..., 0] = np.random.default_rng(3).permutation(vals)[: h * w].reshape(h, w)
    img[..., 1] = 7
    img[..., 2] = np.arange(h * w, dtype=np.uint32).reshape(h, w) % 3
    return img


# ------------------------------------------------------------------ PNG
def png_pixels(data):
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, ihdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert zlib.crc32(kind + body) & 0xFFFFFFFF == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype = ihdr[:4]
    assert (depth, ctype) == (8, 2)
    raw = zlib.decompress(idat)  # an independent inflater
    out = np.zeros((h, w * 3), np.int32)
    prev = np.zeros(w * 3, np.int32)
    for y in range(h):
        f, row = raw[y * (w * 3 + 1)], np.frombuffer(raw, np.uint8, w * 3, y * (w * 3 + 1) + 1).astype(np.int32)
        cur = np.zeros(w * 3, np.int32)
        for i in range(w * 3):
            a = cur[i - 3] if i >= 3 else 0
            b = prev[i]
            c = prev[i - 3] if i >= 3 else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) >> 1
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            cur[i] = (row[i] + p) & 0xFF
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 3).astype(np.uint8)


@pytest.mark.parametrize("shape", [(1, 1), (9, 17), (64, 96)])
def test_png(tmp_path, shape):
    img = smooth_image(*shape)
    pt.write_image(tmp_path / "a.png", img)
    data = (tmp_path / "a.png").read_bytes()
    np.testing.assert_array_equal(png_pixels(data), img)
    np.testing.assert_array_equal(pt.decode_texture(data)[..., :3], img)


def test_png_compresses_repetition(tmp_path):
    img = np.zeros((200, 300, 3), np.uint8)
    img[:, :, 0] = np.arange(300, dtype=np.uint32) % 256
    pt.write_image(tmp_path / "a.png", img)
    data = (tmp_path / "a.png").read_bytes()
    assert len(data) < img.size // 20
    np.testing.assert_array_equal(png_pixels(data), img)


# ------------------------------------------------------------------ JPEG
def jpeg_markers(data):
    pos, out = 2, []
    assert data[:2] == b"\xff\xd8"
    while pos < len(data):
        assert data[pos] == 0xFF
        m = data[pos + 1]
        if m == 0xD9:
            out.append(m)
            break
        n = struct.unpack(">H", data[pos + 2:pos + 4])[0]
        out.append(m)
        if m == 0xDA:  # skip the entropy-coded data
            pos += 2 + n
            while not (data[pos] == 0xFF and data[pos + 1] not in (0x00,)):
                pos += 1
            continue
        if m == 0xC4:  # every Huffman table: at most 16-bit codes, no all-ones code
            counts = list(data[pos + 5:pos + 21])
            assert sum(c * 2.0 ** -(l + 1) for l, c in enumerate(counts)) < 1.0
        pos += 2 + n
    return out


@pytest.mark.parametrize("shape", [(1, 1), (9, 17), (120, 200)])
def test_jpeg(tmp_path, shape):
    img = smooth_image(*shape)
    pt.write_image(tmp_path / "a.jpg", img)
    data = (tmp_path / "a.jpg").read_bytes()
    markers = jpeg_markers(data)
    assert markers[0] == 0xE0 and 0xC0 in markers and markers.count(0xC4) == 4 and markers[-1] == 0xD9
    got = pt.decode_texture(data)[..., :3].astype(np.float64)
    assert got.shape == img.shape
    if shape[0] > 8:
        mse = np.mean((got - img) ** 2)
        assert 10 * np.log10(255.0 ** 2 / mse) > 30.0


def test_jpeg_code_lengths_limited(tmp_path):
    img = skewed_image(256, 512)
    pt.write_image(tmp_path / "a.jpeg", img)
    data = (tmp_path / "a.jpeg").read_bytes()
    jpeg_markers(data)
    assert pt.decode_texture(data).shape == (256, 512, 4)


# ------------------------------------------------------------------ WebP (VP8L reader)
class _Bits:
    def __init__(self, data):
        self.v = int.from_bytes(data, "little")
        self.pos = 0

    def read(self, n):
        r = (self.v >> self.pos) & ((1 << n) - 1)
        self.pos += n
        return r


class _Code:
    def __init__(self, lengths):
        self.single = None
        used = [(l, s) for s, l in enumerate(lengths) if l]
        assert used
        if len(used) == 1:
            self.single = used[0][1]
            return
        assert sum(2.0 ** -l for l, _ in used) == 1.0  # complete
        self.table, code, prev_len = {}, 0, 0
        for l, s in sorted(used):
            code <<= l - prev_len
            prev_len = l
            self.table[(l, code)] = s
            code += 1

    def decode(self, br):
        if self.single is not None:
            return self.single
        code, l = 0, 0
        while True:
            code = (code << 1) | br.read(1)
            l += 1
            if (l, code) in self.table:
                return self.table[(l, code)]
            assert l <= 15


def _read_code(br, size):
    if br.read(1):
        n = br.read(1) + 1
        s0 = br.read(8 if br.read(1) else 1)
        lengths = [0] * size
        lengths[s0] = 1
        if n == 2:
            lengths[br.read(8)] = 1
        else:
            return _Code([1 if s == s0 else 0 for s in range(size)])
        return _Code(lengths)
    order = [17, 18, 0, 1, 2, 3, 4, 5, 16, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15]
    cl = [0] * 19
    for i in range(br.read(4) + 4):
        cl[order[i]] = br.read(3)
    max_symbol = size
    if br.read(1):
        max_symbol = 2 + br.read(2 + 2 * br.read(3))
    clc = _Code(cl)
    lengths, prev = [], 8
    while len(lengths) < size and max_symbol > 0:
        max_symbol -= 1
        s = clc.decode(br)
        if s < 16:
            lengths.append(s)
            if s:
                prev = s
        elif s == 16:
            lengths += [prev] * (3 + br.read(2))
        elif s == 17:
            lengths += [0] * (3 + br.read(3))
        else:
            lengths += [0] * (11 + br.read(7))
    return _Code(lengths + [0] * (size - len(lengths)))


def webp_pixels(data):
    assert data[:4] == b"RIFF" and data[8:16] == b"WEBPVP8L"
    assert struct.unpack("<I", data[4:8])[0] == len(data) - 8
    n = struct.unpack("<I", data[16:20])[0]
    br = _Bits(data[20:20 + n])
    assert br.read(8) == 0x2F
    w, h = br.read(14) + 1, br.read(14) + 1
    br.read(1)
    assert br.read(3) == 0
    assert br.read(1) == 0 and br.read(1) == 0 and br.read(1) == 0  # no transform, cache or meta codes
    codes = [_read_code(br, s) for s in (280, 256, 256, 256, 40)]
    out = np.zeros((h * w, 3), np.uint8)
    for i in range(h * w):
        g = codes[0].decode(br)
        assert g < 256
        r, b = codes[1].decode(br), codes[2].decode(br)
        assert codes[3].decode(br) == 255
        out[i] = (r, g, b)
    return out.reshape(h, w, 3)


@pytest.mark.parametrize("kind", ["smooth", "flat", "skewed"])
def test_webp_lossless(tmp_path, kind):
    img = {"smooth": lambda: smooth_image(23, 31), "flat": lambda: np.full((5, 7, 3), 200, np.uint8),
           "skewed": lambda: skewed_image(128, 256)}[kind]()
    pt.write_image(tmp_path / "a.webp", img)
    np.testing.assert_array_equal(webp_pixels((tmp_path / "a.webp").read_bytes()), img)


def test_ppm_and_errors(tmp_path):
    img = smooth_image(3, 4)
    pt.write_image(tmp_path / "a.ppm", img)
    assert (tmp_path / "a.ppm").read_bytes() == b"P6\n4 3\n255\n" + img.tobytes()
    for bad in ["a.bmp", "noext"]:
        with pytest.raises(pt.PathTracerError) as e:
            pt.write_image(tmp_path / bad, img)
        assert e.value.code == abi.PT_ERR_INVALID_ARG
    with pytest.raises(pt.PathTracerError):
        pt.write_image(tmp_path / "missing" / "a.png", img)
