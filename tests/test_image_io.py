"""Skybox image files (ptw_read_image_rgba / ptw_set_skybox_file): Radiance
RGBE and OpenEXR, the formats of the reference's skybox assets (the skybox
loader world.rs:1872-1957 decodes them with an image library).

The files are written here by small test-side encoders that follow the
published formats: RGBE scanlines (flat and run-length), and scanline OpenEXR
with NONE, RLE, ZIPS, ZIP and PIZ compression (PIZ: value bitmap, 2D wavelet
and the canonical Huffman code with its packed length table).  The decoder
must return the encoded values bit for bit."""
import ctypes as C
import heapq
import struct
import zlib

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi

CHANNEL_TYPE = {"uint": 0, "half": 1, "float": 2}
LINES = {0: 1, 1: 1, 2: 1, 3: 16, 4: 32}


# ------------------------------------------------------------------ RGBE
def rgbe_bytes(rng, h, w):
    """random RGBE pixels (mantissas >= 128 where the exponent is set, a few zero pixels)"""
    px = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
    px[..., 3] = rng.integers(110, 150, size=(h, w))
    px[rng.random((h, w)) < 0.05] = 0
    # make runs so that the run-length coder has something to do
    px[:, : w // 3, :] = px[:, :1, :]
    return px


def rgbe_decode(px):
    e = px[..., 3].astype(np.int32)
    scale = np.ldexp(np.float32(1.0), e - 136).astype(np.float32)
    rgb = px[..., :3].astype(np.float32) * scale[..., None]
    rgb[e == 0] = 0
    return np.concatenate([rgb, np.ones(px.shape[:2] + (1,), np.float32)], axis=-1)


def write_hdr(path, px, rle=True):
    h, w = px.shape[:2]
    out = bytearray(b"#?RADIANCE\n# written by the tests\nFORMAT=32-bit_rle_rgbe\n\n")
    out += f"-Y {h} +X {w}\n".encode()
    for y in range(h):
        if not rle:
            out += px[y].tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 0xFF])
        for c in range(4):
            row = px[y, :, c]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and row[x + run] == row[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, row[x]])
                    x += run
                    continue
                lit = 1
                while x + lit < w and lit < 128 and not (x + lit + 2 < w and row[x + lit] == row[x + lit + 1] == row[x + lit + 2]):
                    lit += 1
                out += bytes([lit]) + row[x : x + lit].tobytes()
                x += lit
    path.write_bytes(bytes(out))


# ------------------------------------------------------------------ OpenEXR
def _attr(name, type_, data):
    return name.encode() + b"\0" + type_.encode() + b"\0" + struct.pack("<i", len(data)) + data


def _rle_bytes(t):
    """OpenEXR run-length code: a negative count c copies -c literal bytes, c >= 0 repeats the next byte c+1 times"""
    out = bytearray()
    i, n = 0, len(t)
    while i < n:
        run = 1
        while i + run < n and run < 128 and t[i + run] == t[i]:
            run += 1
        if run >= 3:
            out += bytes([run - 1, t[i]])
            i += run
            continue
        j = i
        while j < n and j - i < 127 and not (j + 2 < n and t[j] == t[j + 1] == t[j + 2]):
            j += 1
        out += bytes([(-(j - i)) & 0xFF]) + bytes(t[i:j])
        i = j
    return bytes(out)


def _predict_split(raw):
    """ZIP / RLE preprocessing: even bytes then odd bytes, then byte deltas (+128)"""
    t = np.frombuffer(raw, np.uint8)
    s = np.concatenate([t[0::2], t[1::2]]).astype(np.int32)
    d = s.copy()
    d[1:] = (s[1:] - s[:-1] + 128) & 0xFF
    return d.astype(np.uint8).tobytes()


def _wenc14(a, b):
    a = a - 65536 if a >= 32768 else a
    b = b - 65536 if b >= 32768 else b
    return ((a + b) >> 1) & 0xFFFF, (a - b) & 0xFFFF


def _wenc16(a, b):
    ao = (a + 32768) & 0xFFFF
    m = (ao + b) >> 1
    d = ao - b
    if d < 0:
        m = (m + 32768) & 0xFFFF
    return m, d & 0xFFFF


def _wav2_encode(buf, base, nx, ox, ny, oy, mx):
    enc = _wenc14 if mx < (1 << 14) else _wenc16
    n = min(nx, ny)
    p, p2 = 1, 2
    while p2 <= n:
        py = base
        ey = base + oy * (ny - p2)
        oy1, oy2, ox1, ox2 = oy * p, oy * p2, ox * p, ox * p2
        while py <= ey:
            px = py
            ex = py + ox * (nx - p2)
            while px <= ex:
                p01, p10 = px + ox1, px + oy1
                p11 = p10 + ox1
                i00, i01 = enc(buf[px], buf[p01])
                i10, i11 = enc(buf[p10], buf[p11])
                buf[px], buf[p10] = enc(i00, i10)
                buf[p01], buf[p11] = enc(i01, i11)
                px += ox2
            if nx & p:
                p10 = px + oy1
                buf[px], buf[p10] = enc(buf[px], buf[p10])
            py += oy2
        if ny & p:
            px = py
            ex = py + ox * (nx - p2)
            while px <= ex:
                p01 = px + ox1
                buf[px], buf[p01] = enc(buf[px], buf[p01])
                px += ox2
        p, p2 = p2, p2 << 1


class _Bits:
    def __init__(self):
        self.out, self.acc, self.n = bytearray(), 0, 0
        self.total = 0

    def put(self, nbits, value):
        self.acc = (self.acc << nbits) | value
        self.n += nbits
        self.total += nbits
        while self.n >= 8:
            self.n -= 8
            self.out.append((self.acc >> self.n) & 0xFF)
        self.acc &= (1 << self.n) - 1

    def flush(self):
        if self.n:
            self.out.append((self.acc << (8 - self.n)) & 0xFF)
            self.acc = self.n = 0
        return bytes(self.out)


def _huffman_compress(words):
    freq = {}
    for w in words:
        freq[w] = freq.get(w, 0) + 1
    im, rlc = min(freq), max(freq) + 1
    freq[rlc] = 1  # the run-length pseudo symbol
    # code lengths of a Huffman tree
    heap = [(f, s, (s,)) for s, f in freq.items()]
    heapq.heapify(heap)
    length = {s: 0 for s in freq}
    while len(heap) > 1:
        f1, k1, s1 = heapq.heappop(heap)
        f2, k2, s2 = heapq.heappop(heap)
        for s in s1 + s2:
            length[s] += 1
        heapq.heappush(heap, (f1 + f2, min(k1, k2), s1 + s2))
    assert max(length.values()) <= 58
    # canonical codes: longer codes take the smaller values, symbols in increasing order
    count = [0] * 59
    for s in length:
        count[length[s]] += 1
    start, c = [0] * 59, 0
    for l in range(58, 0, -1):
        start[l], c = c, (c + count[l]) >> 1
    code = {}
    for s in sorted(length):
        code[s] = start[length[s]]
        start[length[s]] += 1
    # packed length table: 6 bits per symbol, zero runs as 59..62 (2..5) or 63 + 8 bits (6..261)
    t = _Bits()
    i = im
    while i <= rlc:
        l = length.get(i, 0)
        if l == 0:
            run = 1
            while i + run <= rlc and run < 261 and length.get(i + run, 0) == 0:
                run += 1
            if run >= 6:
                t.put(6, 63)
                t.put(8, run - 6)
                i += run
                continue
            if run >= 2:
                t.put(6, 59 + run - 2)
                i += run
                continue
        t.put(6, l)
        i += 1
    table = t.flush()
    d = _Bits()
    i = 0
    while i < len(words):
        s = words[i]
        run = 0
        while i + 1 + run < len(words) and words[i + 1 + run] == s and run < 255:
            run += 1
        if length[s] + length[rlc] + 8 < length[s] * run:
            d.put(length[s], code[s])
            d.put(length[rlc], code[rlc])
            d.put(8, run)
        else:
            for _ in range(run + 1):
                d.put(length[s], code[s])
        i += run + 1
    nbits = d.total
    data = d.flush()
    return struct.pack("<5i", im, rlc, len(table), nbits, 0) + table + data


def _piz_block(raw, channels, nx, ny):
    """channels: list of (name, kind); raw = the block's lines (channels interleaved per line)"""
    sizes = [1 if kind == "half" else 2 for _, kind in channels]
    words_line = np.frombuffer(raw, "<u2").reshape(ny, -1)
    planes, col = [], 0
    for sz in sizes:
        planes.append(words_line[:, col : col + nx * sz].reshape(-1))
        col += nx * sz
    words = np.concatenate(planes).astype(np.int64)
    bitmap = np.zeros(8192, np.uint8)
    np.bitwise_or.at(bitmap, words >> 3, (1 << (words & 7)).astype(np.uint8))
    bitmap[0] &= 0xFE
    nz = np.nonzero(bitmap)[0]
    mn, mx = (int(nz[0]), int(nz[-1])) if len(nz) else (8191, 0)
    present = np.zeros(65536, bool)
    present[0] = True
    present[np.nonzero(np.unpackbits(bitmap, bitorder="little"))[0]] = True
    lut = np.cumsum(present) - 1
    max_value = int(present.sum() - 1)
    buf = [int(v) for v in lut[words]]
    off = 0
    for sz in sizes:
        for j in range(sz):
            _wav2_encode(buf, off + j, nx, sz, ny, nx * sz, max_value)
        off += nx * ny * sz
    out = struct.pack("<HH", mn, mx)
    if mn <= mx:
        out += bitmap[mn : mx + 1].tobytes()
    huff = _huffman_compress(buf)
    return out + struct.pack("<i", len(huff)) + huff


def write_exr(path, planes, compression, origin=(0, 0), decreasing=False, raw_chunks=(), force=False):
    """planes: {name: array (h, w) of float16 / float32 / uint32}; channel order is alphabetical (as files store it).
    A block whose compressed form is not smaller is stored raw, as writers do, unless `force` (then only a
    compressed form of exactly the raw size, which a reader takes for raw data, is replaced).  Returns the
    number of blocks stored compressed."""
    names = sorted(planes)
    kinds = {n: {np.float16: "half", np.float32: "float", np.uint32: "uint"}[planes[n].dtype.type] for n in names}
    h, w = planes[names[0]].shape
    x0, y0 = origin
    chl = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", CHANNEL_TYPE[kinds[n]], 0, 1, 1) for n in names) + b"\0"
    win = struct.pack("<4i", x0, y0, x0 + w - 1, y0 + h - 1)
    header = (b"\x76\x2f\x31\x01" + struct.pack("<I", 2)
              + _attr("channels", "chlist", chl)
              + _attr("compression", "compression", bytes([compression]))
              + _attr("dataWindow", "box2i", win)
              + _attr("displayWindow", "box2i", win)
              + _attr("lineOrder", "lineOrder", bytes([1 if decreasing else 0]))
              + _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + _attr("screenWindowCenter", "v2f", struct.pack("<2f", 0, 0))
              + _attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
              + b"\0")
    lines = LINES[compression]
    chunks, compressed = [], 0
    for first in range(0, h, lines):
        ny = min(lines, h - first)
        raw = b"".join(planes[n][first + y].astype(planes[n].dtype.newbyteorder("<")).tobytes()
                       for y in range(ny) for n in names)
        k = first // lines
        if k in raw_chunks or compression == 0:
            packed = raw
        elif compression == 1:
            packed = _rle_bytes(_predict_split(raw))
        elif compression in (2, 3):
            packed = zlib.compress(_predict_split(raw), 9)
        else:
            packed = _piz_block(raw, [(n, kinds[n]) for n in names], w, ny)
        if len(packed) == len(raw) or (len(packed) > len(raw) and not force):
            packed = raw
        compressed += packed is not raw
        chunks.append(struct.pack("<ii", y0 + first, len(packed)) + packed)
    table_at = len(header)
    data_at = table_at + 8 * len(chunks)
    order = range(len(chunks) - 1, -1, -1) if decreasing else range(len(chunks))
    offsets, blob = [0] * len(chunks), bytearray()
    for k in order:
        offsets[k] = data_at + len(blob)
        blob += chunks[k]
    path.write_bytes(header + struct.pack(f"<{len(chunks)}Q", *offsets) + bytes(blob))
    return compressed


def expected_rgba(planes):
    h, w = next(iter(planes.values())).shape
    out = np.zeros((h, w, 4), np.float32)
    out[..., 3] = 1
    for i, n in enumerate("RGBA"):
        if n in planes:
            out[..., i] = planes[n].astype(np.float32)
    if "Y" in planes and not all(c in planes for c in "RGB"):
        out[..., :3] = planes["Y"].astype(np.float32)[..., None]
    return out


def random_planes(rng, h, w, kinds, noise=True):
    """sky-like planes: a smooth field plus a little noise (compressible, with many distinct values),
    a run of equal pixels, and a few pixels of arbitrary finite bits"""
    planes = {}
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    for k, (name, kind) in enumerate(kinds.items()):
        field = 2.0 + np.sin(x / (5.0 + k)) + np.cos(y / 7.0) * 0.5 + 0.02 * x
        if noise:
            field = field + rng.normal(0, 0.01, size=(h, w))
        if kind == "half":
            v = field.astype(np.float16)
            v[:, : w // 4] = v[:, :1]
            wild = rng.integers(0, 0x7C00, size=(h, w)).astype(np.uint16).view(np.float16)
            pick = rng.random((h, w)) < 0.01
            v[pick] = wild[pick]
            planes[name] = v
        elif kind == "float":
            v = (field * 10).astype(np.float32)
            bits = v.view(np.uint32) & np.uint32(0xFFFFFF00)  # low mantissa bits clear (sky-like data)
            pick = rng.random((h, w)) < 0.01
            bits[pick] = rng.integers(0, 0x7F800000, size=int(pick.sum()), dtype=np.uint32)
            planes[name] = bits.view(np.float32)
        else:
            planes[name] = (field * 1000).astype(np.uint32)
    return planes


def read(path):
    return pt.read_image(path)


# ------------------------------------------------------------------ tests
@pytest.mark.parametrize("rle", [True, False])
def test_hdr_round_trip(tmp_path, rle):
    rng = np.random.default_rng(3)
    px = rgbe_bytes(rng, 13, 40)
    write_hdr(tmp_path / "a.hdr", px, rle)
    got = read(tmp_path / "a.hdr")
    np.testing.assert_array_equal(got.view(np.uint32), rgbe_decode(px).view(np.uint32))


@pytest.mark.parametrize("compression", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("kinds", [
    {"R": "half", "G": "half", "B": "half", "A": "half"},
    {"R": "float", "G": "float", "B": "float"},
    {"R": "half", "G": "float", "B": "uint", "Z": "half"},
])
def test_exr_round_trip(tmp_path, compression, kinds):
    rng = np.random.default_rng(compression * 7 + len(kinds))
    planes = random_planes(rng, 45, 37, kinds)  # ragged blocks for every compression
    n = write_exr(tmp_path / "a.exr", planes, compression, origin=(3, -5), force=True)
    assert n == (0 if compression == 0 else -(-45 // LINES[compression]))  # every block goes through the decoder
    got = read(tmp_path / "a.exr")
    np.testing.assert_array_equal(got.view(np.uint32), expected_rgba(planes).view(np.uint32))


def test_exr_piz_wavelet_16bit(tmp_path):
    # more than 2^14 distinct 16-bit words in one block: the wavelet's 16-bit (modular) form
    i = np.arange(32 * 288, dtype=np.uint32).reshape(32, 288)
    planes = {"R": i * 5, "G": i * 7 + 1000, "B": (i * 3) ^ 0x5555}
    words = np.concatenate([p.view(np.uint16).ravel() for p in planes.values()])
    assert len(np.unique(words)) > (1 << 14)
    assert write_exr(tmp_path / "a.exr", planes, 4) == 1  # and the smooth ramps compress
    np.testing.assert_array_equal(read(tmp_path / "a.exr").view(np.uint32), expected_rgba(planes).view(np.uint32))


def test_exr_piz_sky_compresses(tmp_path):
    # a smooth sky-like image: PIZ pays off for every block, as in the reference's 4K skybox file
    rng = np.random.default_rng(12)
    ramp = np.linspace(0.5, 3.0, 256)[None, :] + rng.normal(0, 0.002, size=(64, 256))
    planes = {c: (ramp * (k + 1)).astype(np.float16) for k, c in enumerate("RGB")}
    assert write_exr(tmp_path / "a.exr", planes, 4) == 2
    np.testing.assert_array_equal(read(tmp_path / "a.exr").view(np.uint32), expected_rgba(planes).view(np.uint32))


def test_exr_piz_constant_and_zero(tmp_path):
    planes = {"R": np.zeros((40, 20), np.float16), "G": np.full((40, 20), 2.5, np.float16),
              "B": np.zeros((40, 20), np.float16)}
    write_exr(tmp_path / "a.exr", planes, 4, force=True)
    np.testing.assert_array_equal(read(tmp_path / "a.exr"), expected_rgba(planes))


def test_exr_decreasing_lines_and_stored_chunks(tmp_path):
    rng = np.random.default_rng(5)
    planes = random_planes(rng, 70, 33, {"R": "half", "G": "half", "B": "half"})
    write_exr(tmp_path / "a.exr", planes, 3, decreasing=True, raw_chunks=(1,))
    np.testing.assert_array_equal(read(tmp_path / "a.exr").view(np.uint32), expected_rgba(planes).view(np.uint32))


def test_exr_grey(tmp_path):
    rng = np.random.default_rng(9)
    planes = random_planes(rng, 8, 8, {"Y": "half"})
    write_exr(tmp_path / "a.exr", planes, 3)
    np.testing.assert_array_equal(read(tmp_path / "a.exr"), expected_rgba(planes))


@pytest.mark.parametrize("strategy", ["stored", "fixed", "dynamic"])
def test_zip_block_kinds(tmp_path, strategy):
    # the three DEFLATE block kinds, through a ZIP chunk written with each
    rng = np.random.default_rng(2)
    planes = random_planes(rng, 16, 24, {"R": "half", "G": "half", "B": "half"})
    names = sorted(planes)
    raw = b"".join(planes[n][y].tobytes() for y in range(16) for n in names)
    pre = _predict_split(raw)
    if strategy == "stored":
        packed = zlib.compress(pre, 0)
    else:
        co = zlib.compressobj(9, zlib.DEFLATED, 15, 9, zlib.Z_FIXED if strategy == "fixed" else zlib.Z_DEFAULT_STRATEGY)
        packed = co.compress(pre) + co.flush()
    write_exr(tmp_path / "a.exr", planes, 3)  # one 16-line block, replaced by the chosen stream
    body = _rewrite_single_chunk((tmp_path / "a.exr").read_bytes(), packed)
    (tmp_path / "b.exr").write_bytes(body)
    np.testing.assert_array_equal(read(tmp_path / "b.exr").view(np.uint32), expected_rgba(planes).view(np.uint32))


def _rewrite_single_chunk(data, packed):
    off = struct.unpack_from("<Q", data, _header_end(data))[0]
    y = struct.unpack_from("<i", data, off)[0]
    return data[:off] + struct.pack("<ii", y, len(packed)) + packed


def _header_end(data):
    pos = 8
    while data[pos] != 0:
        pos = data.index(b"\0", pos) + 1
        pos = data.index(b"\0", pos) + 1
        pos += 4 + struct.unpack_from("<i", data, pos)[0]
    return pos + 1


def _exr_bytes(tmp_path, **kw):
    rng = np.random.default_rng(1)
    planes = random_planes(rng, 40, 16, {"R": "half", "G": "half", "B": "half"})
    write_exr(tmp_path / "ok.exr", planes, kw.pop("compression", 4), force=True, **kw)
    return bytearray((tmp_path / "ok.exr").read_bytes())


def _expect_error(tmp_path, data, words):
    p = tmp_path / "bad.exr"
    p.write_bytes(bytes(data))
    with pytest.raises(pt.PathTracerError) as e:
        read(p)
    assert e.value.code == abi.PT_ERR_INVALID_ARG
    assert any(w in e.value.message for w in words), e.value.message


def test_bad_files_are_refused(tmp_path):
    good = _exr_bytes(tmp_path)
    _expect_error(tmp_path, good[:100], ["truncated", "out of range"])
    _expect_error(tmp_path, good[: len(good) - 50], ["out of range", "bad PIZ"])
    bad = bytearray(good)
    bad[5] |= 0x02  # tiled
    _expect_error(tmp_path, bad, ["single-part scanline"])
    bad = bytearray(good)
    at = bad.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    bad[at] = 5  # PXR24
    _expect_error(tmp_path, bad, ["unsupported compression"])
    # flip bytes inside the first chunk's coded data: refused or decoded, never a crash
    end = _header_end(good)
    off = struct.unpack_from("<Q", good, end)[0]
    for k in range(20):
        bad = bytearray(good)
        bad[off + 12 + 7 * k] ^= 0x5A
        (tmp_path / "flip.exr").write_bytes(bytes(bad))
        try:
            img = read(tmp_path / "flip.exr")
            assert img.shape == (40, 16, 4)
        except pt.PathTracerError as e:
            assert e.code == abi.PT_ERR_INVALID_ARG
    _expect_error(tmp_path, b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 2 +X 2\n", ["unsupported HDR format"])
    _expect_error(tmp_path, b"P6\n", ["not a Radiance"])
    with pytest.raises(pt.PathTracerError):
        read(tmp_path / "missing.exr")


def test_size_query_and_capacity(tmp_path):
    (tmp_path / "a.exr").write_bytes(bytes(_exr_bytes(tmp_path, compression=3)))
    lib = pt.load()
    w, h = C.c_uint32(), C.c_uint32()
    err = C.create_string_buffer(256)
    assert lib.ptw_read_image_rgba(str(tmp_path / "a.exr").encode(), None, 0, C.byref(w), C.byref(h), err, 256) == 0
    assert (w.value, h.value) == (16, 40)
    small = np.zeros(16 * 40 * 4 - 1, np.float32)
    rc = lib.ptw_read_image_rgba(str(tmp_path / "a.exr").encode(), small.ctypes.data, small.size,
                                 C.byref(w), C.byref(h), err, 256)
    assert rc == abi.PT_ERR_OUT_OF_LIMITS


def test_skybox_file_equals_pixels(tmp_path):
    rng = np.random.default_rng(4)
    planes = random_planes(rng, 32, 64, {"R": "half", "G": "half", "B": "half"})
    write_exr(tmp_path / "sky.exr", planes, 4, force=True)
    a, b = pt.World.cornell_box(), pt.World.cornell_box()
    a.set_skybox_file(tmp_path / "sky.exr")
    b.set_skybox_rgba(expected_rgba(planes))
    ua, ub = a.take_updates(), b.take_updates()
    sa, sb = ua.skybox.contents, ub.skybox.contents
    assert (sa.uniforms.width, sa.uniforms.height) == (sb.uniforms.width, sb.uniforms.height) == (64, 32)
    assert sa.uniforms.total_luminous_flux == sb.uniforms.total_luminous_flux
    n = 64 * 32 * 4
    np.testing.assert_array_equal(np.ctypeslib.as_array(sa.rgba, (n,)), np.ctypeslib.as_array(sb.rgba, (n,)))
    with pytest.raises(pt.PathTracerError):
        a.set_skybox_file(tmp_path / "missing.hdr")
    a.close()
    b.close()


def test_ldr_skybox_files(tmp_path):
    # PNG and JPEG skyboxes, as the reference's image library loads them: samples / max, grey replicated
    from test_texture_io import QUANT, _test_image, encode_jpeg, write_png
    rng = np.random.default_rng(7)
    rgb16 = rng.integers(0, 65536, size=(8, 16, 3))
    (tmp_path / "a.png").write_bytes(write_png(rgb16, 2, 16))
    got = read(tmp_path / "a.png")
    want = np.concatenate([(rgb16 / 65535.0).astype(np.float32), np.ones((8, 16, 1), np.float32)], -1)
    np.testing.assert_allclose(got, want, rtol=1e-6)
    grey_alpha = rng.integers(0, 256, size=(8, 16, 2))
    (tmp_path / "b.png").write_bytes(write_png(grey_alpha, 4, 8))
    got = read(tmp_path / "b.png")
    np.testing.assert_allclose(got[..., 0], grey_alpha[..., 0] / 255.0, rtol=1e-6)
    np.testing.assert_allclose(got[..., 2], grey_alpha[..., 0] / 255.0, rtol=1e-6)
    np.testing.assert_allclose(got[..., 3], grey_alpha[..., 1] / 255.0, rtol=1e-6)
    jpg, _ = encode_jpeg(_test_image(16, 32, 2), [(1, 1), (1, 1), (1, 1)], QUANT)
    (tmp_path / "c.jpg").write_bytes(jpg)
    got = read(tmp_path / "c.jpg")
    np.testing.assert_allclose(got[..., :3], pt.decode_texture(jpg)[..., :3] / 255.0, rtol=1e-6)
    w = pt.World.cornell_box()
    w.set_skybox_file(tmp_path / "c.jpg")  # and the world accepts it
    w.close()
