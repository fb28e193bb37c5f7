"""glTF texture images (ptw_decode_texture_rgba8): PNG and Huffman JPEG, the
encodings the reference's glTF importer accepts (it decodes them with an
image library and converts the decoded formats to RGBA8, world.rs:949-1011).

PNG files are written here by a test-side encoder (all colour types and bit
depths, every filter type, Adam7 interlacing, palettes and tRNS) and must
decode bit for bit.  JPEG files are written by a test-side encoder
(baseline and progressive with spectral selection and successive
approximation, restart intervals, 4:4:4 / 4:2:2 / 4:2:0 / 3:1 sampling,
per-scan Huffman tables built from the symbol counts); the expected pixels
are computed here from the same quantised coefficients (inverse DCT, the
triangle upsampling filter, JFIF colour conversion), so the decoder must
match within one level of rounding."""
import heapq
import struct
import zlib

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi


# ------------------------------------------------------------------ PNG writer
def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _filter_row(f, row, prev, bpp):
    out = bytearray(len(row))
    for i, v in enumerate(row):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
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
        out[i] = (v - p) & 0xFF
    return bytes(out)


def _pack_row(samples, depth):
    """samples: 1-D int array of one row's samples -> bytes"""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    per = 8 // depth
    out = bytearray((len(samples) + per - 1) // per)
    for i, s in enumerate(samples):
        out[i // per] |= int(s) << (8 - depth * (i % per + 1))
    return bytes(out)


ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def write_png(samples, ctype, depth, palette=None, trns=None, interlace=False):
    """samples: (h, w, channels) integer array in the file's sample layout (palette indices for ctype 3)"""
    h, w, ch = samples.shape
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    k = 0
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        rb = (sub.shape[1] * ch * depth + 7) // 8
        prev = bytes(rb)
        for row in sub:
            packed = _pack_row(row.reshape(-1), depth)
            f = k % 5
            k += 1
            raw += bytes([f]) + _filter_row(f, packed, prev, bpp)
            prev = packed
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        out += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        out += _chunk(b"tRNS", bytes(trns))
    out += _chunk(b"tEXt", b"Comment\0written by the tests")  # an ancillary chunk to skip
    z = zlib.compress(bytes(raw), 6)
    out += _chunk(b"IDAT", z[: len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:]) + _chunk(b"IEND", b"")
    return out


def expected_from_png(samples, ctype, depth, palette=None, trns=None):
    """what the importer's RGBA8 conversion gives for the decoded PNG"""
    s = samples.astype(np.int64)
    h, w, _ = s.shape
    if ctype == 3:
        pal = np.asarray(palette, np.int64).reshape(-1, 3)
        rgb = pal[s[..., 0]]
        out = np.concatenate([rgb, np.full((h, w, 1), 255)], axis=-1)
        if trns is not None:
            t = np.full(len(pal), 255)
            t[: len(trns)] = list(trns)
            out[..., 3] = t[s[..., 0]]
        return out.astype(np.uint8)
    if depth < 8:
        s8 = s * (255 // ((1 << depth) - 1))
    elif depth == 16:
        s8 = s >> 8
    else:
        s8 = s
    alpha = None
    if trns is not None:
        key = [int.from_bytes(bytes(trns[i:i + 2]), "big") for i in range(0, len(trns), 2)]
        match = np.all(s[..., : len(key)] == np.array(key), axis=-1)
        alpha = np.where(match, 0, 255)
    chans = s8.shape[-1] + (1 if alpha is not None else 0)
    if alpha is not None:
        s8 = np.concatenate([s8, alpha[..., None]], axis=-1)
    out = np.zeros((h, w, 4), np.int64)
    if chans == 1:
        out[..., :3] = s8[..., :1]
        out[..., 3] = 255
    elif chans == 2:
        out[..., 0], out[..., 1], out[..., 3] = s8[..., 0], s8[..., 1], 255
    elif chans == 3:
        out[..., :3] = s8
        out[..., 3] = 255
    else:
        out[...] = s8
    return out.astype(np.uint8)


PNG_CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
             (4, 8), (4, 16), (6, 8), (6, 16)]


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("ctype,depth", PNG_CASES)
def test_png_round_trip(ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 31 + depth + 7 * interlace)
    h, w = 13, 19
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = (1 << depth) - 1
    palette = None
    if ctype == 3:
        n = min(1 << depth, 200)
        palette = rng.integers(0, 256, size=(n, 3))
        samples = rng.integers(0, n, size=(h, w, 1))
    else:
        samples = rng.integers(0, top + 1, size=(h, w, ch))
        samples[:, :5] = samples[:, :1]  # runs for the filters
    data = write_png(samples, ctype, depth, palette, interlace=interlace)
    got = pt.decode_texture(data)
    np.testing.assert_array_equal(got, expected_from_png(samples, ctype, depth, palette))


@pytest.mark.parametrize("ctype,depth", [(0, 8), (0, 16), (0, 2), (2, 8), (2, 16), (3, 4)])
def test_png_transparency_chunk(ctype, depth):
    rng = np.random.default_rng(depth)
    h, w = 9, 11
    palette = None
    if ctype == 3:
        palette = rng.integers(0, 256, size=(16, 3))
        samples = rng.integers(0, 16, size=(h, w, 1))
        trns = bytes(rng.integers(0, 256, size=10).astype(np.uint8))  # shorter than the palette
    else:
        ch = 1 if ctype == 0 else 3
        samples = rng.integers(0, 4, size=(h, w, ch))  # few values, so the key colour occurs
        key = samples[0, 0]
        trns = b"".join(int(v).to_bytes(2, "big") for v in key)
    data = write_png(samples, ctype, depth, palette, trns)
    np.testing.assert_array_equal(pt.decode_texture(data), expected_from_png(samples, ctype, depth, palette, trns))


def test_png_errors():
    rng = np.random.default_rng(0)
    good = write_png(rng.integers(0, 256, size=(8, 8, 3)), 2, 8)
    for bad, words in [
        (good[:40], ["image data", "CRC", "past the end"]),
        (good[:20] + bytes([good[20] ^ 1]) + good[21:], ["CRC"]),
        (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 8, 8, 3, 2, 0, 0, 0)), ["bit depth"]),
        (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 9000, 8, 8, 2, 0, 0, 0)), ["larger"]),
        (b"GIF89a", ["unsupported image encoding"]),
    ]:
        with pytest.raises(pt.PathTracerError) as e:
            pt.decode_texture(bad)
        assert e.value.code == abi.PT_ERR_INVALID_ARG
        assert any(wd in e.value.message for wd in words), e.value.message


# ------------------------------------------------------------------ JPEG writer
NATURAL = [0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7,
           14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46,
           53, 60, 61, 54, 47, 55, 62, 63]
_K = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * np.cos((2 * x + 1) * u * np.pi / 16) / 2 for u in range(8)]
               for x in range(8)])


def fdct(block):
    return _K.T @ block @ _K  # F[v][u]


def idct(F):
    return _K @ F @ _K.T


def _category(v):
    return int(abs(int(v))).bit_length()


def _bits_of(v, n):
    v = int(v)
    return (v if v >= 0 else v + (1 << n) - 1) & ((1 << n) - 1)


def _huff_lengths(freq):
    items = [(f, s) for s, f in freq.items()]
    if len(items) == 1:
        return {items[0][1]: 1}
    heap = [(f, i, (s,)) for i, (f, s) in enumerate(items)]
    heapq.heapify(heap)
    length = {s: 0 for _, s in items}
    k = len(heap)
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            length[s] += 1
        heapq.heappush(heap, (f1 + f2, k, a + b))
        k += 1
    assert max(length.values()) <= 16
    return length


def _canonical(length):
    counts = [0] * 17
    for s in length.values():
        counts[s] += 1
    order = sorted(length, key=lambda s: (length[s], s))
    code, codes, prev_len = 0, {}, 0
    for s in order:
        code <<= length[s] - prev_len
        prev_len = length[s]
        codes[s] = (code, length[s])
        code += 1
    return counts[1:], order, codes


class _JBits:
    def __init__(self):
        self.out, self.acc, self.n = bytearray(), 0, 0

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def pad(self):
        while self.n:
            self.put(1, 1)


def _emit_scan(events, table_ids):
    """events: ('dc'|'ac', component, symbol, bits, nbits), ('raw', bits, nbits) or ('rst', n);
    returns DHT segments (built from the counts) + the entropy-coded data"""
    freq = {}
    for e in events:
        if e[0] in ("dc", "ac"):
            key = (e[0], table_ids[e[0]][e[1]])
            freq.setdefault(key, {})
            freq[key][e[2]] = freq[key].get(e[2], 0) + 1
    dht, codes = b"", {}
    for (kind, tid), f in sorted(freq.items()):
        counts, order, c = _canonical(_huff_lengths(f))
        codes[(kind, tid)] = c
        body = bytes([(0 if kind == "dc" else 1) << 4 | tid]) + bytes(counts) + bytes(order)
        dht += b"\xff\xc4" + struct.pack(">H", len(body) + 2) + body
    bits = _JBits()
    for e in events:
        if e[0] in ("dc", "ac"):
            code, n = codes[(e[0], table_ids[e[0]][e[1]])][e[2]]
            bits.put(code, n)
            if e[4]:
                bits.put(e[3], e[4])
        elif e[0] == "raw":
            bits.put(e[1], e[2])
        else:
            bits.pad()
            bits.out += bytes([0xFF, 0xD0 + e[1] % 8])
    bits.pad()
    return dht, bytes(bits.out)


def encode_jpeg(rgb, sampling, quality_q, progressive=False, restart=0, grey=False, adobe=None):
    """rgb: (h, w, 3) or (h, w) uint8. sampling: [(h, v)] per component.  Returns (file bytes, coefficient
    planes {component: (bh, bw, 64) int array of quantised coefficients, natural order}, quant tables)"""
    img = rgb.astype(np.float64)
    if grey:
        planes = [img]
    else:
        r, g, b = img[..., 0], img[..., 1], img[..., 2]
        planes = [0.299 * r + 0.587 * g + 0.114 * b,
                  -0.168736 * r - 0.331264 * g + 0.5 * b + 128,
                  0.5 * r - 0.418688 * g - 0.081312 * b + 128]
        if adobe == 0:
            planes = [r, g, b]
    H, W = img.shape[:2]
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    comps = []
    for ci, (plane, (hs, vs)) in enumerate(zip(planes, sampling)):
        cw, ch = -(-W * hs // hmax), -(-H * vs // vmax)
        # subsample by averaging, then pad the plane to whole MCUs by edge replication
        fy, fx = vmax // vs, hmax // hs
        ph, pw = ch * fy, cw * fx
        p = np.pad(plane, ((0, max(0, ph - H)), (0, max(0, pw - W))), mode="edge")[:ph, :pw]
        sub = p.reshape(ch, fy, cw, fx).mean(axis=(1, 3))
        bw, bh = mcux * hs, mcuy * vs
        full = np.pad(sub, ((0, bh * 8 - ch), (0, bw * 8 - cw)), mode="edge")
        q = quality_q[0 if ci == 0 else 1]
        coef = np.zeros((bh, bw, 64), np.int64)
        for by in range(bh):
            for bx in range(bw):
                F = fdct(full[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0).reshape(64)
                coef[by, bx] = np.round(F / q)
        comps.append(dict(id=ci + 1, h=hs, v=vs, tq=0 if ci == 0 else 1, coef=coef, cw=cw, ch=ch, bw=bw, bh=bh))
    out = bytearray(b"\xff\xd8")
    if adobe is not None:
        body = b"Adobe" + struct.pack(">HHHB", 100, 0, 0, adobe)
        out += b"\xff\xee" + struct.pack(">H", len(body) + 2) + body
    for tq, q in enumerate(quality_q[: 1 if grey else 2]):
        body = bytes([tq]) + bytes(int(q[NATURAL[k]]) for k in range(64))
        out += b"\xff\xdb" + struct.pack(">H", len(body) + 2) + body
    body = struct.pack(">BHHB", 8, H, W, len(comps))
    for c in comps:
        body += bytes([c["id"], c["h"] << 4 | c["v"], c["tq"]])
    out += (b"\xff\xc2" if progressive else b"\xff\xc0") + struct.pack(">H", len(body) + 2) + body
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    table_ids = {"dc": {c["id"]: (0 if c["id"] == 1 else 1) for c in comps},
                 "ac": {c["id"]: (0 if c["id"] == 1 else 1) for c in comps}}

    def blocks_of_scan(scomps):
        if len(scomps) == 1:
            c = scomps[0]
            for by in range(-(-c["ch"] // 8)):
                for bx in range(-(-c["cw"] // 8)):
                    yield [(c, by, bx)]
        else:
            for my in range(mcuy):
                for mx in range(mcux):
                    yield [(c, my * c["v"] + v, mx * c["h"] + h) for c in scomps for v in range(c["v"])
                           for h in range(c["h"])]

    def scan(scomps, ss, se, ah, al):
        events, pred, eob = [], {}, [0, []]  # EOB run length and its buffered correction bits

        def flush_eob(cid):
            if eob[0]:
                n = eob[0].bit_length() - 1
                events.append(("ac", cid, n << 4, eob[0] & ((1 << n) - 1), n))
                for b in eob[1]:
                    events.append(("raw", b, 1))
                eob[0], eob[1] = 0, []

        for mcu, blocks in enumerate(blocks_of_scan(scomps)):
            if restart and mcu and mcu % restart == 0:
                flush_eob(scomps[0]["id"])
                events.append(("rst", mcu // restart - 1))
                pred = {}
            for c, by, bx in blocks:
                cf = c["coef"][by, bx]
                cid = c["id"]
                if ss == 0:
                    if ah == 0:
                        v = int(cf[0]) >> al
                        d = v - pred.get(cid, 0)
                        pred[cid] = v
                        n = _category(d)
                        events.append(("dc", cid, n, _bits_of(d, n), n))
                    else:
                        events.append(("raw", (int(cf[0]) >> al) & 1, 1))
                    if not progressive:
                        r = 0
                        for k in range(1, 64):
                            v = int(cf[NATURAL[k]])
                            if v == 0:
                                r += 1
                                continue
                            while r > 15:
                                events.append(("ac", cid, 0xF0, 0, 0))
                                r -= 16
                            n = _category(v)
                            events.append(("ac", cid, (r << 4) | n, _bits_of(v, n), n))
                            r = 0
                        if r:
                            events.append(("ac", cid, 0x00, 0, 0))
                elif ah == 0:
                    r = 0
                    for k in range(ss, se + 1):
                        v = int(cf[NATURAL[k]])
                        mag = abs(v) >> al
                        if mag == 0:
                            r += 1
                            continue
                        flush_eob(cid)
                        while r > 15:
                            events.append(("ac", cid, 0xF0, 0, 0))
                            r -= 16
                        n = mag.bit_length()
                        events.append(("ac", cid, (r << 4) | n, _bits_of(mag if v > 0 else -mag, n), n))
                        r = 0
                    if r:
                        eob[0] += 1
                        if eob[0] == 0x7FFF:
                            flush_eob(cid)
                else:
                    absv = [abs(int(cf[NATURAL[k]])) >> al for k in range(64)]
                    last_new = max([k for k in range(ss, se + 1) if absv[k] == 1], default=-1)
                    r, buf = 0, []
                    for k in range(ss, se + 1):
                        t = absv[k]
                        if t == 0:
                            r += 1
                            continue
                        while r > 15 and k <= last_new:
                            flush_eob(cid)
                            events.append(("ac", cid, 0xF0, 0, 0))
                            r -= 16
                            events.extend(("raw", b, 1) for b in buf)
                            buf = []
                        if t > 1:
                            buf.append(t & 1)
                            continue
                        flush_eob(cid)
                        events.append(("ac", cid, (r << 4) | 1, 1 if cf[NATURAL[k]] > 0 else 0, 1))
                        events.extend(("raw", b, 1) for b in buf)
                        buf, r = [], 0
                    if r or buf:
                        eob[0] += 1
                        eob[1].extend(buf)
                        if eob[0] == 0x7FFF:
                            flush_eob(cid)
        flush_eob(scomps[0]["id"])
        dht, data = _emit_scan(events, table_ids)
        body = bytes([len(scomps)]) + b"".join(bytes([c["id"], table_ids["dc"][c["id"]] << 4 | table_ids["ac"][c["id"]]])
                                               for c in scomps) + bytes([ss, se, ah << 4 | al])
        return dht + b"\xff\xda" + struct.pack(">H", len(body) + 2) + body + data

    if not progressive:
        out += scan(comps, 0, 63, 0, 0)
    else:
        out += scan(comps, 0, 0, 0, 1)            # DC, all but the lowest bit
        for c in comps:
            out += scan([c], 1, 5, 0, 2)          # low AC band, two bits held back
        for c in comps:
            out += scan([c], 6, 63, 0, 1)         # high AC band, one bit held back
        out += scan(comps, 0, 0, 1, 0)            # DC refinement
        for c in comps:
            out += scan([c], 1, 5, 2, 1)          # low band refinements
            out += scan([c], 1, 5, 1, 0)
            out += scan([c], 6, 63, 1, 0)         # high band refinement
    out += b"\xff\xd9"
    return bytes(out), comps


def expected_from_jpeg(comps, H, W, quality_q, grey=False, adobe=None):
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    full = []
    for ci, c in enumerate(comps):
        q = quality_q[0 if ci == 0 else 1].reshape(64)
        bh, bw = c["bh"], c["bw"]
        plane = np.zeros((bh * 8, bw * 8))
        for by in range(bh):
            for bx in range(bw):
                plane[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = idct((c["coef"][by, bx] * q).reshape(8, 8))
        plane = np.clip(np.floor(plane + 128 + 0.5), 0, 255).astype(np.int64)
        cw, ch = c["cw"], c["ch"]
        if c["h"] == hmax and c["v"] == vmax:
            up = plane[:H, :W]
        elif hmax == 2 * c["h"] and vmax in (c["v"], 2 * c["v"]) and cw >= 2:
            up = np.zeros((H, 2 * cw), np.int64)
            for y in range(H):
                if vmax == c["v"]:
                    r = plane[y, :cw]
                    row = np.zeros(2 * cw, np.int64)
                    row[0], row[1] = r[0], (r[0] * 3 + r[1] + 2) >> 2
                    row[2:-2:2] = (r[1:-1] * 3 + r[:-2] + 1) >> 2
                    row[3:-2:2] = (r[1:-1] * 3 + r[2:] + 2) >> 2
                    row[-2], row[-1] = (r[-1] * 3 + r[-2] + 1) >> 2, r[-1]
                else:
                    yc = y // 2
                    yo = min(yc + 1, ch - 1) if y & 1 else max(yc - 1, 0)
                    s = plane[yc, :cw] * 3 + plane[yo, :cw]
                    row = np.zeros(2 * cw, np.int64)
                    row[0], row[1] = (s[0] * 4 + 8) >> 4, (s[0] * 3 + s[1] + 7) >> 4
                    row[2:-2:2] = (s[1:-1] * 3 + s[:-2] + 8) >> 4
                    row[3:-2:2] = (s[1:-1] * 3 + s[2:] + 7) >> 4
                    row[-2], row[-1] = (s[-1] * 3 + s[-2] + 8) >> 4, (s[-1] * 4 + 7) >> 4
                up[y] = row
            up = up[:, :W]
        else:
            ys = (np.arange(H) * c["v"]) // vmax
            xs = (np.arange(W) * c["h"]) // hmax
            up = plane[ys][:, xs]
        full.append(up.astype(np.float64))
    out = np.zeros((H, W, 4), np.int64)
    out[..., 3] = 255
    if grey:
        out[..., :3] = full[0][..., None]
        return out
    if adobe == 0:
        out[..., 0], out[..., 1], out[..., 2] = full
        return out
    y, cb, cr = full[0], full[1] - 128, full[2] - 128
    conv = [y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb]
    for i in range(3):
        out[..., i] = np.clip(np.floor(conv[i] + 0.5), 0, 255)
    return out


def _test_image(h, w, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    img = np.stack([128 + 100 * np.sin(x / 5.0 + c) * np.cos(y / 7.0 - c) for c in range(3)], axis=-1)
    img += rng.normal(0, 12, size=img.shape)
    img[h // 3: h // 3 + 4, :, :] = [250, 10, 30]  # a sharp band: large AC coefficients
    return np.clip(img, 0, 255).astype(np.uint8)


QUANT = (np.array([[1 + (u + v) * 2 for u in range(8)] for v in range(8)], np.float64).reshape(64),
         np.array([[2 + (u + v) * 3 for u in range(8)] for v in range(8)], np.float64).reshape(64))


def _check_jpeg(data, comps, h, w, **kw):
    got = pt.decode_texture(data).astype(np.int64)
    want = expected_from_jpeg(comps, h, w, QUANT, **kw)
    assert got.shape == want.shape
    diff = np.abs(got - want)
    assert diff.max() <= 1, (diff.max(), np.argwhere(diff > 1)[:5])
    assert (diff == 0).mean() > 0.99


@pytest.mark.parametrize("progressive", [False, True])
@pytest.mark.parametrize("sampling", [[(1, 1), (1, 1), (1, 1)], [(2, 1), (1, 1), (1, 1)], [(2, 2), (1, 1), (1, 1)],
                                      [(3, 1), (1, 1), (1, 1)], [(1, 2), (1, 1), (1, 1)]])
def test_jpeg_colour(progressive, sampling):
    h, w = 37, 45  # ragged MCUs in both directions
    img = _test_image(h, w, len(sampling) + progressive)
    data, comps = encode_jpeg(img, sampling, QUANT, progressive=progressive)
    _check_jpeg(data, comps, h, w)
    # and the decoded image is close to the source (a sanity check of the encoder itself)
    got = pt.decode_texture(data)[..., :3].astype(np.float64)
    assert np.abs(got - img).mean() < 12


@pytest.mark.parametrize("progressive", [False, True])
def test_jpeg_grey_and_restarts(progressive):
    h, w = 30, 50
    img = _test_image(h, w, 3)[..., 1]
    data, comps = encode_jpeg(img, [(1, 1)], QUANT, progressive=progressive, restart=3, grey=True)
    _check_jpeg(data, comps, h, w, grey=True)


def test_jpeg_interleaved_restarts_and_adobe_rgb():
    h, w = 40, 40
    img = _test_image(h, w, 5)
    data, comps = encode_jpeg(img, [(2, 2), (1, 1), (1, 1)], QUANT, restart=2)
    _check_jpeg(data, comps, h, w)
    data, comps = encode_jpeg(img, [(1, 1), (1, 1), (1, 1)], QUANT, adobe=0)  # Adobe transform 0: RGB samples
    _check_jpeg(data, comps, h, w, adobe=0)


def test_jpeg_errors():
    img = _test_image(16, 16, 1)
    data, _ = encode_jpeg(img, [(1, 1), (1, 1), (1, 1)], QUANT)
    for bad, words in [
        (data[:2], ["not a JPEG"]),
        (data[:300], ["no end-of-image", "truncated", "corrupt"]),
        (data.replace(b"\xff\xc0", b"\xff\xc3", 1), ["unsupported coding"]),
        (data.replace(b"\xff\xc0\x00\x11\x08", b"\xff\xc0\x00\x11\x0c", 1), ["8-bit"]),
    ]:
        with pytest.raises(pt.PathTracerError) as e:
            pt.decode_texture(bad)
        assert any(wd in e.value.message for wd in words), e.value.message
    # truncated or flipped entropy data: an error or an image, never a crash
    for cut in range(len(data) - 200, len(data), 17):
        try:
            pt.decode_texture(data[:cut])
        except pt.PathTracerError as e:
            assert e.code == abi.PT_ERR_INVALID_ARG
    for k in range(30):
        bad = bytearray(data)
        bad[len(data) - 100 + k * 3] ^= 0x3C
        try:
            pt.decode_texture(bytes(bad))
        except pt.PathTracerError as e:
            assert e.code == abi.PT_ERR_INVALID_ARG
