// image_io.cpp - skybox image files for the world builder: Radiance RGBE
// (.hdr) and OpenEXR (.exr), the two formats the reference's skybox loader
// reads through its image decoder (world.rs:1872-1957; its assets are a 2K
// .hdr and a 4K PIZ-compressed .exr).
//
// OpenEXR support: single-part scanline files, HALF / FLOAT / UINT channels
// (no subsampling), compression NONE, RLE, ZIPS, ZIP and PIZ; R, G, B and A
// channels (a lone Y channel is read as grey; missing A is 1).  ZIP blocks
// are zlib streams (inflated by the decoder below, RFC 1950/1951) of bytes
// that were delta-predicted and split into even and odd halves; PIZ blocks
// hold a value bitmap, a canonical Huffman code of the 16-bit words with a
// run-length symbol, and a two-dimensional Haar-style wavelet per channel
// plane, as the OpenEXR format specifies them.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pt_world.h"

namespace {

bool read_file(const char* path, std::vector<uint8_t>& data, std::string& err) {
    FILE* f = fopen(path, "rb");
    if (!f) {
        err = std::string("cannot read ") + path + ": " + strerror(errno);
        return false;
    }
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) data.insert(data.end(), buf, buf + n);
    fclose(f);
    return true;
}

// ------------------------------------------------------------- Radiance HDR
// "#?RADIANCE"/"#?RGBE" header, FORMAT=32-bit_rle_rgbe, "-Y H +X W"
// resolution, new-style run-length scanlines or flat pixels
bool read_hdr(const std::vector<uint8_t>& data, std::vector<float>& rgba, uint32_t& w, uint32_t& h, std::string& err,
              bool size_only) {
    size_t pos = 0;
    auto line = [&]() {
        std::string s;
        while (pos < data.size() && data[pos] != '\n') s.push_back((char)data[pos++]);
        if (pos < data.size()) pos++;
        return s;
    };
    const std::string magic = line();
    if (magic.rfind("#?", 0) != 0) {
        err = "not a Radiance HDR file";
        return false;
    }
    for (;;) {
        if (pos >= data.size()) {
            err = "truncated HDR header";
            return false;
        }
        const std::string s = line();
        if (s.empty()) break;
        if (s.rfind("FORMAT=", 0) == 0 && s != "FORMAT=32-bit_rle_rgbe") {
            err = "unsupported HDR format " + s;
            return false;
        }
    }
    const std::string res = line();
    int hh = 0, ww = 0;
    if (sscanf(res.c_str(), "-Y %d +X %d", &hh, &ww) != 2 || hh <= 0 || ww <= 0) {
        err = "unsupported HDR orientation: " + res;
        return false;
    }
    w = (uint32_t)ww;
    h = (uint32_t)hh;
    if (size_only) return true;
    rgba.assign((size_t)w * h * 4, 0.0f);
    std::vector<uint8_t> scan((size_t)w * 4);
    for (uint32_t y = 0; y < h; ++y) {
        if (pos + 4 > data.size()) {
            err = "truncated HDR data";
            return false;
        }
        if (w >= 8 && w < 32768 && data[pos] == 2 && data[pos + 1] == 2 && !(data[pos + 2] & 0x80)) {
            if ((uint32_t)((data[pos + 2] << 8) | data[pos + 3]) != w) {
                err = "bad HDR scanline";
                return false;
            }
            pos += 4;
            for (int c = 0; c < 4; ++c) {
                uint32_t x = 0;
                while (x < w) {
                    if (pos >= data.size()) {
                        err = "truncated HDR data";
                        return false;
                    }
                    uint32_t count = data[pos++];
                    if (count > 128) {
                        count -= 128;
                        if (pos >= data.size() || x + count > w) {
                            err = "bad HDR run";
                            return false;
                        }
                        const uint8_t v = data[pos++];
                        for (uint32_t k = 0; k < count; ++k) scan[(x++) * 4 + c] = v;
                    } else {
                        if (count == 0 || pos + count > data.size() || x + count > w) {
                            err = "bad HDR run";
                            return false;
                        }
                        for (uint32_t k = 0; k < count; ++k) scan[(x++) * 4 + c] = data[pos++];
                    }
                }
            }
        } else {
            if (pos + (size_t)w * 4 > data.size()) {
                err = "truncated HDR data";
                return false;
            }
            memcpy(scan.data(), &data[pos], (size_t)w * 4);
            pos += (size_t)w * 4;
        }
        for (uint32_t x = 0; x < w; ++x) {
            const uint8_t* p = &scan[x * 4];
            float* o = &rgba[((size_t)y * w + x) * 4];
            if (p[3] == 0) {
                o[0] = o[1] = o[2] = 0.0f;
            } else {
                const float scale = std::ldexp(1.0f, (int)p[3] - 136);
                o[0] = (float)p[0] * scale;
                o[1] = (float)p[1] * scale;
                o[2] = (float)p[2] * scale;
            }
            o[3] = 1.0f;
        }
    }
    return true;
}

// ------------------------------------------------------------- inflate
struct BitIn {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool bad = false;
    uint32_t bits(int k) {  // least significant bit first
        while (cnt < k) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((1u << k) - 1u);
        buf >>= k;
        cnt -= k;
        return v;
    }
};

// canonical Huffman code: symbols sorted by code length, then value
struct Huff {
    uint16_t count[16] = {0};
    std::vector<uint16_t> symbol;
    bool build(const uint8_t* lengths, int n) {
        for (int l = 0; l < 16; ++l) count[l] = 0;
        for (int i = 0; i < n; ++i) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = (left << 1) - count[l];
            if (left < 0) return false;  // over-subscribed
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; ++l) offs[l + 1] = (uint16_t)(offs[l] + count[l]);
        symbol.assign((size_t)n, 0);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    int decode(BitIn& in) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)in.bits(1);
            if (in.bad) return -1;
            const int c = count[l];
            if (code - c < first) return symbol[(size_t)(index + (code - first))];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        return -1;
    }
};

bool inflate_raw(BitIn& in, std::vector<uint8_t>& out, size_t limit) {
    static const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                                          35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2,
                                          3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                                           6145, 8193, 12289, 16385, 24577};
    static const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                           6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    int last = 0;
    while (!last) {
        last = (int)in.bits(1);
        const uint32_t type = in.bits(2);
        if (in.bad) return false;
        if (type == 0) {
            in.buf = 0;  // stored: align to a byte
            in.cnt = 0;
            if (in.pos + 4 > in.n) return false;
            const uint32_t len = in.p[in.pos] | (in.p[in.pos + 1] << 8);
            const uint32_t nlen = in.p[in.pos + 2] | (in.p[in.pos + 3] << 8);
            in.pos += 4;
            if ((len ^ 0xffffu) != nlen || in.pos + len > in.n || out.size() + len > limit) return false;
            out.insert(out.end(), in.p + in.pos, in.p + in.pos + len);
            in.pos += len;
            continue;
        }
        Huff lit, dist;
        if (type == 1) {
            uint8_t l[288];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            lit.build(l, 288);
            uint8_t d[30];
            for (int i = 0; i < 30; ++i) d[i] = 5;
            dist.build(d, 30);
        } else if (type == 2) {
            const int nlen = (int)in.bits(5) + 257, ndist = (int)in.bits(5) + 1, ncode = (int)in.bits(4) + 4;
            if (in.bad || nlen > 286 || ndist > 30) return false;
            static const uint8_t kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[kOrder[i]] = (uint8_t)in.bits(3);
            Huff code;
            if (in.bad || !code.build(cl, 19)) return false;
            uint8_t lens[286 + 30] = {0};
            int idx = 0;
            while (idx < nlen + ndist) {
                const int sym = code.decode(in);
                if (sym < 0) return false;
                if (sym < 16) {
                    lens[idx++] = (uint8_t)sym;
                } else {
                    int rep, val = 0;
                    if (sym == 16) {
                        if (idx == 0) return false;
                        val = lens[idx - 1];
                        rep = 3 + (int)in.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)in.bits(3);
                    } else {
                        rep = 11 + (int)in.bits(7);
                    }
                    if (in.bad || idx + rep > nlen + ndist) return false;
                    while (rep--) lens[idx++] = (uint8_t)val;
                }
            }
            if (!lit.build(lens, nlen) || !dist.build(lens + nlen, ndist)) return false;
        } else {
            return false;
        }
        for (;;) {
            const int sym = lit.decode(in);
            if (sym < 0) return false;
            if (sym < 256) {
                if (out.size() >= limit) return false;
                out.push_back((uint8_t)sym);
            } else if (sym == 256) {
                break;
            } else {
                const int li = sym - 257;
                if (li >= 29) return false;
                const size_t len = kLenBase[li] + in.bits(kLenExtra[li]);
                const int ds = dist.decode(in);
                if (ds < 0 || ds >= 30 || in.bad) return false;
                const size_t d = kDistBase[ds] + in.bits(kDistExtra[ds]);
                if (in.bad || d > out.size() || out.size() + len > limit) return false;
                const size_t from = out.size() - d;
                for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
            }
        }
    }
    return true;
}

// zlib stream (RFC 1950) into at most `limit` bytes
bool zlib_inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t limit) {
    if (n < 6 || (p[0] & 0x0f) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) return false;
    BitIn in{p + 2, n - 2};
    out.clear();
    return inflate_raw(in, out, limit);
}

// ------------------------------------------------------------- OpenEXR
float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h >> 15) << 31;
    const uint32_t exp = (h >> 10) & 0x1f, man = h & 0x3ff;
    float f;
    if (exp == 0) {
        f = std::ldexp((float)man, -24);  // zero or subnormal
        uint32_t u;
        memcpy(&u, &f, 4);
        u |= sign;
        memcpy(&f, &u, 4);
        return f;
    }
    const uint32_t u = exp == 31 ? (sign | 0x7f800000u | (man << 13)) : (sign | ((exp + 112u) << 23) | (man << 13));
    memcpy(&f, &u, 4);
    return f;
}

struct Channel {
    std::string name;
    int type;  // 0 UINT, 1 HALF, 2 FLOAT
    int size() const { return type == 1 ? 2 : 4; }
};

// PIZ: canonical Huffman code of 16-bit words (OpenEXR's packed code-length
// table, lengths up to 58, zero runs coded 59..63) with a run-length symbol
struct PizHuffman {
    static constexpr int kShortZeroRun = 59, kLongZeroRun = 63, kShortestLongRun = 6;
    std::vector<uint64_t> code;  // per symbol: length | code << 6
    bool unpack_table(const uint8_t*& p, const uint8_t* end, int im, int iM) {
        code.assign(65537, 0);
        uint64_t c = 0;
        int lc = 0;
        auto get = [&](int nbits, uint64_t& v) {
            while (lc < nbits) {
                if (p >= end) return false;
                c = (c << 8) | *p++;
                lc += 8;
            }
            lc -= nbits;
            v = (c >> lc) & ((1ull << nbits) - 1ull);
            return true;
        };
        for (int i = im; i <= iM; ++i) {
            uint64_t l;
            if (!get(6, l)) return false;
            code[(size_t)i] = l;
            if (l == (uint64_t)kLongZeroRun) {
                uint64_t z;
                if (!get(8, z)) return false;
                const int run = (int)z + kShortestLongRun;
                if (i + run > iM + 1) return false;
                for (int k = 0; k < run; ++k) code[(size_t)(i + k)] = 0;
                i += run - 1;
            } else if (l >= (uint64_t)kShortZeroRun) {
                const int run = (int)l - kShortZeroRun + 2;
                if (i + run > iM + 1) return false;
                for (int k = 0; k < run; ++k) code[(size_t)(i + k)] = 0;
                i += run - 1;
            }
        }
        // canonical codes: longer codes take the smaller values
        uint64_t n[59] = {0};
        for (int i = 0; i <= 65536; ++i) n[code[(size_t)i]] += 1;
        uint64_t start = 0;
        for (int l = 58; l > 0; --l) {
            const uint64_t next = (start + n[l]) >> 1;
            n[l] = start;
            start = next;
        }
        for (int i = 0; i <= 65536; ++i) {
            const uint64_t l = code[(size_t)i];
            if (l > 0) code[(size_t)i] = l | (n[l]++ << 6);
        }
        return true;
    }
};

bool piz_huffman_decode(const uint8_t* p, size_t n, std::vector<uint16_t>& out, size_t count) {
    if (n < 20) return false;
    auto u32 = [](const uint8_t* q) { return (uint32_t)q[0] | (q[1] << 8) | (q[2] << 16) | ((uint32_t)q[3] << 24); };
    const int im = (int)u32(p), iM = (int)u32(p + 4);
    const uint32_t table_bytes = u32(p + 8), nbits = u32(p + 12);
    if (im < 0 || iM > 65536 || im > iM || table_bytes > n - 20) return false;
    const uint8_t* t = p + 20;
    const uint8_t* q = t + table_bytes;  // the coded words follow the packed table
    const uint8_t* end = p + n;
    PizHuffman h;
    if (!h.unpack_table(t, q, im, iM)) return false;
    if ((size_t)(end - q) * 8 < nbits) return false;
    // decode tables: per code length, the first code and the symbols in code order
    std::vector<std::vector<int>> by_len(59);
    std::vector<uint64_t> first(59, 0);
    for (int i = im; i <= iM; ++i) {
        const uint64_t l = h.code[(size_t)i] & 63u;
        if (l) by_len[l].push_back(i);
    }
    for (int l = 1; l < 59; ++l)
        if (!by_len[l].empty()) first[l] = h.code[(size_t)by_len[l][0]] >> 6;  // symbols were numbered in order
    // codes up to kFast bits resolve with one table lookup; longer ones bit by bit
    constexpr int kFast = 12;
    std::vector<uint32_t> fast((size_t)1 << kFast, 0);  // length << 24 | symbol
    for (int l = 1; l <= kFast; ++l)
        for (size_t j = 0; j < by_len[l].size(); ++j) {
            const uint64_t c = first[l] + j;
            if (c >> l) return false;  // not a valid canonical code
            const size_t lo = (size_t)(c << (kFast - l)), n = (size_t)1 << (kFast - l);
            for (size_t e = lo; e < lo + n; ++e) fast[e] = ((uint32_t)l << 24) | (uint32_t)by_len[l][j];
        }
    const auto get_bit = [&](uint64_t b) { return (uint32_t)(q[b >> 3] >> (7 - (b & 7))) & 1u; };
    out.clear();
    out.reserve(count);
    const int rlc = iM;
    uint64_t bit = 0;
    while (bit < nbits) {
        int sym = -1;
        if (bit + kFast <= nbits) {
            // peek kFast bits: they lie within the 3 bytes from bit / 8
            const size_t byte = (size_t)(bit >> 3);
            uint32_t w = (uint32_t)q[byte] << 16;
            if (byte + 1 < (size_t)(end - q)) w |= (uint32_t)q[byte + 1] << 8;
            if (byte + 2 < (size_t)(end - q)) w |= q[byte + 2];
            const uint32_t e = fast[(w >> (24 - kFast - (bit & 7))) & ((1u << kFast) - 1u)];
            if (e) {
                sym = (int)(e & 0xffffffu);
                bit += e >> 24;
            }
        }
        if (sym < 0) {
            uint64_t v = 0;
            for (int len = 1;; ++len) {
                if (len > 58 || bit >= nbits) return false;
                v = (v << 1) | get_bit(bit++);
                const auto& syms = by_len[len];
                if (!syms.empty() && v >= first[len] && v - first[len] < syms.size()) {
                    sym = syms[(size_t)(v - first[len])];
                    break;
                }
            }
        }
        if (sym == rlc) {
            if (bit + 8 > nbits || out.empty()) return false;
            uint32_t cnt = 0;
            for (int k = 0; k < 8; ++k) cnt = (cnt << 1) | get_bit(bit++);
            if (out.size() + cnt > count) return false;
            const uint16_t s = out.back();
            out.insert(out.end(), cnt, s);
        } else {
            if (out.size() >= count) return false;
            out.push_back((uint16_t)sym);
        }
    }
    return out.size() == count;
}

// inverse of the 2D wavelet of one plane (nx x ny samples, strides ox, oy)
void wav2_decode(uint16_t* in, int nx, int ox, int ny, int oy, uint16_t mx) {
    const bool w14 = mx < (1 << 14);
    const int n = nx < ny ? nx : ny;
    int p = 1, p2;
    while (p <= n) p <<= 1;
    p >>= 1;
    p2 = p;
    p >>= 1;
    const auto dec14 = [](uint16_t l, uint16_t h, uint16_t& a, uint16_t& b) {
        const int hi = (int16_t)h;
        const int ai = (int16_t)l + (hi & 1) + (hi >> 1);
        a = (uint16_t)(int16_t)ai;
        b = (uint16_t)(int16_t)(ai - hi);
    };
    const auto dec16 = [](uint16_t l, uint16_t h, uint16_t& a, uint16_t& b) {
        const int m = l, d = h;
        const int bb = (m - (d >> 1)) & 0xffff;
        const int aa = (d + bb - (1 << 15)) & 0xffff;
        b = (uint16_t)bb;
        a = (uint16_t)aa;
    };
    const auto dec = [&](uint16_t l, uint16_t h, uint16_t& a, uint16_t& b) {
        if (w14)
            dec14(l, h, a, b);
        else
            dec16(l, h, a, b);
    };
    while (p >= 1) {
        uint16_t* py = in;
        uint16_t* ey = in + (ptrdiff_t)oy * (ny - p2);
        const int oy1 = oy * p, oy2 = oy * p2, ox1 = ox * p, ox2 = ox * p2;
        uint16_t i00, i01, i10, i11;
        for (; py <= ey; py += oy2) {
            uint16_t* px = py;
            uint16_t* ex = py + (ptrdiff_t)ox * (nx - p2);
            for (; px <= ex; px += ox2) {
                uint16_t* p01 = px + ox1;
                uint16_t* p10 = px + oy1;
                uint16_t* p11 = p10 + ox1;
                dec(*px, *p10, i00, i10);
                dec(*p01, *p11, i01, i11);
                dec(i00, i01, *px, *p01);
                dec(i10, i11, *p10, *p11);
            }
            if (nx & p) {
                uint16_t* p10 = px + oy1;
                dec(*px, *p10, i00, *p10);
                *px = i00;
            }
        }
        if (ny & p) {
            uint16_t* px = py;
            uint16_t* ex = py + (ptrdiff_t)ox * (nx - p2);
            for (; px <= ex; px += ox2) {
                uint16_t* p01 = px + ox1;
                dec(*px, *p01, i00, *p01);
                *px = i00;
            }
        }
        p2 = p;
        p >>= 1;
    }
}

// one PIZ block -> raw block bytes (lines, then channels, then pixels)
bool piz_decode(const uint8_t* p, size_t n, const std::vector<Channel>& ch, int nx, int ny, std::vector<uint8_t>& raw) {
    if (n < 4) return false;
    const uint16_t minnz = (uint16_t)(p[0] | (p[1] << 8)), maxnz = (uint16_t)(p[2] | (p[3] << 8));
    size_t pos = 4;
    std::vector<uint8_t> bitmap(8192, 0);
    if (minnz <= maxnz) {
        if (maxnz >= 8192 || pos + (maxnz - minnz + 1) > n) return false;
        memcpy(&bitmap[minnz], p + pos, (size_t)(maxnz - minnz + 1));
        pos += (size_t)(maxnz - minnz + 1);
    }
    // reverse lookup: the k-th value present (0 always counts as present)
    std::vector<uint16_t> lut(65536, 0);
    uint32_t k = 0;
    for (uint32_t i = 0; i < 65536; ++i)
        if (i == 0 || (bitmap[i >> 3] & (1u << (i & 7)))) lut[k++] = (uint16_t)i;
    const uint16_t maxv = (uint16_t)(k - 1);
    if (pos + 4 > n) return false;
    const uint32_t hlen = (uint32_t)p[pos] | (p[pos + 1] << 8) | (p[pos + 2] << 16) | ((uint32_t)p[pos + 3] << 24);
    pos += 4;
    if (pos + hlen > n) return false;
    size_t words = 0;
    for (const Channel& c : ch) words += (size_t)nx * ny * (c.size() / 2);
    std::vector<uint16_t> buf;
    if (!piz_huffman_decode(p + pos, hlen, buf, words)) return false;
    size_t off = 0;
    for (const Channel& c : ch) {
        const int sz = c.size() / 2;
        for (int j = 0; j < sz; ++j) wav2_decode(buf.data() + off + j, nx, sz, ny, nx * sz, maxv);
        off += (size_t)nx * ny * sz;
    }
    for (uint16_t& v : buf) v = lut[v];
    // channel planes (line after line) back to line-interleaved bytes
    raw.assign(words * 2, 0);
    std::vector<size_t> start(ch.size());
    off = 0;
    for (size_t i = 0; i < ch.size(); ++i) {
        start[i] = off;
        off += (size_t)nx * ny * (ch[i].size() / 2);
    }
    size_t o = 0;
    for (int y = 0; y < ny; ++y)
        for (size_t i = 0; i < ch.size(); ++i) {
            const size_t cnt = (size_t)nx * (ch[i].size() / 2);
            for (size_t q = 0; q < cnt; ++q) {
                const uint16_t v = buf[start[i] + (size_t)y * cnt + q];
                raw[o++] = (uint8_t)(v & 0xff);
                raw[o++] = (uint8_t)(v >> 8);
            }
        }
    return true;
}

// ZIP / RLE post-processing: undo the byte predictor, then interleave halves
void unpredict_interleave(std::vector<uint8_t>& t) {
    for (size_t i = 1; i < t.size(); ++i) t[i] = (uint8_t)(t[i - 1] + t[i] - 128);
    std::vector<uint8_t> out(t.size());
    const size_t half = (t.size() + 1) / 2;
    for (size_t i = 0; i < t.size(); ++i) out[i] = (i & 1) ? t[half + i / 2] : t[i / 2];
    t.swap(out);
}

bool rle_decode(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t limit) {
    out.clear();
    size_t i = 0;
    while (i < n) {
        const int c = (int8_t)p[i++];
        if (c < 0) {
            const size_t len = (size_t)(-c);
            if (i + len > n || out.size() + len > limit) return false;
            out.insert(out.end(), p + i, p + i + len);
            i += len;
        } else {
            if (i >= n || out.size() + (size_t)c + 1 > limit) return false;
            out.insert(out.end(), (size_t)c + 1, p[i++]);
        }
    }
    return true;
}

bool read_exr(const std::vector<uint8_t>& d, std::vector<float>& rgba, uint32_t& w, uint32_t& h, std::string& err,
              bool size_only) {
    auto fail = [&](const char* m) {
        err = std::string("EXR: ") + m;
        return false;
    };
    if (d.size() < 8 || d[0] != 0x76 || d[1] != 0x2f || d[2] != 0x31 || d[3] != 0x01) return fail("not an OpenEXR file");
    const uint32_t version = d[4] | (d[5] << 8) | (d[6] << 16) | ((uint32_t)d[7] << 24);
    if ((version & 0xff) != 2) return fail("unsupported version");
    if (version & 0x1a00) return fail("only single-part scanline images are supported (no tiles, deep data or parts)");
    size_t pos = 8;
    std::vector<Channel> ch;
    int compression = -1;
    int32_t win[4] = {0, 0, -1, -1};
    auto cstr = [&](std::string& s) {
        s.clear();
        while (pos < d.size() && d[pos]) s.push_back((char)d[pos++]);
        if (pos >= d.size()) return false;
        ++pos;
        return true;
    };
    auto i32 = [&](size_t at) {
        return (int32_t)(d[at] | (d[at + 1] << 8) | (d[at + 2] << 16) | ((uint32_t)d[at + 3] << 24));
    };
    for (;;) {
        std::string name, type;
        if (!cstr(name)) return fail("truncated header");
        if (name.empty()) break;
        if (!cstr(type) || pos + 4 > d.size()) return fail("truncated header");
        const int32_t size = i32(pos);
        pos += 4;
        if (size < 0 || pos + (size_t)size > d.size()) return fail("truncated header");
        const size_t vend = pos + (size_t)size;
        if (name == "channels" && type == "chlist") {
            size_t q = pos;
            while (q < vend && d[q]) {
                Channel c;
                while (q < vend && d[q]) c.name.push_back((char)d[q++]);
                ++q;
                if (q + 16 > vend) return fail("bad channel list");
                c.type = i32(q);
                const int32_t xs = i32(q + 8), ys = i32(q + 12);
                if (c.type < 0 || c.type > 2) return fail("unknown channel type");
                if (xs != 1 || ys != 1) return fail("subsampled channels are not supported");
                q += 16;
                ch.push_back(c);
            }
        } else if (name == "compression" && size >= 1) {
            compression = d[pos];
        } else if (name == "dataWindow" && size >= 16) {
            for (int k = 0; k < 4; ++k) win[k] = i32(pos + 4 * (size_t)k);
        }
        pos = vend;
    }
    if (ch.empty()) return fail("no channels");
    if (win[2] < win[0] || win[3] < win[1]) return fail("empty data window");
    const int64_t W = (int64_t)win[2] - win[0] + 1, H = (int64_t)win[3] - win[1] + 1;
    if (W > 65536 || H > 65536) return fail("image too large");
    int lines;
    switch (compression) {
        case 0: case 1: case 2: lines = 1; break;
        case 3: lines = 16; break;
        case 4: lines = 32; break;
        default: return fail("unsupported compression (NONE, RLE, ZIPS, ZIP and PIZ are read)");
    }
    w = (uint32_t)W;
    h = (uint32_t)H;
    size_t pixel_bytes = 0;
    for (const Channel& c : ch) pixel_bytes += (size_t)c.size();
    int ir = -1, ig = -1, ib = -1, ia = -1, iy = -1;
    for (size_t i = 0; i < ch.size(); ++i) {
        if (ch[i].name == "R") ir = (int)i;
        if (ch[i].name == "G") ig = (int)i;
        if (ch[i].name == "B") ib = (int)i;
        if (ch[i].name == "A") ia = (int)i;
        if (ch[i].name == "Y") iy = (int)i;
    }
    if ((ir < 0 || ig < 0 || ib < 0) && iy < 0) return fail("no R, G, B (or Y) channels");
    if (size_only) return true;
    const int64_t chunks = (H + lines - 1) / lines;
    if (pos + (size_t)chunks * 8 > d.size()) return fail("truncated offset table");
    rgba.assign((size_t)W * H * 4, 0.0f);
    for (size_t i = 0; i < rgba.size(); i += 4) rgba[i + 3] = 1.0f;
    // chunk k holds lines [k * lines, k * lines + ny) of the data window (the
    // offset table is in increasing y whatever the line order), so chunks
    // decode independently into disjoint rows
    auto decode_chunk = [&](int64_t k, std::vector<uint8_t>& raw) -> const char* {
        uint64_t off = 0;
        for (int b = 7; b >= 0; --b) off = (off << 8) | d[pos + (size_t)k * 8 + (size_t)b];
        if (off + 8 > d.size()) return "chunk offset out of range";
        const int32_t y0 = i32(off), packed = i32(off + 4);
        if (packed < 0 || off + 8 + (uint64_t)packed > d.size()) return "chunk size out of range";
        const int64_t first = (int64_t)y0 - win[1];
        if (first != k * lines) return "chunk line out of order";
        const int ny = (int)(first + lines <= H ? lines : H - first);
        const size_t expect = (size_t)W * ny * pixel_bytes;
        const uint8_t* src = &d[off + 8];
        if ((size_t)packed == expect || compression == 0) {
            if ((size_t)packed != expect) return "uncompressed chunk has the wrong size";
            raw.assign(src, src + packed);
        } else if (compression == 1) {
            if (!rle_decode(src, (size_t)packed, raw, expect) || raw.size() != expect) return "bad RLE chunk";
            unpredict_interleave(raw);
        } else if (compression == 2 || compression == 3) {
            if (!zlib_inflate(src, (size_t)packed, raw, expect) || raw.size() != expect) return "bad ZIP chunk";
            unpredict_interleave(raw);
        } else {
            if (!piz_decode(src, (size_t)packed, ch, (int)W, ny, raw) || raw.size() != expect) return "bad PIZ chunk";
        }
        // lines of the block: every channel's W values in turn
        size_t o = 0;
        for (int y = 0; y < ny; ++y) {
            float* row = &rgba[(size_t)(first + y) * W * 4];
            for (size_t i = 0; i < ch.size(); ++i) {
                int dst = -1;
                if ((int)i == ir) dst = 0;
                else if ((int)i == ig) dst = 1;
                else if ((int)i == ib) dst = 2;
                else if ((int)i == ia) dst = 3;
                const bool grey = (int)i == iy && (ir < 0 || ig < 0 || ib < 0);
                for (int64_t x = 0; x < W; ++x) {
                    float v;
                    const uint8_t* e = &raw[o];
                    if (ch[i].type == 1) {
                        v = half_to_float((uint16_t)(e[0] | (e[1] << 8)));
                    } else {
                        uint32_t u = e[0] | (e[1] << 8) | (e[2] << 16) | ((uint32_t)e[3] << 24);
                        if (ch[i].type == 2)
                            memcpy(&v, &u, 4);
                        else
                            v = (float)u;
                    }
                    o += (size_t)ch[i].size();
                    if (dst >= 0) row[x * 4 + dst] = v;
                    if (grey) row[x * 4] = row[x * 4 + 1] = row[x * 4 + 2] = v;
                }
            }
        }
        return nullptr;
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t nthreads = std::min<int64_t>(chunks, std::max(1u, std::min(hw, 16u)));
    std::atomic<int64_t> next{0};
    std::vector<const char*> errors((size_t)nthreads, nullptr);
    auto worker = [&](int64_t t) {
        std::vector<uint8_t> raw;
        for (int64_t k; !errors[(size_t)t] && (k = next.fetch_add(1)) < chunks;) errors[(size_t)t] = decode_chunk(k, raw);
    };
    std::vector<std::thread> pool;
    for (int64_t t = 1; t < nthreads; ++t) pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool) th.join();
    for (const char* e : errors)
        if (e) return fail(e);
    return true;
}

bool read_image(const char* path, std::vector<float>& rgba, uint32_t& w, uint32_t& h, std::string& err,
                bool size_only = false) {
    std::vector<uint8_t> data;
    if (!read_file(path, data, err)) return false;
    if (data.size() >= 4 && data[0] == 0x76 && data[1] == 0x2f && data[2] == 0x31 && data[3] == 0x01)
        return read_exr(data, rgba, w, h, err, size_only);
    return read_hdr(data, rgba, w, h, err, size_only);
}

void put_error(char* error, size_t size, const std::string& msg) {
    if (error && size) snprintf(error, size, "%s", msg.c_str());
}

}  // namespace

extern "C" int ptw_read_image_rgba(const char* path, float* rgba, uint64_t capacity, uint32_t* width, uint32_t* height,
                                   char* error, size_t error_size) {
    if (!path || !width || !height) return PT_ERR_INVALID_ARG;
    std::vector<float> px;
    uint32_t w = 0, h = 0;
    std::string err;
    if (!read_image(path, px, w, h, err, rgba == nullptr)) {
        put_error(error, error_size, err);
        return PT_ERR_INVALID_ARG;
    }
    *width = w;
    *height = h;
    if (!rgba) return PT_OK;
    if (capacity < px.size()) {
        put_error(error, error_size, "output buffer too small");
        return PT_ERR_OUT_OF_LIMITS;
    }
    memcpy(rgba, px.data(), px.size() * sizeof(float));
    return PT_OK;
}

extern "C" int ptw_set_skybox_file(ptw_world* world, const char* path, char* error, size_t error_size) {
    if (!world || !path) return PT_ERR_INVALID_ARG;
    std::vector<float> px;
    uint32_t w = 0, h = 0;
    std::string err;
    if (!read_image(path, px, w, h, err)) {
        put_error(error, error_size, err);
        return PT_ERR_INVALID_ARG;
    }
    const int rc = ptw_set_skybox_rgba(world, px.data(), w, h);
    if (rc) put_error(error, error_size, ptw_last_error(world));
    return rc;
}
