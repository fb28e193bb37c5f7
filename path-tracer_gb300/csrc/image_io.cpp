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
#include <array>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/pt_world.h"

namespace {

// skybox images up to 2^28 pixels (4 GiB as RGBA32F); the reference's are 2K and 4K equirects
constexpr int64_t kMaxSkyPixels = (int64_t)1 << 28;

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
    if ((uint64_t)ww * (uint64_t)hh > (uint64_t)kMaxSkyPixels) {
        err = "HDR image too large";
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
    if (W > 65536 || H > 65536 || W * H > kMaxSkyPixels) return fail("image too large");
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
    for (int64_t t = 1; t < nthreads; ++t) {
        try {
            pool.emplace_back(worker, t);
        } catch (const std::system_error&) {
            break;  // worker 0 takes the remaining chunks
        }
    }
    worker(0);
    for (auto& th : pool) th.join();
    for (const char* e : errors)
        if (e) return fail(e);
    return true;
}

// ------------------------------------------------------------- PNG
// Decoded samples as the image library hands them to the glTF importer:
// palette and low-bit-depth grey expanded to 8 bits, a tRNS chunk expanded
// to an alpha channel, 16-bit samples kept.
struct Raster {
    uint32_t w = 0, h = 0;
    int channels = 0;  // 1 grey, 2 grey + alpha, 3 RGB, 4 RGBA
    int depth = 8;     // 8 or 16
    std::vector<uint16_t> v;
};

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

uint32_t crc32_png(const uint8_t* d, size_t n) {
    static const std::array<uint32_t, 256> table = [] {
        std::array<uint32_t, 256> t{};
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    uint32_t c = 0xffffffffu;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ d[i]) & 0xff] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

bool decode_png(const uint8_t* d, size_t n, Raster& out, std::string& err, uint32_t max_side) {
    static const uint8_t kSig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    if (n < 8 || memcmp(d, kSig, 8) != 0) {
        err = "not a PNG file";
        return false;
    }
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, palette, trns;
    bool seen_ihdr = false, seen_iend = false;
    for (size_t pos = 8; pos + 12 <= n && !seen_iend;) {
        const uint32_t len = be32(d + pos);
        if (len > n - pos - 12) {
            err = "PNG chunk runs past the end of the file";
            return false;
        }
        const uint8_t* type = d + pos + 4;
        const uint8_t* body = d + pos + 8;
        if (crc32_png(type, (size_t)len + 4) != be32(body + len)) {
            err = "PNG chunk CRC mismatch";
            return false;
        }
        if (!memcmp(type, "IHDR", 4)) {
            if (len != 13) {
                err = "bad PNG header";
                return false;
            }
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            seen_ihdr = true;
            if (body[10] != 0 || body[11] != 0 || interlace > 1) {
                err = "unsupported PNG compression, filter or interlace method";
                return false;
            }
        } else if (!memcmp(type, "PLTE", 4)) {
            palette.assign(body, body + len);
        } else if (!memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!memcmp(type, "IEND", 4)) {
            seen_iend = true;
        } else if (!(type[0] & 0x20)) {
            err = "unknown critical PNG chunk";
            return false;
        }
        pos += (size_t)len + 12;
    }
    if (!seen_ihdr || w == 0 || h == 0 || w > 65536 || h > 65536) {
        err = "bad PNG header";
        return false;
    }
    if (w > max_side || h > max_side) {
        err = "image larger than the atlas";
        return false;
    }
    int samples;  // per pixel in the file
    switch (ctype) {
        case 0: samples = 1; break;
        case 2: samples = 3; break;
        case 3: samples = 1; break;
        case 4: samples = 2; break;
        case 6: samples = 4; break;
        default: err = "bad PNG colour type"; return false;
    }
    const bool depth_ok = ctype == 0   ? (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)
                          : ctype == 3 ? (depth == 1 || depth == 2 || depth == 4 || depth == 8)
                                       : (depth == 8 || depth == 16);
    if (!depth_ok) {
        err = "bad PNG bit depth";
        return false;
    }
    if (ctype == 3 && (palette.empty() || palette.size() % 3)) {
        err = "PNG palette missing";
        return false;
    }
    const int bpp_bits = samples * depth;
    const size_t fb = (size_t)std::max(1, bpp_bits / 8);  // filter byte distance
    // Adam7 passes (x0, y0, dx, dy), or one pass
    static const int kAdam7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                                     {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    const int npass = interlace ? 7 : 1;
    size_t raw_size = 0;
    for (int ps = 0; ps < npass; ++ps) {
        const int* a = interlace ? kAdam7[ps] : nullptr;
        const uint64_t pw = a ? (w > (uint32_t)a[0] ? (w - a[0] + a[2] - 1) / a[2] : 0) : w;
        const uint64_t ph = a ? (h > (uint32_t)a[1] ? (h - a[1] + a[3] - 1) / a[3] : 0) : h;
        if (pw && ph) raw_size += (size_t)ph * (1 + (size_t)((pw * bpp_bits + 7) / 8));
    }
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), raw, raw_size) || raw.size() != raw_size) {
        err = "bad PNG image data";
        return false;
    }
    const bool has_trns = !trns.empty() && ctype != 4 && ctype != 6;
    out.w = w;
    out.h = h;
    out.depth = (ctype == 3 || depth < 8) ? 8 : depth;
    out.channels = ctype == 3 ? (has_trns ? 4 : 3) : samples + (has_trns ? 1 : 0);
    out.v.assign((size_t)w * h * out.channels, 0);
    const uint16_t maxv = out.depth == 16 ? 65535 : 255;
    size_t at = 0;
    std::vector<uint8_t> prev, cur;
    for (int ps = 0; ps < npass; ++ps) {
        const int* a = interlace ? kAdam7[ps] : nullptr;
        const uint32_t x0 = a ? a[0] : 0, y0 = a ? a[1] : 0, dx = a ? a[2] : 1, dy = a ? a[3] : 1;
        const uint32_t pw = w > x0 ? (w - x0 + dx - 1) / dx : 0, ph = h > y0 ? (h - y0 + dy - 1) / dy : 0;
        if (!pw || !ph) continue;
        const size_t rb = (size_t)(((uint64_t)pw * bpp_bits + 7) / 8);
        prev.assign(rb, 0);
        cur.assign(rb, 0);
        for (uint32_t r = 0; r < ph; ++r) {
            const uint8_t f = raw[at++];
            const uint8_t* src = &raw[at];
            at += rb;
            for (size_t i = 0; i < rb; ++i) {
                const int left = i >= fb ? cur[i - fb] : 0, up = prev[i], ul = i >= fb ? prev[i - fb] : 0;
                int v = src[i];
                switch (f) {
                    case 0: break;
                    case 1: v += left; break;
                    case 2: v += up; break;
                    case 3: v += (left + up) >> 1; break;
                    case 4: {
                        const int pp = left + up - ul, pa = std::abs(pp - left), pb = std::abs(pp - up),
                                  pc = std::abs(pp - ul);
                        v += (pa <= pb && pa <= pc) ? left : (pb <= pc ? up : ul);
                        break;
                    }
                    default: err = "bad PNG filter type"; return false;
                }
                cur[i] = (uint8_t)v;
            }
            // unpack the row's samples into the output
            const uint32_t y = y0 + r * dy;
            for (uint32_t c = 0; c < pw; ++c) {
                const uint32_t x = x0 + c * dx;
                uint16_t* o = &out.v[((size_t)y * w + x) * out.channels];
                uint32_t s[4] = {0, 0, 0, 0};
                for (int k = 0; k < samples; ++k) {
                    const uint64_t bit = ((uint64_t)c * samples + k) * depth;
                    if (depth == 16)
                        s[k] = ((uint32_t)cur[bit / 8] << 8) | cur[bit / 8 + 1];
                    else if (depth == 8)
                        s[k] = cur[bit / 8];
                    else
                        s[k] = (cur[bit / 8] >> (8 - depth - (bit % 8))) & ((1u << depth) - 1u);
                }
                if (ctype == 3) {
                    const uint32_t i = s[0];
                    if ((size_t)i * 3 + 2 >= palette.size()) {
                        err = "PNG palette index out of range";
                        return false;
                    }
                    o[0] = palette[i * 3];
                    o[1] = palette[i * 3 + 1];
                    o[2] = palette[i * 3 + 2];
                    if (has_trns) o[3] = i < trns.size() ? trns[i] : 255;
                    continue;
                }
                const uint32_t scale = depth < 8 ? 255u / ((1u << depth) - 1u) : 1u;
                for (int k = 0; k < samples; ++k) o[k] = (uint16_t)(s[k] * scale);
                if (has_trns) {
                    bool key;
                    if (ctype == 0)
                        key = trns.size() >= 2 && s[0] == (((uint32_t)trns[0] << 8 | trns[1]) & (depth == 16 ? 0xffffu : (1u << depth) - 1u));
                    else
                        key = trns.size() >= 6 && s[0] == (((uint32_t)trns[0] << 8) | trns[1]) &&
                              s[1] == (((uint32_t)trns[2] << 8) | trns[3]) && s[2] == (((uint32_t)trns[4] << 8) | trns[5]);
                    o[samples] = key ? 0 : maxv;
                }
            }
            std::swap(prev, cur);
        }
    }
    return true;
}

// ------------------------------------------------------------- JPEG
// Huffman-coded JPEG (ITU-T T.81): baseline, extended sequential and
// progressive, 8-bit samples, 1, 3 or 4 components with sampling factors
// 1..4, restart intervals.  Floating-point separable inverse DCT, chroma
// upsampled with the triangle filter for 2:1 horizontal and 2:1 horizontal +
// vertical subsampling (replication otherwise), JFIF YCbCr -> RGB.
const uint8_t kNatural[64 + 16] = {
    0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
    41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
    30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63,
    // a malformed run past coefficient 63 lands on 63
    63, 63, 63, 63, 63, 63, 63, 63, 63, 63, 63, 63, 63, 63, 63, 63};

struct JHuff {
    bool present = false;
    uint8_t sym[256] = {0};
    int32_t maxcode[18];
    int32_t valoff[18];
    uint16_t fast[1 << 9];  // 9-bit lookahead: length << 8 | symbol, 0 for longer codes
    bool build(const uint8_t counts[16], const uint8_t* syms, int n) {
        memcpy(sym, syms, (size_t)n);
        int32_t code = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            valoff[l] = k - code;
            code += counts[l - 1];
            k += counts[l - 1];
            if (code > (1 << l)) return false;  // over-subscribed
            maxcode[l] = counts[l - 1] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7fffffff;
        memset(fast, 0, sizeof fast);
        code = 0;
        k = 0;
        for (int l = 1; l <= 9; ++l, code <<= 1)
            for (int i = 0; i < counts[l - 1]; ++i, ++code, ++k)
                for (int e = code << (9 - l); e < ((code + 1) << (9 - l)); ++e) fast[e] = (uint16_t)(l << 8 | sym[k]);
        present = true;
        return true;
    }
};

struct JBits {
    const uint8_t* d;
    size_t n, pos;
    uint64_t acc = 0;
    int cnt = 0;
    bool marker = false;  // stopped at a marker: zeros are fed from here on
    void fill() {
        while (cnt <= 56) {
            uint32_t b = 0;
            if (!marker && pos < n) {
                b = d[pos];
                if (b == 0xff) {
                    if (pos + 1 < n && d[pos + 1] == 0x00) {
                        pos += 2;
                    } else {
                        marker = true;
                        b = 0;
                    }
                } else {
                    ++pos;
                }
            }
            acc |= (uint64_t)b << (56 - cnt);
            cnt += 8;
        }
    }
    uint32_t peek(int k) {
        if (cnt < k) fill();
        return (uint32_t)(acc >> (64 - k));
    }
    void skip(int k) {
        acc <<= k;
        cnt -= k;
    }
    uint32_t get(int k) {
        if (k == 0) return 0;
        const uint32_t v = peek(k);
        skip(k);
        return v;
    }
    int decode(const JHuff& h) {
        const uint32_t e = h.fast[peek(9)];
        if (e) {
            skip((int)(e >> 8));
            return (int)(e & 0xff);
        }
        const uint32_t look = peek(16);
        for (int l = 10; l <= 16; ++l) {
            const int32_t code = (int32_t)(look >> (16 - l));
            if (code <= h.maxcode[l]) {
                skip(l);
                const int32_t i = h.valoff[l] + code;
                return i >= 0 && i < 256 ? h.sym[i] : -1;
            }
        }
        return -1;
    }
    static int extend(uint32_t v, int t) { return t && v < (1u << (t - 1)) ? (int)v - (1 << t) + 1 : (int)v; }
};

struct JComp {
    int id = 0, h = 1, v = 1, tq = 0;
    int dc = 0, ac = 0;
    int bw = 0, bh = 0;  // blocks of the MCU-aligned grid
    int pred = 0;
    bool latched = false;
    uint16_t q[64] = {0};
    std::vector<int16_t> coef;
};

bool decode_jpeg(const uint8_t* d, size_t n, Raster& out, std::string& err, uint32_t max_side) {
    auto fail = [&](const char* m) {
        err = std::string("JPEG: ") + m;
        return false;
    };
    if (n < 4 || d[0] != 0xff || d[1] != 0xd8) return fail("not a JPEG file");
    uint16_t qt[4][64] = {{0}};
    bool qt_present[4] = {false, false, false, false};
    JHuff hdc[4], hac[4];
    std::vector<JComp> comps;
    int W = 0, H = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    bool progressive = false, frame = false;
    int adobe = -1;  // APP14 colour transform, -1 when absent
    uint32_t restart = 0;
    size_t pos = 2;
    for (;;) {
        while (pos < n && d[pos] != 0xff) ++pos;  // tolerate junk between segments
        while (pos < n && d[pos] == 0xff) ++pos;
        if (pos >= n) return fail("no end-of-image marker");
        const uint8_t m = d[pos++];
        if (m == 0xd9) break;
        if (m == 0xd8 || (m >= 0xd0 && m <= 0xd7) || m == 0x01) continue;
        if (pos + 2 > n) return fail("truncated segment");
        const size_t len = ((size_t)d[pos] << 8) | d[pos + 1];
        if (len < 2 || pos + len > n) return fail("truncated segment");
        const uint8_t* s = d + pos + 2;
        const size_t sl = len - 2;
        pos += len;
        if (m == 0xdb) {  // DQT
            for (size_t i = 0; i < sl;) {
                const int pq = s[i] >> 4, tq = s[i] & 15;
                if (tq > 3 || pq > 1 || i + 1 + 64 * (size_t)(pq + 1) > sl) return fail("bad quantisation table");
                for (int k = 0; k < 64; ++k)
                    qt[tq][kNatural[k]] = pq ? (uint16_t)(s[i + 1 + 2 * k] << 8 | s[i + 2 + 2 * k]) : s[i + 1 + k];
                qt_present[tq] = true;
                i += 1 + 64 * (size_t)(pq + 1);
            }
        } else if (m == 0xc4) {  // DHT
            for (size_t i = 0; i < sl;) {
                if (i + 17 > sl) return fail("bad Huffman table");
                const int tc = s[i] >> 4, th = s[i] & 15;
                int total = 0;
                for (int k = 0; k < 16; ++k) total += s[i + 1 + k];
                if (tc > 1 || th > 3 || total > 256 || i + 17 + (size_t)total > sl) return fail("bad Huffman table");
                if (!(tc ? hac[th] : hdc[th]).build(s + i + 1, s + i + 17, total)) return fail("bad Huffman table");
                i += 17 + (size_t)total;
            }
        } else if (m == 0xdd) {  // DRI
            if (sl < 2) return fail("bad restart interval");
            restart = ((uint32_t)s[0] << 8) | s[1];
        } else if (m == 0xee) {  // APP14
            if (sl >= 12 && !memcmp(s, "Adobe", 5)) adobe = s[11];
        } else if (m == 0xc0 || m == 0xc1 || m == 0xc2) {
            if (frame) return fail("more than one frame");
            frame = true;
            progressive = m == 0xc2;
            if (sl < 6 || s[0] != 8) return fail("only 8-bit samples are supported");
            H = s[1] << 8 | s[2];
            W = s[3] << 8 | s[4];
            const int nc = s[5];
            if (W == 0 || H == 0) return fail("zero image size (DNL is not supported)");
            if ((uint32_t)W > max_side || (uint32_t)H > max_side) return fail("image larger than the atlas");
            if ((nc != 1 && nc != 3 && nc != 4) || sl < 6 + 3 * (size_t)nc) return fail("unsupported component count");
            for (int c = 0; c < nc; ++c) {
                JComp jc;
                jc.id = s[6 + 3 * c];
                jc.h = s[7 + 3 * c] >> 4;
                jc.v = s[7 + 3 * c] & 15;
                jc.tq = s[8 + 3 * c];
                if (jc.h < 1 || jc.h > 4 || jc.v < 1 || jc.v > 4 || jc.tq > 3) return fail("bad component");
                hmax = std::max(hmax, jc.h);
                vmax = std::max(vmax, jc.v);
                comps.push_back(jc);
            }
            mcux = (W + 8 * hmax - 1) / (8 * hmax);
            mcuy = (H + 8 * vmax - 1) / (8 * vmax);
            for (JComp& c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.coef.assign((size_t)c.bw * c.bh * 64, 0);
            }
        } else if ((m >= 0xc3 && m <= 0xcf) && m != 0xc4 && m != 0xc8 && m != 0xcc) {
            return fail("unsupported coding (lossless, hierarchical or arithmetic)");
        } else if (m == 0xda) {  // SOS
            if (!frame || sl < 1) return fail("scan before frame");
            const int ns = s[0];
            if (ns < 1 || ns > 4 || sl < 4 + 2 * (size_t)ns) return fail("bad scan header");
            JComp* sc[4];
            for (int i = 0; i < ns; ++i) {
                sc[i] = nullptr;
                for (JComp& c : comps)
                    if (c.id == s[1 + 2 * i]) sc[i] = &c;
                if (!sc[i]) return fail("scan names an unknown component");
                sc[i]->dc = s[2 + 2 * i] >> 4;
                sc[i]->ac = s[2 + 2 * i] & 15;
                if (sc[i]->dc > 3 || sc[i]->ac > 3) return fail("bad table selector");
                if (!sc[i]->latched) {
                    if (!qt_present[sc[i]->tq]) return fail("missing quantisation table");
                    memcpy(sc[i]->q, qt[sc[i]->tq], sizeof sc[i]->q);
                    sc[i]->latched = true;
                }
            }
            const int ss = s[1 + 2 * ns], se = s[2 + 2 * ns], ah = s[3 + 2 * ns] >> 4, al = s[3 + 2 * ns] & 15;
            if (progressive) {
                if (ss > se || se > 63 || (ss == 0 && se != 0) || (ss > 0 && ns != 1) || al > 13)
                    return fail("bad progressive scan");
            } else if (ss != 0 || se != 63 || ah || al) {
                return fail("bad sequential scan");
            }
            const bool dc_scan = ss == 0;
            for (int i = 0; i < ns; ++i) {
                if (((!progressive || (dc_scan && ah == 0)) && !hdc[sc[i]->dc].present) ||
                    ((!progressive || !dc_scan) && !hac[sc[i]->ac].present))
                    return fail("missing Huffman table");
                sc[i]->pred = 0;
            }
            JBits bits{d, n, pos};
            int eobrun = 0;
            bool bad = false;
            // one block of component c at coefficient offset `blk`
            auto block = [&](JComp& c, int16_t* coef) {
                if (!progressive) {
                    const int t = bits.decode(hdc[c.dc]);
                    if (t < 0 || t > 11) return bad = true, void();
                    c.pred += JBits::extend(bits.get(t), t);
                    coef[0] = (int16_t)c.pred;
                    for (int k = 1; k < 64;) {
                        const int rs = bits.decode(hac[c.ac]);
                        if (rs < 0) return bad = true, void();
                        const int r = rs >> 4, sz = rs & 15;
                        if (!sz) {
                            if (r != 15) break;
                            k += 16;
                            continue;
                        }
                        k += r;
                        coef[kNatural[k]] = (int16_t)JBits::extend(bits.get(sz), sz);
                        ++k;
                    }
                } else if (dc_scan) {
                    if (ah == 0) {
                        const int t = bits.decode(hdc[c.dc]);
                        if (t < 0 || t > 11) return bad = true, void();
                        c.pred += JBits::extend(bits.get(t), t);
                        coef[0] = (int16_t)(c.pred * (1 << al));
                    } else if (bits.get(1)) {
                        coef[0] = (int16_t)(coef[0] | (1 << al));
                    }
                } else if (ah == 0) {
                    if (eobrun > 0) {
                        --eobrun;
                        return;
                    }
                    for (int k = ss; k <= se;) {
                        const int rs = bits.decode(hac[c.ac]);
                        if (rs < 0) return bad = true, void();
                        const int r = rs >> 4, sz = rs & 15;
                        if (!sz) {
                            if (r < 15) {
                                eobrun = (1 << r) - 1;
                                if (r) eobrun += (int)bits.get(r);
                                break;
                            }
                            k += 16;
                            continue;
                        }
                        k += r;
                        coef[kNatural[k]] = (int16_t)(JBits::extend(bits.get(sz), sz) * (1 << al));
                        ++k;
                    }
                } else {
                    // successive-approximation refinement of AC coefficients
                    const int p1 = 1 << al, m1 = -p1;
                    int k = ss;
                    const auto refine = [&](int16_t& cf) {
                        if (bits.get(1) && (cf & p1) == 0) cf = (int16_t)(cf + (cf >= 0 ? p1 : m1));
                    };
                    if (eobrun == 0) {
                        for (; k <= se; ++k) {
                            const int rs = bits.decode(hac[c.ac]);
                            if (rs < 0) return bad = true, void();
                            int r = rs >> 4, val = 0;
                            if (rs & 15) {
                                val = bits.get(1) ? p1 : m1;
                            } else if (r != 15) {
                                eobrun = 1 << r;
                                if (r) eobrun += (int)bits.get(r);
                                break;
                            }
                            while (k <= se) {
                                int16_t& cf = coef[kNatural[k]];
                                if (cf != 0) {
                                    refine(cf);
                                } else if (--r < 0) {
                                    break;
                                }
                                ++k;
                            }
                            if (val && k <= se) coef[kNatural[k]] = (int16_t)val;
                        }
                    }
                    if (eobrun > 0) {
                        for (; k <= se; ++k)
                            if (coef[kNatural[k]] != 0) refine(coef[kNatural[k]]);
                        --eobrun;
                    }
                }
            };
            auto restart_marker = [&]() {
                bits.acc = 0;
                bits.cnt = 0;
                bits.marker = false;
                size_t p = bits.pos;
                while (p + 1 < n && !(d[p] == 0xff && d[p + 1] != 0x00 && d[p + 1] != 0xff)) ++p;
                if (p + 1 < n && d[p + 1] >= 0xd0 && d[p + 1] <= 0xd7) p += 2;
                bits.pos = p;
                for (int i = 0; i < ns; ++i) sc[i]->pred = 0;
                eobrun = 0;
            };
            uint32_t mcu = 0;
            if (ns == 1) {
                JComp& c = *sc[0];
                const int cw = ((W * c.h + hmax - 1) / hmax + 7) / 8, ch = ((H * c.v + vmax - 1) / vmax + 7) / 8;
                for (int by = 0; by < ch && !bad; ++by)
                    for (int bx = 0; bx < cw && !bad; ++bx, ++mcu) {
                        if (restart && mcu && mcu % restart == 0) restart_marker();
                        block(c, &c.coef[((size_t)by * c.bw + bx) * 64]);
                    }
            } else {
                for (int my = 0; my < mcuy && !bad; ++my)
                    for (int mx = 0; mx < mcux && !bad; ++mx, ++mcu) {
                        if (restart && mcu && mcu % restart == 0) restart_marker();
                        for (int i = 0; i < ns; ++i) {
                            JComp& c = *sc[i];
                            for (int v = 0; v < c.v; ++v)
                                for (int h = 0; h < c.h; ++h)
                                    block(c, &c.coef[((size_t)(my * c.v + v) * c.bw + (mx * c.h + h)) * 64]);
                        }
                    }
            }
            if (bad) return fail("corrupt entropy-coded data");
            // continue after the scan's data: the next marker that is not a restart marker
            size_t p = bits.pos;
            while (p + 1 < n && !(d[p] == 0xff && d[p + 1] != 0x00 && d[p + 1] != 0xff &&
                                  !(d[p + 1] >= 0xd0 && d[p + 1] <= 0xd7)))
                ++p;
            pos = p;
        } else if (m == 0xdc) {
            return fail("DNL marker is not supported");
        }
        // APPn, COM and other segments are skipped
    }
    if (!frame) return fail("no frame");
    // dequantise and inverse-transform every block into component planes
    static const std::array<float, 64> kCos = [] {
        std::array<float, 64> t{};
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                t[x * 8 + u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0) / 2.0);
        return t;
    }();
    std::vector<std::vector<uint8_t>> plane(comps.size());
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        JComp& c = comps[ci];
        const size_t stride = (size_t)c.bw * 8;
        plane[ci].assign(stride * c.bh * 8, 0);
        for (int by = 0; by < c.bh; ++by)
            for (int bx = 0; bx < c.bw; ++bx) {
                const int16_t* cf = &c.coef[((size_t)by * c.bw + bx) * 64];
                float f[64], t[64];
                for (int i = 0; i < 64; ++i) f[i] = (float)cf[i] * (float)c.q[i];
                for (int v = 0; v < 8; ++v)  // rows: horizontal frequencies -> x
                    for (int x = 0; x < 8; ++x) {
                        float a = 0.0f;
                        for (int u = 0; u < 8; ++u) a += kCos[x * 8 + u] * f[v * 8 + u];
                        t[v * 8 + x] = a;
                    }
                for (int y = 0; y < 8; ++y)
                    for (int x = 0; x < 8; ++x) {
                        float a = 0.0f;
                        for (int v = 0; v < 8; ++v) a += kCos[y * 8 + v] * t[v * 8 + x];
                        const float px = std::floor(a + 128.0f + 0.5f);
                        plane[ci][((size_t)by * 8 + y) * stride + (size_t)bx * 8 + x] =
                            (uint8_t)(px < 0.0f ? 0.0f : px > 255.0f ? 255.0f : px);
                    }
            }
        std::vector<int16_t>().swap(c.coef);
    }
    // upsample every component to the image size
    std::vector<std::vector<uint8_t>> full(comps.size());
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        const JComp& c = comps[ci];
        const size_t stride = (size_t)c.bw * 8;
        const int cw = (W * c.h + hmax - 1) / hmax, ch = (H * c.v + vmax - 1) / vmax;
        const std::vector<uint8_t>& in = plane[ci];
        std::vector<uint8_t>& o = full[ci];
        o.assign((size_t)W * H, 0);
        const bool h2 = hmax == 2 * c.h, v1 = vmax == c.v, v2 = vmax == 2 * c.v;
        if (c.h == hmax && c.v == vmax) {
            for (int y = 0; y < H; ++y) memcpy(&o[(size_t)y * W], &in[(size_t)y * stride], (size_t)W);
        } else if (h2 && (v1 || v2) && cw >= 2) {
            std::vector<int> row(2 * (size_t)cw);
            for (int y = 0; y < H; ++y) {
                if (v1) {
                    const uint8_t* r = &in[(size_t)y * stride];
                    row[0] = r[0];
                    row[1] = (r[0] * 3 + r[1] + 2) >> 2;
                    for (int x = 1; x < cw - 1; ++x) {
                        row[2 * x] = (r[x] * 3 + r[x - 1] + 1) >> 2;
                        row[2 * x + 1] = (r[x] * 3 + r[x + 1] + 2) >> 2;
                    }
                    row[2 * cw - 2] = (r[cw - 1] * 3 + r[cw - 2] + 1) >> 2;
                    row[2 * cw - 1] = r[cw - 1];
                } else {
                    // the nearer input row counts three times, the other once
                    const int yc = y / 2, yo = (y & 1) ? std::min(yc + 1, ch - 1) : std::max(yc - 1, 0);
                    const uint8_t* r0 = &in[(size_t)yc * stride];
                    const uint8_t* r1 = &in[(size_t)yo * stride];
                    int last = 0, cur = r0[0] * 3 + r1[0], next = r0[1] * 3 + r1[1];
                    row[0] = (cur * 4 + 8) >> 4;
                    row[1] = (cur * 3 + next + 7) >> 4;
                    last = cur;
                    cur = next;
                    for (int x = 1; x < cw - 1; ++x) {
                        next = r0[x + 1] * 3 + r1[x + 1];
                        row[2 * x] = (cur * 3 + last + 8) >> 4;
                        row[2 * x + 1] = (cur * 3 + next + 7) >> 4;
                        last = cur;
                        cur = next;
                    }
                    row[2 * cw - 2] = (cur * 3 + last + 8) >> 4;
                    row[2 * cw - 1] = (cur * 4 + 7) >> 4;
                }
                for (int x = 0; x < W; ++x) o[(size_t)y * W + x] = (uint8_t)row[(size_t)x];
            }
        } else {
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x)
                    o[(size_t)y * W + x] = in[(size_t)(y * c.v / vmax) * stride + (size_t)(x * c.h / hmax)];
        }
    }
    out.w = (uint32_t)W;
    out.h = (uint32_t)H;
    out.depth = 8;
    out.channels = comps.size() == 1 ? 1 : 3;
    out.v.assign((size_t)W * H * out.channels, 0);
    const bool rgb_ids = comps.size() == 3 && comps[0].id == 'R' && comps[1].id == 'G' && comps[2].id == 'B';
    const bool ycc = comps.size() == 3 ? (adobe >= 0 ? adobe != 0 : !rgb_ids) : adobe == 2;
    const auto clamp8 = [](float v) { return (uint16_t)(v < 0.0f ? 0.0f : v > 255.0f ? 255.0f : std::floor(v + 0.5f)); };
    for (size_t i = 0; i < (size_t)W * H; ++i) {
        if (comps.size() == 1) {
            out.v[i] = full[0][i];
            continue;
        }
        uint16_t r = full[0][i], g = full[1][i], b = full[2][i];
        if (ycc) {
            const float y = full[0][i], cb = (float)full[1][i] - 128.0f, cr = (float)full[2][i] - 128.0f;
            r = clamp8(y + 1.402f * cr);
            g = clamp8(y - 0.344136f * cb - 0.714136f * cr);
            b = clamp8(y + 1.772f * cb);
        }
        if (comps.size() == 4) {  // Adobe CMYK is stored inverted: ink-free = 255
            const uint32_t k = full[3][i];
            r = (uint16_t)((r * k + 127) / 255);
            g = (uint16_t)((g * k + 127) / 255);
            b = (uint16_t)((b * k + 127) / 255);
        }
        out.v[i * 3] = r;
        out.v[i * 3 + 1] = g;
        out.v[i * 3 + 2] = b;
    }
    return true;
}

// glTF texture image (PNG or JPEG) -> RGBA8 by the importer's conversion of
// the decoded format (world.rs:949-1011): grey -> (l, l, l, 255); grey +
// alpha (two channels) -> (l, a, 0, 255); RGB -> (r, g, b, 255); 16-bit
// samples keep their high byte.
bool decode_texture(const uint8_t* d, size_t n, std::vector<uint8_t>& rgba, uint32_t& w, uint32_t& h, std::string& err,
                    uint32_t max_side) {
    Raster r;
    if (n >= 8 && d[0] == 0x89 && d[1] == 'P') {
        if (!decode_png(d, n, r, err, max_side)) return false;
    } else if (n >= 2 && d[0] == 0xff && d[1] == 0xd8) {
        if (!decode_jpeg(d, n, r, err, max_side)) return false;
    } else {
        err = "unsupported image encoding (PNG and JPEG are read)";
        return false;
    }
    w = r.w;
    h = r.h;
    rgba.assign((size_t)w * h * 4, 0);
    const int shift = r.depth == 16 ? 8 : 0;
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        const uint16_t* s = &r.v[i * r.channels];
        uint8_t* o = &rgba[i * 4];
        switch (r.channels) {
            case 1: o[0] = o[1] = o[2] = (uint8_t)(s[0] >> shift); o[3] = 255; break;
            case 2: o[0] = (uint8_t)(s[0] >> shift); o[1] = (uint8_t)(s[1] >> shift); o[2] = 0; o[3] = 255; break;
            case 3: for (int k = 0; k < 3; ++k) o[k] = (uint8_t)(s[k] >> shift); o[3] = 255; break;
            default: for (int k = 0; k < 4; ++k) o[k] = (uint8_t)(s[k] >> shift); break;
        }
    }
    return true;
}

// an 8- or 16-bit raster to RGBA32F as the image library's conversion does:
// samples divided by their maximum, grey replicated to RGB, alpha 1 if absent
void raster_to_rgba32f(const Raster& r, std::vector<float>& rgba) {
    const float inv = 1.0f / (r.depth == 16 ? 65535.0f : 255.0f);
    rgba.assign((size_t)r.w * r.h * 4, 1.0f);
    for (size_t i = 0; i < (size_t)r.w * r.h; ++i) {
        const uint16_t* s = &r.v[i * r.channels];
        float* o = &rgba[i * 4];
        if (r.channels <= 2) {
            o[0] = o[1] = o[2] = s[0] * inv;
            if (r.channels == 2) o[3] = s[1] * inv;
        } else {
            for (int k = 0; k < r.channels; ++k) o[k] = s[k] * inv;
        }
    }
}

bool decode_image(const std::vector<uint8_t>& data, std::vector<float>& rgba, uint32_t& w, uint32_t& h,
                  std::string& err, bool size_only = false) {
    if (data.size() >= 4 && data[0] == 0x76 && data[1] == 0x2f && data[2] == 0x31 && data[3] == 0x01)
        return read_exr(data, rgba, w, h, err, size_only);
    const bool png = data.size() >= 8 && data[0] == 0x89 && data[1] == 'P' && data[2] == 'N' && data[3] == 'G';
    const bool jpeg = data.size() >= 2 && data[0] == 0xff && data[1] == 0xd8;
    if (png || jpeg) {  // low dynamic range skyboxes
        Raster r;
        constexpr uint32_t kMaxSide = 65536;
        if (!(png ? decode_png(data.data(), data.size(), r, err, kMaxSide)
                  : decode_jpeg(data.data(), data.size(), r, err, kMaxSide)))
            return false;
        w = r.w;
        h = r.h;
        if ((uint64_t)w * h > (uint64_t)kMaxSkyPixels) {
            err = "image too large";
            return false;
        }
        if (!size_only) raster_to_rgba32f(r, rgba);
        return true;
    }
    return read_hdr(data, rgba, w, h, err, size_only);
}

bool read_image(const char* path, std::vector<float>& rgba, uint32_t& w, uint32_t& h, std::string& err,
                bool size_only = false) {
    std::vector<uint8_t> data;
    if (!read_file(path, data, err)) return false;
    return decode_image(data, rgba, w, h, err, size_only);
}

// the message, with every byte outside printable ASCII (an echo of the file's
// own bytes) shown as '?', so that callers always receive plain text
void put_error(char* error, size_t size, const std::string& msg) {
    if (!error || !size) return;
    std::string clean(msg);
    for (char& c : clean)
        if ((unsigned char)c < 0x20 || (unsigned char)c > 0x7e) c = '?';
    snprintf(error, size, "%s", clean.c_str());
}

}  // namespace

namespace ptimg {
bool decode_texture_rgba8(const uint8_t* bytes, size_t size, std::vector<uint8_t>& rgba, uint32_t& width,
                          uint32_t& height, std::string& error, uint32_t max_side) {
    return decode_texture(bytes, size, rgba, width, height, error, max_side);
}
}  // namespace ptimg

extern "C" int ptw_read_image_rgba(const char* path, float* rgba, uint64_t capacity, uint32_t* width, uint32_t* height,
                                   char* error, size_t error_size) try {
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
} catch (const std::bad_alloc&) {
    put_error(error, error_size, "out of host memory");
    return PT_ERR_OOM;
}

extern "C" int ptw_set_skybox_file(ptw_world* world, const char* path, char* error, size_t error_size) try {
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
} catch (const std::bad_alloc&) {
    put_error(error, error_size, "out of host memory");
    return PT_ERR_OOM;
}

extern "C" int ptw_set_skybox_bytes(ptw_world* world, const void* bytes, size_t size, char* error,
                                    size_t error_size) try {
    if (!world || !bytes) return PT_ERR_INVALID_ARG;
    const std::vector<uint8_t> data((const uint8_t*)bytes, (const uint8_t*)bytes + size);
    std::vector<float> px;
    uint32_t w = 0, h = 0;
    std::string err;
    if (!decode_image(data, px, w, h, err)) {
        put_error(error, error_size, err);
        return PT_ERR_INVALID_ARG;
    }
    const int rc = ptw_set_skybox_rgba(world, px.data(), w, h);
    if (rc) put_error(error, error_size, ptw_last_error(world));
    return rc;
} catch (const std::bad_alloc&) {
    put_error(error, error_size, "out of host memory");
    return PT_ERR_OOM;
}

extern "C" int ptw_decode_texture_rgba8(const void* bytes, size_t size, uint8_t* rgba, uint64_t capacity,
                                        uint32_t* width, uint32_t* height, char* error, size_t error_size) try {
    if (!bytes || !width || !height) return PT_ERR_INVALID_ARG;
    std::vector<uint8_t> px;
    uint32_t w = 0, h = 0;
    std::string err;
    if (!decode_texture((const uint8_t*)bytes, size, px, w, h, err, PT_ATLAS_SIZE)) {
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
    memcpy(rgba, px.data(), px.size());
    return PT_OK;
} catch (const std::bad_alloc&) {
    put_error(error, error_size, "out of host memory");
    return PT_ERR_OOM;
}
