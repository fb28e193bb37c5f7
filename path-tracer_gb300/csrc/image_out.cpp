// image_out.cpp - the headless renderer's output images: PNG, JPEG and
// lossless WebP (the formats the reference's `render --output` accepts,
// headless.rs:30,118-126, saved there through an image library) and PPM.
//
//   PNG: 8-bit RGB, a filter chosen per row (the one with the smallest sum
//        of absolute filtered bytes), zlib stream of LZ77 matches (hash
//        chains over a 32 KiB window) in fixed-Huffman DEFLATE blocks.
//   JPEG: baseline JFIF, 4:2:0 chroma, the example quantisation tables of
//        ITU-T T.81 Annex K scaled to a quality (75, as the image library's
//        default), per-image optimal Huffman tables limited to 16 bits by
//        the Annex K.2 procedure, float DCT.
//   WebP: VP8L lossless, no transforms, one prefix-code group, every pixel
//        a literal (green, red, blue, alpha codes).
#include <algorithm>
#include <array>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <queue>
#include <string>
#include <vector>

#include "../../include/pt_world.h"

namespace {

// LSB-first bit writer (DEFLATE, VP8L)
struct LsbBits {
    std::vector<uint8_t> out;
    uint64_t acc = 0;
    int n = 0;
    void put(uint32_t v, int bits) {
        acc |= (uint64_t)v << n;
        n += bits;
        while (n >= 8) {
            out.push_back((uint8_t)acc);
            acc >>= 8;
            n -= 8;
        }
    }
    // a Huffman code is sent most significant bit first
    void put_code(uint32_t code, int len) {
        uint32_t r = 0;
        for (int i = 0; i < len; ++i) r |= ((code >> i) & 1u) << (len - 1 - i);
        put(r, len);
    }
    void flush() {
        if (n > 0) out.push_back((uint8_t)acc);
        acc = 0;
        n = 0;
    }
};

// ------------------------------------------------------------------ DEFLATE
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                                6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void fixed_literal(LsbBits& b, uint32_t sym) {
    if (sym < 144)
        b.put_code(0x30 + sym, 8);
    else if (sym < 256)
        b.put_code(0x190 + sym - 144, 9);
    else if (sym < 280)
        b.put_code(sym - 256, 7);
    else
        b.put_code(0xC0 + sym - 280, 8);
}

// zlib stream: LZ77 over hash chains, fixed Huffman blocks
std::vector<uint8_t> zlib_compress(const std::vector<uint8_t>& in) {
    constexpr uint32_t kWindow = 32768, kHashBits = 15, kMaxChain = 64;
    LsbBits b;
    b.out = {0x78, 0x9c};
    std::vector<int32_t> head((size_t)1 << kHashBits, -1), prev(kWindow, -1);
    const size_t n = in.size();
    const auto hash = [&](size_t i) {
        return (((uint32_t)in[i] << 16) ^ ((uint32_t)in[i + 1] << 8) ^ in[i + 2]) * 2654435761u >> (32 - kHashBits);
    };
    size_t i = 0;
    bool first = true;
    // blocks of at most 1 MiB input, so one block's bits stay bounded
    while (i < n || first) {
        const size_t end = std::min(n, i + ((size_t)1 << 20));
        b.put(end == n ? 1u : 0u, 1);  // BFINAL
        b.put(1u, 2);                   // fixed Huffman
        first = false;
        while (i < end) {
            uint32_t best_len = 0, best_dist = 0;
            if (i + 3 <= n) {
                const uint32_t h = hash(i);
                int32_t cand = head[h];
                for (uint32_t chain = 0; cand >= 0 && chain < kMaxChain; ++chain) {
                    const size_t dist = i - (size_t)cand;
                    if (dist > kWindow - 1) break;
                    uint32_t len = 0;
                    const size_t max_len = std::min<size_t>(258, end - i);
                    while (len < max_len && in[(size_t)cand + len] == in[i + len]) ++len;
                    if (len > best_len) {
                        best_len = len;
                        best_dist = (uint32_t)dist;
                        if (len == max_len) break;
                    }
                    cand = prev[(size_t)cand % kWindow];
                }
            }
            const size_t step = best_len >= 3 ? best_len : 1;
            if (best_len >= 3) {
                int li = 28;
                while (kLenBase[li] > best_len) --li;
                fixed_literal(b, 257 + (uint32_t)li);
                b.put(best_len - kLenBase[li], kLenExtra[li]);
                int di = 29;
                while (kDistBase[di] > best_dist) --di;
                b.put_code((uint32_t)di, 5);
                b.put(best_dist - kDistBase[di], kDistExtra[di]);
            } else {
                fixed_literal(b, in[i]);
            }
            for (size_t k = 0; k < step; ++k, ++i)
                if (i + 3 <= n) {
                    const uint32_t h = hash(i);
                    prev[i % kWindow] = head[h];
                    head[h] = (int32_t)i;
                }
        }
        fixed_literal(b, 256);  // end of block
    }
    b.flush();
    uint32_t a = 1, s = 0;
    for (uint8_t v : in) {
        a = (a + v) % 65521;
        s = (s + a) % 65521;
    }
    const uint32_t adler = (s << 16) | a;
    for (int sh = 24; sh >= 0; sh -= 8) b.out.push_back((uint8_t)(adler >> sh));
    return b.out;
}

uint32_t crc32(const uint8_t* d, size_t n) {
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

void be32(std::vector<uint8_t>& o, uint32_t v) {
    for (int s = 24; s >= 0; s -= 8) o.push_back((uint8_t)(v >> s));
}

std::vector<uint8_t> png_bytes(const uint8_t* rgb, uint32_t w, uint32_t h) {
    const size_t row = (size_t)w * 3;
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (row + 1));
    std::vector<uint8_t> cand(row), best(row);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* cur = rgb + (size_t)y * row;
        const uint8_t* up = y ? cur - row : nullptr;
        long best_cost = -1;
        uint8_t best_f = 0;
        for (uint8_t f = 0; f < 5; ++f) {
            long cost = 0;
            for (size_t i = 0; i < row; ++i) {
                const int a = i >= 3 ? cur[i - 3] : 0, bb = up ? up[i] : 0, c = (up && i >= 3) ? up[i - 3] : 0;
                int p;
                switch (f) {
                    case 0: p = 0; break;
                    case 1: p = a; break;
                    case 2: p = bb; break;
                    case 3: p = (a + bb) >> 1; break;
                    default: {
                        const int pp = a + bb - c, pa = std::abs(pp - a), pb = std::abs(pp - bb), pc = std::abs(pp - c);
                        p = (pa <= pb && pa <= pc) ? a : (pb <= pc ? bb : c);
                    }
                }
                cand[i] = (uint8_t)(cur[i] - p);
                cost += std::abs((int)(int8_t)cand[i]);
            }
            if (best_cost < 0 || cost < best_cost) {
                best_cost = cost;
                best_f = f;
                best.swap(cand);
            }
        }
        raw.push_back(best_f);
        raw.insert(raw.end(), best.begin(), best.end());
    }
    std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    const auto chunk = [&](const char* type, const std::vector<uint8_t>& d) {
        be32(out, (uint32_t)d.size());
        const size_t at = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), d.begin(), d.end());
        be32(out, crc32(&out[at], d.size() + 4));
    };
    std::vector<uint8_t> ihdr;
    be32(ihdr, w);
    be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
    chunk("IHDR", ihdr);
    chunk("IDAT", zlib_compress(raw));
    chunk("IEND", {});
    return out;
}

// ------------------------------------------------------------------ Huffman code lengths
// lengths of an optimal prefix code for `freq`, limited to `max_len` bits:
// Huffman's construction, then the length-limiting adjustment of ITU-T T.81
// Annex K.2 (a code point is reserved when `reserve` so no code is all ones)
std::vector<uint8_t> code_lengths(const std::vector<uint64_t>& freq, int max_len, bool reserve) {
    const size_t n = freq.size();
    std::vector<uint8_t> len(n, 0);
    std::vector<size_t> used;
    for (size_t i = 0; i < n; ++i)
        if (freq[i]) used.push_back(i);
    if (used.empty()) return len;
    const size_t m = used.size() + (reserve ? 1 : 0);
    if (m == 1) {
        len[used[0]] = 1;
        return len;
    }
    // tree over leaves 0..m-1 (m-1: the reserved one)
    using Node = std::pair<uint64_t, int>;
    std::priority_queue<Node, std::vector<Node>, std::greater<Node>> pq;
    std::vector<int> parent(2 * m, -1);
    for (size_t k = 0; k < m; ++k) pq.push({k < used.size() ? freq[used[k]] : 1, (int)k});
    int next = (int)m;
    while (pq.size() > 1) {
        const Node x = pq.top();
        pq.pop();
        const Node y = pq.top();
        pq.pop();
        parent[(size_t)x.second] = next;
        parent[(size_t)y.second] = next;
        pq.push({x.first + y.first, next++});
    }
    std::vector<int> depth(m);
    std::vector<int> bits(64, 0);
    for (size_t k = 0; k < m; ++k) {
        int d = 0;
        for (int p = (int)k; parent[(size_t)p] >= 0; p = parent[(size_t)p]) ++d;
        depth[k] = d;
        bits[(size_t)d] += 1;
    }
    // Annex K.2: move codes longer than max_len up the tree
    for (int i = 63; i > max_len; --i)
        while (bits[(size_t)i] > 0) {
            int j = i - 2;
            while (bits[(size_t)j] == 0) --j;
            bits[(size_t)i] -= 2;
            bits[(size_t)i - 1] += 1;
            bits[(size_t)j + 1] += 2;
            bits[(size_t)j] -= 1;
        }
    if (reserve) {  // drop the reserved code point: the longest code
        int i = max_len;
        while (bits[(size_t)i] == 0) --i;
        bits[(size_t)i] -= 1;
    }
    // assign lengths: more frequent symbols get shorter codes
    std::vector<size_t> order = used;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return freq[a] > freq[b]; });
    size_t k = 0;
    for (int l = 1; l <= max_len; ++l)
        for (int c = 0; c < bits[(size_t)l]; ++c) len[order[k++]] = (uint8_t)l;
    return len;
}

// canonical codes from lengths (shorter codes first, then by symbol)
std::vector<uint32_t> canonical(const std::vector<uint8_t>& len) {
    int max_len = 0;
    for (uint8_t l : len) max_len = std::max<int>(max_len, l);
    std::vector<uint32_t> count((size_t)max_len + 1, 0), next((size_t)max_len + 2, 0), code(len.size(), 0);
    for (uint8_t l : len)
        if (l) count[l] += 1;
    uint32_t c = 0;
    for (int l = 1; l <= max_len; ++l) {
        c = (c + count[(size_t)l - 1]) << 1;
        next[(size_t)l] = c;
    }
    for (size_t s = 0; s < len.size(); ++s)
        if (len[s]) code[s] = next[len[s]]++;
    return code;
}

// ------------------------------------------------------------------ JPEG
const uint8_t kZig[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
                          41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
                          30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
// ITU-T T.81 Annex K, tables K.1 and K.2 (natural order)
const uint8_t kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kChromaQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                              24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

struct MsbBits {  // JPEG entropy-coded segment: MSB first, 0xFF stuffed
    std::vector<uint8_t>* out;
    uint32_t acc = 0;
    int n = 0;
    void put(uint32_t v, int bits) {
        for (int i = bits - 1; i >= 0; --i) {
            acc = (acc << 1) | ((v >> i) & 1u);
            if (++n == 8) {
                out->push_back((uint8_t)acc);
                if (acc == 0xff) out->push_back(0);
                acc = 0;
                n = 0;
            }
        }
    }
    void flush() {
        while (n) put(1, 1);
    }
};

int category(int v) {
    int a = std::abs(v), c = 0;
    while (a) {
        ++c;
        a >>= 1;
    }
    return c;
}

std::vector<uint8_t> jpeg_bytes(const uint8_t* rgb, uint32_t w, uint32_t h, int quality) {
    quality = std::min(100, std::max(1, quality));
    const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
    uint16_t q[2][64];
    for (int i = 0; i < 64; ++i) {
        q[0][i] = (uint16_t)std::min(255, std::max(1, (kLumaQ[i] * scale + 50) / 100));
        q[1][i] = (uint16_t)std::min(255, std::max(1, (kChromaQ[i] * scale + 50) / 100));
    }
    const uint32_t mw = (w + 15) / 16, mh = (h + 15) / 16;  // 16x16 MCUs
    // planes padded to whole MCUs by edge replication
    const uint32_t pw = mw * 16, ph = mh * 16, cw = pw / 2, ch = ph / 2;
    std::vector<float> Y((size_t)pw * ph), Cb((size_t)cw * ch), Cr((size_t)cw * ch);
    for (uint32_t y = 0; y < ph; ++y)
        for (uint32_t x = 0; x < pw; ++x) {
            const uint8_t* p = rgb + ((size_t)std::min(y, h - 1) * w + std::min(x, w - 1)) * 3;
            Y[(size_t)y * pw + x] = 0.299f * p[0] + 0.587f * p[1] + 0.114f * p[2] - 128.0f;
        }
    for (uint32_t y = 0; y < ch; ++y)
        for (uint32_t x = 0; x < cw; ++x) {
            float cb = 0, cr = 0;
            for (uint32_t dy = 0; dy < 2; ++dy)
                for (uint32_t dx = 0; dx < 2; ++dx) {
                    const uint8_t* p = rgb + ((size_t)std::min(2 * y + dy, h - 1) * w + std::min(2 * x + dx, w - 1)) * 3;
                    cb += -0.168736f * p[0] - 0.331264f * p[1] + 0.5f * p[2];
                    cr += 0.5f * p[0] - 0.418688f * p[1] - 0.081312f * p[2];
                }
            Cb[(size_t)y * cw + x] = cb * 0.25f;
            Cr[(size_t)y * cw + x] = cr * 0.25f;
        }
    static const std::array<float, 64> kCos = [] {
        std::array<float, 64> t{};
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                t[x * 8 + u] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * M_PI / 16.0) / 2.0);
        return t;
    }();
    // quantised coefficients of every block, in MCU order: Y Y Y Y Cb Cr
    struct Block {
        int c;  // 0 Y, 1 Cb, 2 Cr
        int16_t z[64];  // zigzag order
    };
    std::vector<Block> blocks;
    blocks.reserve((size_t)mw * mh * 6);
    const auto fdct = [&](const std::vector<float>& plane, uint32_t stride, uint32_t bx, uint32_t by, int comp) {
        float t[64], f[64];
        for (int y = 0; y < 8; ++y)
            for (int u = 0; u < 8; ++u) {
                float a = 0;
                for (int x = 0; x < 8; ++x) a += kCos[x * 8 + u] * plane[(size_t)(by + y) * stride + bx + x];
                t[y * 8 + u] = a;
            }
        for (int v = 0; v < 8; ++v)
            for (int u = 0; u < 8; ++u) {
                float a = 0;
                for (int y = 0; y < 8; ++y) a += kCos[y * 8 + v] * t[y * 8 + u];
                f[v * 8 + u] = a;
            }
        Block b;
        b.c = comp;
        const uint16_t* qt = q[comp == 0 ? 0 : 1];
        for (int k = 0; k < 64; ++k) b.z[k] = (int16_t)std::lround(f[kZig[k]] / (float)qt[kZig[k]]);
        blocks.push_back(b);
    };
    for (uint32_t my = 0; my < mh; ++my)
        for (uint32_t mx = 0; mx < mw; ++mx) {
            for (uint32_t k = 0; k < 4; ++k) fdct(Y, pw, mx * 16 + (k & 1) * 8, my * 16 + (k >> 1) * 8, 0);
            fdct(Cb, cw, mx * 8, my * 8, 1);
            fdct(Cr, cw, mx * 8, my * 8, 2);
        }
    // symbol statistics -> optimal tables (DC/AC x luma/chroma)
    std::vector<uint64_t> freq[4] = {std::vector<uint64_t>(12, 0), std::vector<uint64_t>(256, 0),
                                     std::vector<uint64_t>(12, 0), std::vector<uint64_t>(256, 0)};
    const auto walk = [&](auto&& emit) {
        int pred[3] = {0, 0, 0};
        for (const Block& b : blocks) {
            const int t = b.c == 0 ? 0 : 1;
            const int d = b.z[0] - pred[b.c];
            pred[b.c] = b.z[0];
            emit(2 * t, category(d), d, category(d));
            int r = 0;
            for (int k = 1; k < 64; ++k) {
                const int v = b.z[k];
                if (v == 0) {
                    ++r;
                    continue;
                }
                while (r > 15) {
                    emit(2 * t + 1, 0xF0, 0, 0);
                    r -= 16;
                }
                emit(2 * t + 1, (r << 4) | category(v), v, category(v));
                r = 0;
            }
            if (r) emit(2 * t + 1, 0x00, 0, 0);
        }
    };
    walk([&](int table, int sym, int, int) { freq[table][(size_t)sym] += 1; });
    std::vector<uint8_t> len[4];
    std::vector<uint32_t> code[4];
    for (int t = 0; t < 4; ++t) {
        len[t] = code_lengths(freq[t], 16, true);
        code[t] = canonical(len[t]);
    }
    std::vector<uint8_t> out = {0xFF, 0xD8};
    const auto seg = [&](uint8_t marker, const std::vector<uint8_t>& body) {
        out.push_back(0xFF);
        out.push_back(marker);
        out.push_back((uint8_t)((body.size() + 2) >> 8));
        out.push_back((uint8_t)(body.size() + 2));
        out.insert(out.end(), body.begin(), body.end());
    };
    seg(0xE0, {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0});
    for (int t = 0; t < 2; ++t) {
        std::vector<uint8_t> body = {(uint8_t)t};
        for (int k = 0; k < 64; ++k) body.push_back((uint8_t)q[t][kZig[k]]);
        seg(0xDB, body);
    }
    seg(0xC0, {8, (uint8_t)(h >> 8), (uint8_t)h, (uint8_t)(w >> 8), (uint8_t)w, 3, 1, 0x22, 0, 2, 0x11, 1, 3, 0x11, 1});
    for (int t = 0; t < 4; ++t) {
        std::vector<uint8_t> body = {(uint8_t)(((t & 1) << 4) | (t >> 1))};
        std::vector<std::pair<int, int>> syms;  // (length, symbol)
        for (size_t s = 0; s < len[t].size(); ++s)
            if (len[t][s]) syms.push_back({len[t][s], (int)s});
        std::sort(syms.begin(), syms.end());
        for (int l = 1; l <= 16; ++l)
            body.push_back((uint8_t)std::count_if(syms.begin(), syms.end(), [&](auto& p) { return p.first == l; }));
        for (auto& p : syms) body.push_back((uint8_t)p.second);
        seg(0xC4, body);
    }
    seg(0xDA, {3, 1, 0x00, 2, 0x11, 3, 0x11, 0, 63, 0});
    MsbBits bits{&out};
    walk([&](int table, int sym, int value, int nbits) {
        bits.put(code[table][(size_t)sym], len[table][(size_t)sym]);
        if (nbits) bits.put((uint32_t)(value >= 0 ? value : value + (1 << nbits) - 1), nbits);
    });
    bits.flush();
    out.push_back(0xFF);
    out.push_back(0xD9);
    return out;
}

// ------------------------------------------------------------------ WebP (VP8L)
void vp8l_code(LsbBits& b, const std::vector<uint64_t>& freq, std::vector<uint8_t>& len, std::vector<uint32_t>& code) {
    std::vector<size_t> used;
    for (size_t s = 0; s < freq.size(); ++s)
        if (freq[s]) used.push_back(s);
    len.assign(freq.size(), 0);
    code.assign(freq.size(), 0);
    if (used.size() <= 2 && (used.empty() || used.back() < 256)) {
        // simple code: one or two 8-bit symbols (one symbol: a zero-length code)
        b.put(1, 1);
        const size_t s0 = used.empty() ? 0 : used[0];
        b.put(used.size() == 2 ? 1u : 0u, 1);
        b.put(s0 < 2 ? 0u : 1u, 1);
        b.put((uint32_t)s0, s0 < 2 ? 1 : 8);
        if (used.size() == 2) {
            b.put((uint32_t)used[1], 8);
            len[s0] = len[used[1]] = 1;
            code[s0] = 0;
            code[used[1]] = 1;
        }
        return;
    }
    len = code_lengths(freq, 15, false);
    code = canonical(len);
    // the code lengths themselves: a code-length code over 0..15 (literal lengths; no run codes)
    std::vector<uint64_t> cl_freq(19, 0);
    for (uint8_t l : len) cl_freq[l] += 1;
    std::vector<uint8_t> cl_len = code_lengths(cl_freq, 7, false);
    size_t nonzero = 0;
    for (uint8_t l : cl_len) nonzero += l != 0;
    if (nonzero == 1)  // a single code-length symbol still needs a one-bit code
        for (size_t s = 0; s < 19; ++s)
            if (!cl_len[s]) {
                cl_len[s] = 1;
                for (size_t t = 0; t < 19; ++t)
                    if (cl_freq[t]) cl_len[t] = 1;
                break;
            }
    const std::vector<uint32_t> cl_code = canonical(cl_len);
    static const int kOrder[19] = {17, 18, 0, 1, 2, 3, 4, 5, 16, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15};
    int count = 19;
    while (count > 4 && cl_len[(size_t)kOrder[count - 1]] == 0) --count;
    b.put(0, 1);  // normal code
    b.put((uint32_t)(count - 4), 4);
    for (int i = 0; i < count; ++i) b.put(cl_len[(size_t)kOrder[i]], 3);
    b.put(0, 1);  // every symbol of the alphabet is coded
    for (uint8_t l : len) b.put_code(cl_code[l], cl_len[l]);
}

std::vector<uint8_t> webp_bytes(const uint8_t* rgb, uint32_t w, uint32_t h) {
    const size_t n = (size_t)w * h;
    std::vector<uint64_t> fg(256 + 24, 0), fr(256, 0), fb(256, 0), fa(256, 0), fd(40, 0);
    for (size_t i = 0; i < n; ++i) {
        fr[rgb[3 * i]] += 1;
        fg[rgb[3 * i + 1]] += 1;
        fb[rgb[3 * i + 2]] += 1;
    }
    fa[255] = n;
    LsbBits b;
    b.put(0x2f, 8);
    b.put(w - 1, 14);
    b.put(h - 1, 14);
    b.put(0, 1);  // no alpha in use
    b.put(0, 3);  // version 0
    b.put(0, 1);  // no transform
    b.put(0, 1);  // no colour cache
    b.put(0, 1);  // one prefix-code group
    std::vector<uint8_t> lg, lr, lb, la, ld;
    std::vector<uint32_t> cg, cr, cb, ca, cd;
    vp8l_code(b, fg, lg, cg);
    vp8l_code(b, fr, lr, cr);
    vp8l_code(b, fb, lb, cb);
    vp8l_code(b, fa, la, ca);
    vp8l_code(b, fd, ld, cd);
    for (size_t i = 0; i < n; ++i) {
        const uint8_t r = rgb[3 * i], g = rgb[3 * i + 1], bl = rgb[3 * i + 2];
        b.put_code(cg[g], lg[g]);
        b.put_code(cr[r], lr[r]);
        b.put_code(cb[bl], lb[bl]);
        b.put_code(ca[255], la[255]);
    }
    b.flush();
    std::vector<uint8_t> out = {'R', 'I', 'F', 'F', 0, 0, 0, 0, 'W', 'E', 'B', 'P', 'V', 'P', '8', 'L'};
    const auto le32 = [&](size_t at, uint32_t v) {
        for (int k = 0; k < 4; ++k) out[at + (size_t)k] = (uint8_t)(v >> (8 * k));
    };
    out.resize(out.size() + 4);
    le32(16, (uint32_t)b.out.size());
    out.insert(out.end(), b.out.begin(), b.out.end());
    if (b.out.size() & 1) out.push_back(0);
    le32(4, (uint32_t)(out.size() - 8));
    return out;
}

std::string extension(const std::string& path) {
    const size_t dot = path.rfind('.');
    std::string e = dot == std::string::npos ? "" : path.substr(dot + 1);
    for (char& c : e) c = (char)std::tolower((unsigned char)c);
    return e;
}

}  // namespace

extern "C" int ptw_write_image(const char* path, const uint8_t* rgb8, uint32_t width, uint32_t height, char* error,
                               size_t error_size) try {
    const auto fail = [&](int rc, const std::string& m) {
        if (error && error_size) snprintf(error, error_size, "%s", m.c_str());
        return rc;
    };
    if (!path || !rgb8 || width == 0 || height == 0) return fail(PT_ERR_INVALID_ARG, "path, pixels and a size are required");
    const std::string ext = extension(path);
    std::vector<uint8_t> data;
    if (ext == "png") {
        data = png_bytes(rgb8, width, height);
    } else if (ext == "jpg" || ext == "jpeg") {
        if (width > 65535 || height > 65535) return fail(PT_ERR_OUT_OF_LIMITS, "JPEG images are at most 65535 pixels on a side");
        data = jpeg_bytes(rgb8, width, height, 75);
    } else if (ext == "webp") {
        if (width > 16384 || height > 16384) return fail(PT_ERR_OUT_OF_LIMITS, "WebP images are at most 16384 pixels on a side");
        data = webp_bytes(rgb8, width, height);
    } else if (ext == "ppm") {
        const std::string hdr = "P6\n" + std::to_string(width) + " " + std::to_string(height) + "\n255\n";
        data.assign(hdr.begin(), hdr.end());
        data.insert(data.end(), rgb8, rgb8 + (size_t)width * height * 3);
    } else {
        return fail(PT_ERR_INVALID_ARG, "the output must have a .png, .jpg, .jpeg, .webp or .ppm extension");
    }
    FILE* f = fopen(path, "wb");
    if (!f) return fail(PT_ERR_INVALID_ARG, std::string("cannot save ") + path + ": " + strerror(errno));
    const bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
    if (fclose(f) != 0 || !ok) return fail(PT_ERR_INVALID_ARG, std::string("cannot save ") + path);
    return PT_OK;
} catch (const std::bad_alloc&) {
    if (error && error_size) snprintf(error, error_size, "out of host memory");
    return PT_ERR_OOM;
}
