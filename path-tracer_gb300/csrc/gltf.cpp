// gltf.cpp - glTF 2.0 scene import into the world builder (the reference's
// Scene::new glTF path, world.rs:1078-1337, materials world.rs:1992-2155).
//
// Reads .glb (binary container) and .gltf (JSON with external or base64
// buffers): the default scene's node tree (matrix or TRS transforms, walked
// with the same LIFO stack as the reference so triangles arrive in the same
// order), triangle primitives (POSITION, NORMAL, TANGENT, TEXCOORD_0,
// indices of any integer width, normalised integer texture coordinates) and
// materials (pbrMetallicRoughness, emissive factor and strength, IOR,
// KHR_materials_specular, alpha mode and cutoff, OpenPBR_* extras).  Per
// primitive the positions are transformed by the node matrix, normals by its
// inverse transpose and tangents by the matrix; ptw_add_mesh then applies
// the reference's normalisation and tangent rules.  Texture images (PNG or
// JPEG, from data URIs, files or buffer views) are decoded, converted to RGBA8
// by the reference's format rules and packed into 8192^2 sRGB or linear atlas
// layers (world.rs:890-1076); each material slot gets its layer and UV
// offset/scale in the atlas.
#include <algorithm>
#include <atomic>
#include <climits>
#include <exception>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/pt_world.h"

namespace ptimg {
bool decode_texture_rgba8(const uint8_t* bytes, size_t size, std::vector<uint8_t>& rgba, uint32_t& width,
                          uint32_t& height, std::string& error, uint32_t max_side);
}

namespace {

// ------------------------------------------------------------------ JSON
struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json* get(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    double number(const char* key, double dflt) const {
        const Json* j = get(key);
        return j && j->kind == Number ? j->num : dflt;
    }
    // a number member as an integer (truncated); NaN and values outside the
    // range of long become LONG_MIN, which every caller rejects as an index,
    // count, offset or length
    long integer(const char* key, long dflt) const {
        const Json* j = get(key);
        if (!j || j->kind != Number) return dflt;
        const double v = j->num;
        if (!(v > -9.2e18 && v < 9.2e18)) return LONG_MIN;
        return (long)v;
    }
    std::string string(const char* key, const char* dflt) const {
        const Json* j = get(key);
        return j && j->kind == String ? j->str : std::string(dflt);
    }
};

struct JsonParser {
    const char* p;
    const char* end;
    std::string error;
    int depth = 0;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const char* what) {
        if (error.empty()) error = what;
        return false;
    }
    bool parse(Json& out) {
        ws();
        if (p >= end) return fail("unexpected end of JSON");
        if (++depth > 256) return fail("JSON nested too deeply");
        bool ok;
        switch (*p) {
            case '{': ok = object(out); break;
            case '[': ok = array(out); break;
            case '"': out.kind = Json::String; ok = string(out.str); break;
            case 't': ok = literal("true", out, Json::Bool, true); break;
            case 'f': ok = literal("false", out, Json::Bool, false); break;
            case 'n': ok = literal("null", out, Json::Null, false); break;
            default: ok = number(out); break;
        }
        --depth;
        return ok;
    }
    bool literal(const char* word, Json& out, Json::Kind kind, bool value) {
        const size_t n = strlen(word);
        if ((size_t)(end - p) < n || strncmp(p, word, n) != 0) return fail("bad JSON literal");
        p += n;
        out.kind = kind;
        out.b = value;
        return true;
    }
    bool number(Json& out) {
        const char* s = p;
        if (p < end && (*p == '-' || *p == '+')) ++p;
        while (p < end && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '-' || *p == '+'))
            ++p;
        if (p == s) return fail("bad JSON value");
        out.kind = Json::Number;
        out.num = std::strtod(std::string(s, p).c_str(), nullptr);
        return true;
    }
    static void utf8(std::string& s, unsigned cp) {
        if (cp < 0x80) {
            s += (char)cp;
        } else if (cp < 0x800) {
            s += (char)(0xC0 | (cp >> 6));
            s += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            s += (char)(0xE0 | (cp >> 12));
            s += (char)(0x80 | ((cp >> 6) & 0x3F));
            s += (char)(0x80 | (cp & 0x3F));
        } else {
            s += (char)(0xF0 | (cp >> 18));
            s += (char)(0x80 | ((cp >> 12) & 0x3F));
            s += (char)(0x80 | ((cp >> 6) & 0x3F));
            s += (char)(0x80 | (cp & 0x3F));
        }
    }
    bool hex4(unsigned& v) {
        if (end - p < 4) return fail("bad JSON escape");
        v = 0;
        for (int i = 0; i < 4; ++i) {
            const char c = *p++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (unsigned)(c - 'A' + 10);
            else return fail("bad JSON escape");
        }
        return true;
    }
    bool string(std::string& s) {
        ++p;  // opening quote
        while (p < end && *p != '"') {
            if (*p == '\\') {
                ++p;
                if (p >= end) break;
                const char c = *p++;
                switch (c) {
                    case 'n': s += '\n'; break;
                    case 't': s += '\t'; break;
                    case 'r': s += '\r'; break;
                    case 'b': s += '\b'; break;
                    case 'f': s += '\f'; break;
                    case 'u': {
                        unsigned cp;
                        if (!hex4(cp)) return false;
                        if (cp >= 0xD800 && cp < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                            p += 2;
                            unsigned lo;
                            if (!hex4(lo)) return false;
                            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                        }
                        utf8(s, cp);
                        break;
                    }
                    default: s += c; break;
                }
            } else {
                s += *p++;
            }
        }
        if (p >= end) return fail("unterminated JSON string");
        ++p;
        return true;
    }
    bool array(Json& out) {
        out.kind = Json::Array;
        ++p;
        ws();
        if (p < end && *p == ']') {
            ++p;
            return true;
        }
        for (;;) {
            out.arr.emplace_back();
            if (!parse(out.arr.back())) return false;
            ws();
            if (p < end && *p == ',') {
                ++p;
                continue;
            }
            if (p < end && *p == ']') {
                ++p;
                return true;
            }
            return fail("expected , or ] in JSON array");
        }
    }
    bool object(Json& out) {
        out.kind = Json::Object;
        ++p;
        ws();
        if (p < end && *p == '}') {
            ++p;
            return true;
        }
        for (;;) {
            ws();
            if (p >= end || *p != '"') return fail("expected a key in JSON object");
            std::string key;
            if (!string(key)) return false;
            ws();
            if (p >= end || *p != ':') return fail("expected : in JSON object");
            ++p;
            out.obj.emplace_back(std::move(key), Json());
            if (!parse(out.obj.back().second)) return false;
            ws();
            if (p < end && *p == ',') {
                ++p;
                continue;
            }
            if (p < end && *p == '}') {
                ++p;
                return true;
            }
            return fail("expected , or } in JSON object");
        }
    }
};

// ------------------------------------------------------------------ math
struct M4 {
    float m[16];  // column-major: column c at m[4c .. 4c+3]
};
M4 identity() {
    M4 r{};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
}
// a * b, each result column = a.x * b.c.x + a.y * b.c.y + a.z * b.c.z + a.w * b.c.w
M4 mul(const M4& a, const M4& b) {
    M4 r;
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row)
            r.m[4 * c + row] = ((a.m[row] * b.m[4 * c] + a.m[4 + row] * b.m[4 * c + 1]) + a.m[8 + row] * b.m[4 * c + 2]) +
                               a.m[12 + row] * b.m[4 * c + 3];
    return r;
}
M4 from_trs(const float t[3], const float q[4], const float s[3]) {
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    const float x2 = x + x, y2 = y + y, z2 = z + z;
    const float xx = x * x2, xy = x * y2, xz = x * z2, yy = y * y2, yz = y * z2, zz = z * z2;
    const float wx = w * x2, wy = w * y2, wz = w * z2;
    M4 r{};
    // rotation columns scaled by s, translation in the last column
    const float c0[3] = {1.0f - (yy + zz), xy + wz, xz - wy};
    const float c1[3] = {xy - wz, 1.0f - (xx + zz), yz + wx};
    const float c2[3] = {xz + wy, yz - wx, 1.0f - (xx + yy)};
    for (int i = 0; i < 3; ++i) {
        r.m[i] = c0[i] * s[0];
        r.m[4 + i] = c1[i] * s[1];
        r.m[8 + i] = c2[i] * s[2];
        r.m[12 + i] = t[i];
    }
    r.m[15] = 1.0f;
    return r;
}
// inverse transpose of the upper 3x3 (normals), in double
void normal_matrix(const M4& a, double n[9]) {
    const double m00 = a.m[0], m10 = a.m[1], m20 = a.m[2];
    const double m01 = a.m[4], m11 = a.m[5], m21 = a.m[6];
    const double m02 = a.m[8], m12 = a.m[9], m22 = a.m[10];
    const double c00 = m11 * m22 - m12 * m21, c01 = m12 * m20 - m10 * m22, c02 = m10 * m21 - m11 * m20;
    const double det = m00 * c00 + m01 * c01 + m02 * c02;
    const double id = det != 0.0 ? 1.0 / det : 0.0;
    // inverse transpose = cofactor matrix / det (row-major here: n[3*row + col])
    n[0] = c00 * id;
    n[1] = c01 * id;
    n[2] = c02 * id;
    n[3] = (m02 * m21 - m01 * m22) * id;
    n[4] = (m00 * m22 - m02 * m20) * id;
    n[5] = (m01 * m20 - m00 * m21) * id;
    n[6] = (m01 * m12 - m02 * m11) * id;
    n[7] = (m02 * m10 - m00 * m12) * id;
    n[8] = (m00 * m11 - m01 * m10) * id;
}

// ------------------------------------------------------------------ glTF
// Guillotine packer for one atlas layer: a list of free rectangles; an image
// takes the free rectangle it fits with the shortest leftover side (ties: the
// shorter longer side), and the remainder is cut along its shorter leftover
// side into two free rectangles.
struct AtlasPacker {
    struct Rect {
        int x, y, w, h;
    };
    std::vector<Rect> free{{0, 0, (int)PT_ATLAS_SIZE, (int)PT_ATLAS_SIZE}};
    bool place(int w, int h, int& x, int& y) {
        long best = -1, best_short = LONG_MAX, best_long = LONG_MAX;
        for (size_t i = 0; i < free.size(); ++i) {
            const Rect& f = free[i];
            if (w > f.w || h > f.h) continue;
            const long a = f.w - w, b = f.h - h, sh = std::min(a, b), lo = std::max(a, b);
            if (sh < best_short || (sh == best_short && lo < best_long)) {
                best = (long)i;
                best_short = sh;
                best_long = lo;
            }
        }
        if (best < 0) return false;
        const Rect f = free[(size_t)best];
        free.erase(free.begin() + best);
        x = f.x;
        y = f.y;
        Rect right, below;
        if (f.w - w < f.h - h) {
            right = {f.x + w, f.y, f.w - w, h};
            below = {f.x, f.y + h, f.w, f.h - h};
        } else {
            right = {f.x + w, f.y, f.w - w, f.h};
            below = {f.x, f.y + h, w, f.h - h};
        }
        if (right.w > 0 && right.h > 0) free.push_back(right);
        if (below.w > 0 && below.h > 0) free.push_back(below);
        return true;
    }
};

struct AtlasSlot {
    int32_t layer = -1;
    float uv[4] = {0, 0, 0, 0};  // offset x, y, scale x, y
};

// largest accessor count accepted (elements): far beyond any scene this
// renderer holds, small enough that count x stride cannot overflow
constexpr long kMaxAccessorCount = 1L << 28;

// an array element used as a node index: -1 (rejected as out of range) unless
// it is a number within the range of long
inline long index_of(const Json& j) {
    if (j.kind != Json::Number || !(j.num > -9.2e18 && j.num < 9.2e18)) return -1;
    return (long)j.num;
}

// [offset, offset + length) lies within a buffer of `size` bytes (no overflow)
inline bool in_range(long offset, long length, size_t size) {
    return offset >= 0 && length >= 0 && (unsigned long)offset <= size && (unsigned long)length <= size - (unsigned long)offset;
}

struct Loader {
    ptw_world* world;
    std::string dir;
    Json doc;
    std::vector<std::vector<uint8_t>> buffers;
    std::map<long, uint32_t> material_cache;  // glTF material index -> world material
    std::map<long, AtlasSlot> srgb_slots, linear_slots;  // image index -> atlas placement
    std::string error;

    bool fail(const std::string& msg) {
        if (error.empty()) error = msg;
        return false;
    }

    static bool read_file(const std::string& path, std::vector<uint8_t>& out) {
        std::ifstream f(path, std::ios::binary);
        if (!f) return false;
        f.seekg(0, std::ios::end);
        const std::streamoff n = f.tellg();
        if (n < 0) return false;
        f.seekg(0);
        out.resize((size_t)n);
        if (n) f.read(reinterpret_cast<char*>(out.data()), n);
        return (bool)f;
    }

    static bool base64(const std::string& s, std::vector<uint8_t>& out) {
        auto val = [](char c) -> int {
            if (c >= 'A' && c <= 'Z') return c - 'A';
            if (c >= 'a' && c <= 'z') return c - 'a' + 26;
            if (c >= '0' && c <= '9') return c - '0' + 52;
            if (c == '+') return 62;
            if (c == '/') return 63;
            return -1;
        };
        uint32_t acc = 0;
        int bits = 0;
        for (char c : s) {
            if (c == '=') break;
            const int v = val(c);
            if (v < 0) return false;
            acc = (acc << 6) | (uint32_t)v;
            bits += 6;
            if (bits >= 8) {
                bits -= 8;
                out.push_back((uint8_t)((acc >> bits) & 0xFF));
            }
        }
        return true;
    }

    bool open(const std::string& path) {
        std::vector<uint8_t> file;
        if (!read_file(path, file)) return fail("cannot read " + path);
        const size_t slash = path.find_last_of('/');
        dir = slash == std::string::npos ? "" : path.substr(0, slash + 1);
        return open_bytes(file);
    }

    // a .glb container or .gltf JSON held in memory; relative URIs resolve against `dir`
    bool open_bytes(const std::vector<uint8_t>& file) {
        std::vector<uint8_t> bin;
        const char* json_begin;
        size_t json_size;
        if (file.size() >= 12 && memcmp(file.data(), "glTF", 4) == 0) {
            uint32_t version, length;
            memcpy(&version, file.data() + 4, 4);
            memcpy(&length, file.data() + 8, 4);
            if (version != 2) return fail("only glTF 2.0 binaries are supported");
            if (length > file.size()) return fail("truncated .glb");
            size_t off = 12;
            json_begin = nullptr;
            json_size = 0;
            while (off + 8 <= length) {
                uint32_t clen, ctype;
                memcpy(&clen, file.data() + off, 4);
                memcpy(&ctype, file.data() + off + 4, 4);
                off += 8;
                if (off + clen > length) return fail("truncated .glb chunk");
                if (ctype == 0x4E4F534Au && !json_begin) {  // "JSON"
                    json_begin = reinterpret_cast<const char*>(file.data() + off);
                    json_size = clen;
                } else if (ctype == 0x004E4942u && bin.empty()) {  // "BIN\0"
                    bin.assign(file.data() + off, file.data() + off + clen);
                }
                off += (clen + 3u) & ~3u;
            }
            if (!json_begin) return fail(".glb without a JSON chunk");
        } else {
            json_begin = reinterpret_cast<const char*>(file.data());
            json_size = file.size();
        }
        JsonParser jp{json_begin, json_begin + json_size, {}};
        if (!jp.parse(doc) || doc.kind != Json::Object) return fail("bad glTF JSON: " + jp.error);
        const Json* asset = doc.get("asset");
        if (!asset || asset->string("version", "").rfind("2", 0) != 0) return fail("not a glTF 2.0 asset");
        if (const Json* req = doc.get("extensionsRequired"))
            for (const Json& e : req->arr)
                if (e.str != "KHR_materials_emissive_strength" && e.str != "KHR_materials_ior" &&
                    e.str != "KHR_materials_specular")
                    return fail("required glTF extension not supported: " + e.str);
        if (const Json* bufs = doc.get("buffers")) {
            for (size_t i = 0; i < bufs->arr.size(); ++i) {
                const Json& b = bufs->arr[i];
                std::vector<uint8_t> data;
                const Json* uri = b.get("uri");
                if (!uri) {
                    if (i != 0 || bin.empty()) return fail("buffer without uri and no .glb BIN chunk");
                    data = bin;
                } else if (uri->str.rfind("data:", 0) == 0) {
                    const size_t comma = uri->str.find(',');
                    if (comma == std::string::npos || uri->str.find(";base64") == std::string::npos ||
                        !base64(uri->str.substr(comma + 1), data))
                        return fail("unsupported data URI in buffer " + std::to_string(i));
                } else if (!read_file(dir + uri->str, data)) {
                    return fail("cannot read buffer " + uri->str);
                }
                const long need = b.integer("byteLength", 0);
                if (need < 0 || (size_t)need > data.size()) return fail("buffer shorter than its byteLength");
                buffers.push_back(std::move(data));
            }
        }
        return true;
    }

    // one component of a float accessor; normalised integers map to [0, 1] / [-1, 1]
    static bool component(const uint8_t* e, long ctype, bool norm, float* out) {
        float v;
        switch (ctype) {
            case 5126: memcpy(&v, e, 4); break;
            case 5121: v = norm ? (float)e[0] / 255.0f : (float)e[0]; break;
            case 5120: {
                const int8_t s = (int8_t)e[0];
                v = norm ? std::fmax((float)s / 127.0f, -1.0f) : (float)s;
                break;
            }
            case 5123: {
                uint16_t u;
                memcpy(&u, e, 2);
                v = norm ? (float)u / 65535.0f : (float)u;
                break;
            }
            case 5122: {
                int16_t s;
                memcpy(&s, e, 2);
                v = norm ? std::fmax((float)s / 32767.0f, -1.0f) : (float)s;
                break;
            }
            case 5125: {
                uint32_t u;
                memcpy(&u, e, 4);
                v = (float)u;
                break;
            }
            default: return false;
        }
        *out = v;
        return true;
    }

    // the sparse substitution of accessor `a` (glTF 2.0 3.6.2.3): `count`
    // element indices (unsigned, strictly increasing) and their values
    // replace elements of the dense (or all-zero) data; `put(i, bytes)`
    // stores one element read from the values view
    template <class Put>
    bool sparse(const Json& a, size_t n, size_t elem, Put&& put) {
        const Json* sp = a.get("sparse");
        if (!sp) return true;
        const size_t cnt = (size_t)sp->integer("count", 0);
        const Json* ind = sp->get("indices");
        const Json* val = sp->get("values");
        if (!ind || !val || cnt == 0 || cnt > n) return fail("malformed sparse accessor");
        const long ict = ind->integer("componentType", 0);
        const size_t isz = ict == 5125 ? 4 : ict == 5123 ? 2 : ict == 5121 ? 1 : 0;
        if (!isz) return fail("sparse indices must be unsigned integers");
        const uint8_t *ib, *vb;
        size_t ist, iav, vst, vav;
        if (!view(ind->integer("bufferView", -1), ind->integer("byteOffset", 0), isz, &ib, &ist, &iav) ||
            !view(val->integer("bufferView", -1), val->integer("byteOffset", 0), elem, &vb, &vst, &vav))
            return false;
        if (cnt * isz > iav || cnt * elem > vav) return fail("sparse accessor runs past its buffer view");
        for (size_t k = 0; k < cnt; ++k) {
            uint32_t i = 0;
            if (isz == 4) memcpy(&i, ib + k * isz, 4);
            else if (isz == 2) {
                uint16_t u;
                memcpy(&u, ib + k * isz, 2);
                i = u;
            } else {
                i = ib[k];
            }
            if (i >= n) return fail("sparse index out of range");
            if (!put(i, vb + k * elem)) return fail("unsupported accessor component type");
        }
        return true;
    }

    // accessor i as float components (count x ncomp), normalised integers mapped to [0, 1] / [-1, 1]
    bool read_floats(long index, int want_comps, std::vector<float>& out, size_t* count) {
        const Json* accs = doc.get("accessors");
        if (!accs || index < 0 || (size_t)index >= accs->arr.size()) return fail("accessor out of range");
        const Json& a = accs->arr[(size_t)index];
        const std::string type = a.string("type", "");
        const int comps = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
        if (comps != want_comps) return fail("accessor has type " + type);
        const long ctype = a.integer("componentType", 0);
        const bool norm = a.get("normalized") && a.get("normalized")->b;
        const long cnt = a.integer("count", 0);
        if (cnt < 0 || cnt > kMaxAccessorCount) return fail("accessor count out of range");
        const size_t n = (size_t)cnt;
        const int csize = ctype == 5126 || ctype == 5125 ? 4 : ctype == 5123 || ctype == 5122 ? 2 : 1;
        *count = n;
        const size_t elem = (size_t)csize * comps;
        if (a.get("bufferView")) {  // else all zeros before the sparse substitution
            const uint8_t* base;
            size_t stride, avail;
            if (!view(a.integer("bufferView", -1), a.integer("byteOffset", 0), elem, &base, &stride, &avail))
                return false;
            if (n && (n - 1) * stride + elem > avail) return fail("accessor runs past its buffer view");
            out.assign(n * comps, 0.0f);
            for (size_t i = 0; i < n; ++i)
                for (int c = 0; c < comps; ++c)
                    if (!component(base + i * stride + (size_t)c * csize, ctype, norm, &out[i * comps + c]))
                        return fail("unsupported accessor component type");
        } else {
            out.assign(n * comps, 0.0f);
        }
        return sparse(a, n, elem, [&](uint32_t i, const uint8_t* e) {
            for (int c = 0; c < comps; ++c)
                if (!component(e + (size_t)c * csize, ctype, norm, &out[(size_t)i * comps + c])) return false;
            return true;
        });
    }

    bool read_indices(long index, std::vector<uint32_t>& out) {
        const Json* accs = doc.get("accessors");
        if (!accs || index < 0 || (size_t)index >= accs->arr.size()) return fail("accessor out of range");
        const Json& a = accs->arr[(size_t)index];
        const long ctype = a.integer("componentType", 0);
        const int csize = ctype == 5125 ? 4 : ctype == 5123 ? 2 : ctype == 5121 ? 1 : 0;
        if (!csize || a.string("type", "") != "SCALAR") return fail("index accessor must be unsigned SCALAR");
        const long cnt = a.integer("count", 0);
        if (cnt < 0 || cnt > kMaxAccessorCount) return fail("index accessor count out of range");
        const size_t n = (size_t)cnt;
        const auto get = [&](const uint8_t* e) -> uint32_t {
            if (csize == 4) {
                uint32_t u;
                memcpy(&u, e, 4);
                return u;
            }
            if (csize == 2) {
                uint16_t u;
                memcpy(&u, e, 2);
                return u;
            }
            return e[0];
        };
        if (a.get("bufferView")) {
            const uint8_t* base;
            size_t stride, avail;
            if (!view(a.integer("bufferView", -1), a.integer("byteOffset", 0), (size_t)csize, &base, &stride, &avail))
                return false;
            if (n && (n - 1) * stride + (size_t)csize > avail) return fail("index accessor runs past its buffer view");
            out.assign(n, 0u);
            for (size_t i = 0; i < n; ++i) out[i] = get(base + i * stride);
        } else {
            out.assign(n, 0u);
        }
        return sparse(a, n, (size_t)csize, [&](uint32_t i, const uint8_t* e) {
            out[i] = get(e);
            return true;
        });
    }

    bool view(long index, long offset, size_t elem, const uint8_t** base, size_t* stride, size_t* avail) {
        const Json* views = doc.get("bufferViews");
        if (!views || index < 0 || (size_t)index >= views->arr.size()) return fail("buffer view out of range");
        const Json& v = views->arr[(size_t)index];
        const long b = v.integer("buffer", -1);
        if (b < 0 || (size_t)b >= buffers.size()) return fail("buffer out of range");
        const long voff = v.integer("byteOffset", 0), vlen = v.integer("byteLength", 0);
        if (!in_range(voff, vlen, buffers[(size_t)b].size()) || offset < 0 || offset > vlen)
            return fail("buffer view out of range");
        *base = buffers[(size_t)b].data() + voff + offset;
        const long st = v.integer("byteStride", 0);
        // glTF 2.0 3.6.2.4: a stride is a multiple of 4 in [4, 252]
        if (v.get("byteStride") && (st < 4 || st > 252 || st % 4 != 0)) return fail("invalid buffer view byteStride");
        *stride = st > 0 ? (size_t)st : elem;
        *avail = (size_t)(vlen - offset);
        return true;
    }

    bool has_texture(const Json* t) const { return t && t->kind == Json::Object; }

    // textureInfo -> textures[index].source (the image index), -1 without one
    long texture_image(const Json* info) const {
        if (!has_texture(info)) return -1;
        const Json* textures = doc.get("textures");
        const long ti = info->integer("index", -1);
        if (!textures || ti < 0 || (size_t)ti >= textures->arr.size()) return -1;
        return textures->arr[(size_t)ti].integer("source", -1);
    }

    // the encoded bytes of image i: a data URI, a file beside the glTF, or a buffer view
    bool image_bytes(size_t i, std::vector<uint8_t>& out) {
        const Json& im = doc.get("images")->arr[i];
        if (const Json* uri = im.get("uri")) {
            if (uri->str.rfind("data:", 0) == 0) {
                const size_t comma = uri->str.find(',');
                if (comma == std::string::npos || uri->str.find(";base64") == std::string::npos ||
                    !base64(uri->str.substr(comma + 1), out))
                    return fail("unsupported data URI in image " + std::to_string(i));
                return true;
            }
            if (!read_file(dir + uri->str, out)) return fail("cannot read image " + uri->str);
            return true;
        }
        const Json* views = doc.get("bufferViews");
        const long vi = im.integer("bufferView", -1);
        if (!views || vi < 0 || (size_t)vi >= views->arr.size()) return fail("image without uri or buffer view");
        const Json& v = views->arr[(size_t)vi];
        const long b = v.integer("buffer", -1), off = v.integer("byteOffset", 0), len = v.integer("byteLength", 0);
        if (b < 0 || (size_t)b >= buffers.size() || !in_range(off, len, buffers[(size_t)b].size()))
            return fail("image buffer view out of range");
        out.assign(buffers[(size_t)b].begin() + off, buffers[(size_t)b].begin() + off + len);
        return true;
    }

    // world.rs:893-1076: every image of the file decoded to RGBA8 and packed,
    // in image order, into sRGB atlas layers if any material uses it as a base
    // colour, emission or specular colour texture, else into linear layers;
    // a new layer is opened when an image fits in none of the open ones
    bool images() {
        const Json* imgs = doc.get("images");
        if (!imgs || imgs->arr.empty()) return true;
        std::set<long> srgb;
        if (const Json* mats = doc.get("materials"))
            for (const Json& m : mats->arr) {
                if (const Json* pbr = m.get("pbrMetallicRoughness")) srgb.insert(texture_image(pbr->get("baseColorTexture")));
                srgb.insert(texture_image(m.get("emissiveTexture")));
                if (const Json* ext = m.get("extensions"))
                    if (const Json* sp = ext->get("KHR_materials_specular"))
                        srgb.insert(texture_image(sp->get("specularColorTexture")));
            }
        const size_t n = imgs->arr.size();
        std::vector<std::vector<uint8_t>> encoded(n), rgba(n);
        std::vector<uint32_t> w(n), h(n);
        for (size_t i = 0; i < n; ++i)
            if (!image_bytes(i, encoded[i])) return false;
        // decode in parallel; each image is independent
        std::vector<std::string> errs(n);
        std::atomic<size_t> next{0};
        const auto worker = [&]() {
            for (size_t i; (i = next.fetch_add(1)) < n;) {
                if (!ptimg::decode_texture_rgba8(encoded[i].data(), encoded[i].size(), rgba[i], w[i], h[i], errs[i],
                                                 PT_ATLAS_SIZE) && errs[i].empty())
                    errs[i] = "decode failed";
                std::vector<uint8_t>().swap(encoded[i]);
            }
        };
        const size_t nt = std::min<size_t>(n, std::max(1u, std::min(std::thread::hardware_concurrency(), 16u)));
        std::vector<std::thread> pool;
        for (size_t t = 1; t < nt; ++t) {
            try {
                pool.emplace_back(worker);
            } catch (const std::system_error&) {
                break;  // the calling thread's worker takes the remaining images
            }
        }
        worker();
        for (auto& t : pool) t.join();
        for (size_t i = 0; i < n; ++i)
            if (!errs[i].empty()) return fail("image " + std::to_string(i) + ": " + errs[i]);
        struct Layer {
            AtlasPacker packer;
            std::vector<uint8_t> pixels;
        };
        std::vector<Layer> layers[2];  // [0] linear, [1] sRGB
        std::vector<std::pair<int, AtlasSlot>> placed(n);
        const size_t layer_bytes = (size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
        for (size_t i = 0; i < n; ++i) {
            const int kind = srgb.count((long)i) ? 1 : 0;
            auto& ls = layers[kind];
            int x = 0, y = 0;
            size_t li = 0;
            while (li < ls.size() && !ls[li].packer.place((int)w[i], (int)h[i], x, y)) ++li;
            if (li == ls.size()) {
                ls.emplace_back();
                ls.back().pixels.assign(layer_bytes, 0);
                if (!ls.back().packer.place((int)w[i], (int)h[i], x, y))
                    return fail("image " + std::to_string(i) + " is larger than the atlas");
            }
            uint8_t* dst = ls[li].pixels.data();
            for (uint32_t r = 0; r < h[i]; ++r)
                memcpy(dst + (((size_t)(y + r) * PT_ATLAS_SIZE) + (size_t)x) * 4, rgba[i].data() + (size_t)r * w[i] * 4,
                       (size_t)w[i] * 4);
            std::vector<uint8_t>().swap(rgba[i]);
            AtlasSlot a;
            a.layer = (int32_t)li;
            a.uv[0] = (float)x / (float)PT_ATLAS_SIZE;
            a.uv[1] = (float)y / (float)PT_ATLAS_SIZE;
            a.uv[2] = (float)w[i] / (float)PT_ATLAS_SIZE;
            a.uv[3] = (float)h[i] / (float)PT_ATLAS_SIZE;
            placed[i] = {kind, a};
        }
        // hand the layers to the world; its layer indices may start after layers added earlier
        std::vector<int32_t> index[2];
        for (int kind = 0; kind < 2; ++kind)
            for (Layer& l : layers[kind]) {
                int32_t li = -1;
                if (ptw_add_atlas_layer(world, kind, l.pixels.data(), &li) != PT_OK) return fail(ptw_last_error(world));
                index[kind].push_back(li);
                std::vector<uint8_t>().swap(l.pixels);
            }
        for (size_t i = 0; i < n; ++i) {
            AtlasSlot a = placed[i].second;
            a.layer = index[placed[i].first][(size_t)a.layer];
            (placed[i].first ? srgb_slots : linear_slots)[(long)i] = a;
        }
        return true;
    }

    // GpuMaterial::new, world.rs:1992-2155
    bool material(const Json* m, uint32_t* out) {
        pt_material g;
        ptw_default_material(&g);
        const Json empty;
        const Json& mat = m ? *m : empty;
        const Json* pbr = mat.get("pbrMetallicRoughness");
        const Json& p = pbr ? *pbr : empty;
        // atlas layer and UV offset/scale of each texture slot; -1 and zeros without one
        const auto slot = [&](const Json* t, bool srgb, int32_t* layer, float* uv) {
            const long img = texture_image(t);
            const auto& slots = srgb ? srgb_slots : linear_slots;
            const auto it = img >= 0 ? slots.find(img) : slots.end();
            const AtlasSlot none;
            const AtlasSlot& a = it == slots.end() ? none : it->second;
            *layer = a.layer;
            for (int i = 0; i < 4; ++i) uv[i] = a.uv[i];
        };
        slot(p.get("baseColorTexture"), true, &g.base_color_tex_layer, g.base_color_uv);
        slot(p.get("metallicRoughnessTexture"), false, &g.metallic_roughness_tex_layer, g.metallic_roughness_uv);
        slot(mat.get("normalTexture"), false, &g.normal_tex_layer, g.normal_uv);
        slot(mat.get("emissiveTexture"), true, &g.emission_tex_layer, g.emission_uv);
        const Json* spec_ext = mat.get("extensions") ? mat.get("extensions")->get("KHR_materials_specular") : nullptr;
        slot(spec_ext ? spec_ext->get("specularTexture") : nullptr, false, &g.specular_weight_tex_layer,
             g.specular_weight_uv);
        slot(spec_ext ? spec_ext->get("specularColorTexture") : nullptr, true, &g.specular_color_tex_layer,
             g.specular_color_uv);
        const Json* bcf = p.get("baseColorFactor");
        for (int i = 0; i < 4; ++i)
            g.base_color[i] = bcf && bcf->arr.size() == 4 ? (float)bcf->arr[i].num : 1.0f;
        g.base_weight = 1.0f;
        g.base_metalness = (float)p.number("metallicFactor", 1.0);
        g.base_diffuse_roughness = (float)p.number("roughnessFactor", 1.0);
        g.emission_weight = 1.0f;
        const Json* ef = mat.get("emissiveFactor");
        for (int i = 0; i < 3; ++i)
            g.emission_color_and_luminance[i] = ef && ef->arr.size() == 3 ? (float)ef->arr[i].num : 0.0f;
        g.emission_color_and_luminance[3] = 1.0f;
        g.specular_color_and_weight[0] = g.specular_color_and_weight[1] = g.specular_color_and_weight[2] = 1.0f;
        g.specular_color_and_weight[3] = 1.0f;
        g.specular_roughness = 0.3f;
        g.specular_roughness_anisotropy = 0.0f;
        g.specular_haze = 0.0f;
        g.specular_haze_spread = 0.3f;
        g.specular_ior = 1.5f;
        g.specular_retroreflectivity = 0.0f;
        g.normal_scale = 1.0f;
        if (const Json* nt = mat.get("normalTexture"))
            if (has_texture(nt)) g.normal_scale = (float)nt->number("scale", 1.0);
        if (const Json* ext = mat.get("extensions")) {
            if (const Json* es = ext->get("KHR_materials_emissive_strength"))
                g.emission_color_and_luminance[3] = (float)es->number("emissiveStrength", 1.0);
            if (const Json* ior = ext->get("KHR_materials_ior")) g.specular_ior = (float)ior->number("ior", 1.5);
            if (const Json* sp = ext->get("KHR_materials_specular")) {
                g.specular_color_and_weight[3] = (float)sp->number("specularFactor", 1.0);
                if (const Json* sc = sp->get("specularColorFactor"))
                    for (int i = 0; i < 3 && i < (int)sc->arr.size(); ++i)
                        g.specular_color_and_weight[i] = (float)sc->arr[i].num;
            }
        }
        const std::string mode = mat.string("alphaMode", "OPAQUE");
        g.alpha_mode = mode == "MASK" ? PT_ALPHA_MODE_MASK : mode == "BLEND" ? PT_ALPHA_MODE_BLEND : PT_ALPHA_MODE_OPAQUE;
        g.alpha_cutoff = (float)mat.number("alphaCutoff", 0.5);
        if (const Json* extras = mat.get("extras")) {
            // OpenPBR values in [0, 1]; out-of-range values are ignored as in the reference
            const auto apply = [&](const char* key, float* target) {
                const Json* v = extras->get(key);
                if (v && v->kind == Json::Number) {
                    const float f = (float)v->num;
                    if (f >= 0.0f && f <= 1.0f) *target = f;
                }
            };
            apply("OpenPBR_base_weight", &g.base_weight);
            apply("OpenPBR_emission_weight", &g.emission_weight);
            apply("OpenPBR_specular_roughness", &g.specular_roughness);
            apply("OpenPBR_specular_roughness_anisotropy", &g.specular_roughness_anisotropy);
            apply("OpenPBR_specular_haze", &g.specular_haze);
            apply("OpenPBR_specular_haze_spread", &g.specular_haze_spread);
            apply("OpenPBR_specular_retroreflectivity", &g.specular_retroreflectivity);
        }
        return ptw_add_material(world, &g, out) == PT_OK || fail(ptw_last_error(world));
    }

    bool primitive(const Json& prim, const M4& model, const double nm[9]) {
        if (prim.integer("mode", 4) != 4) return true;  // only triangles, as the reference
        const Json* attrs = prim.get("attributes");
        if (!attrs || !attrs->get("POSITION")) return true;  // no positions: skipped
        std::vector<float> pos, nor, tan, uv;
        size_t nv = 0, n2 = 0;
        if (!read_floats(attrs->integer("POSITION", -1), 3, pos, &nv)) return false;
        std::vector<uint32_t> idx;
        if (prim.get("indices")) {
            if (!read_indices(prim.integer("indices", -1), idx)) return false;
            for (uint32_t i : idx)
                if (i >= nv) return fail("index out of range");
        }
        const bool has_n = attrs->get("NORMAL") != nullptr;
        const bool has_t = has_n && attrs->get("TANGENT") != nullptr;
        const bool has_uv = attrs->get("TEXCOORD_0") != nullptr;
        if (has_n && (!read_floats(attrs->integer("NORMAL", -1), 3, nor, &n2) || n2 != nv))
            return error.empty() ? fail("NORMAL count differs from POSITION") : false;
        if (has_t && (!read_floats(attrs->integer("TANGENT", -1), 4, tan, &n2) || n2 != nv))
            return error.empty() ? fail("TANGENT count differs from POSITION") : false;
        if (has_uv && (!read_floats(attrs->integer("TEXCOORD_0", -1), 2, uv, &n2) || n2 != nv))
            return error.empty() ? fail("TEXCOORD_0 count differs from POSITION") : false;
        // transform_point3 / transform_vector3 with the node matrix
        for (size_t i = 0; i < nv; ++i) {
            const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
            for (int r = 0; r < 3; ++r)
                pos[3 * i + r] = ((model.m[r] * x + model.m[4 + r] * y) + model.m[8 + r] * z) + model.m[12 + r];
        }
        bool placeholder = false;
        for (size_t i = 0; has_t && i < nv; ++i) {
            const float* t = &tan[4 * i];
            if (t[0] == 1.0f && t[1] == 0.0f && t[2] == 0.0f && t[3] == 1.0f) placeholder = true;
        }
        for (size_t i = 0; has_n && i < nv; ++i) {
            const double x = nor[3 * i], y = nor[3 * i + 1], z = nor[3 * i + 2];
            for (int r = 0; r < 3; ++r) nor[3 * i + r] = (float)(nm[3 * r] * x + nm[3 * r + 1] * y + nm[3 * r + 2] * z);
        }
        for (size_t i = 0; has_t && i < nv; ++i) {
            const float x = tan[4 * i], y = tan[4 * i + 1], z = tan[4 * i + 2];
            for (int r = 0; r < 3; ++r) tan[4 * i + r] = (model.m[r] * x + model.m[4 + r] * y) + model.m[8 + r] * z;
        }
        uint32_t mi;
        const Json* mats = doc.get("materials");
        const long mat_index = prim.integer("material", -1);
        if (mat_index >= 0) {
            auto it = material_cache.find(mat_index);
            if (it != material_cache.end()) {
                mi = it->second;
            } else {
                if (!mats || (size_t)mat_index >= mats->arr.size()) return fail("material out of range");
                if (!material(&mats->arr[(size_t)mat_index], &mi)) return false;
                material_cache[mat_index] = mi;
            }
        } else if (!material(nullptr, &mi)) {
            return false;
        }
        ptw_mesh mesh;
        mesh.positions = pos.data();
        mesh.normals = has_n ? nor.data() : nullptr;
        mesh.uvs = has_uv ? uv.data() : nullptr;
        mesh.tangents = has_t && !placeholder ? tan.data() : nullptr;
        mesh.vertex_count = (uint32_t)nv;
        mesh.indices = idx.empty() ? nullptr : idx.data();
        mesh.index_count = (uint32_t)idx.size();
        mesh.material_index = mi;
        if (idx.empty() && nv % 3 != 0) return fail("non-indexed primitive with a vertex count not a multiple of 3");
        return ptw_add_mesh(world, &mesh) == PT_OK || fail(ptw_last_error(world));
    }

    bool load() {
        if (!images()) return false;
        const Json* nodes = doc.get("nodes");
        const Json* meshes = doc.get("meshes");
        std::vector<long> roots;
        const Json* scenes = doc.get("scenes");
        const long scene = doc.integer("scene", scenes && !scenes->arr.empty() ? 0 : -1);
        if (scene >= 0 && scenes && (size_t)scene < scenes->arr.size()) {
            if (const Json* sn = scenes->arr[(size_t)scene].get("nodes"))
                for (const Json& n : sn->arr) roots.push_back(index_of(n));
        } else if (nodes) {
            for (size_t i = 0; i < nodes->arr.size(); ++i) roots.push_back((long)i);
        }
        // the reference's LIFO node stack: the last root first, children pushed in order
        std::vector<std::pair<long, M4>> stack;
        for (long r : roots) stack.emplace_back(r, identity());
        size_t visited = 0;
        while (!stack.empty()) {
            const auto [ni, parent] = stack.back();
            stack.pop_back();
            if (!nodes || ni < 0 || (size_t)ni >= nodes->arr.size()) return fail("node out of range");
            if (++visited > 4 * nodes->arr.size() + 16) return fail("node graph is not a tree");
            const Json& node = nodes->arr[(size_t)ni];
            M4 local = identity();
            if (const Json* mtx = node.get("matrix")) {
                if (mtx->arr.size() != 16) return fail("node matrix must have 16 numbers");
                for (int i = 0; i < 16; ++i) local.m[i] = (float)mtx->arr[i].num;
            } else {
                float t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
                if (const Json* v = node.get("translation"))
                    for (int i = 0; i < 3 && i < (int)v->arr.size(); ++i) t[i] = (float)v->arr[i].num;
                if (const Json* v = node.get("rotation"))
                    for (int i = 0; i < 4 && i < (int)v->arr.size(); ++i) q[i] = (float)v->arr[i].num;
                if (const Json* v = node.get("scale"))
                    for (int i = 0; i < 3 && i < (int)v->arr.size(); ++i) s[i] = (float)v->arr[i].num;
                local = from_trs(t, q, s);
            }
            const M4 model = mul(parent, local);
            if (node.get("mesh")) {
                const long mi = node.integer("mesh", -1);
                if (!meshes || mi < 0 || (size_t)mi >= meshes->arr.size()) return fail("mesh out of range");
                double nm[9];
                normal_matrix(model, nm);
                if (const Json* prims = meshes->arr[(size_t)mi].get("primitives"))
                    for (const Json& prim : prims->arr)
                        if (!primitive(prim, model, nm)) return false;
            }
            if (const Json* ch = node.get("children"))
                for (const Json& c : ch->arr) stack.emplace_back(index_of(c), model);
        }
        return true;
    }
};

}  // namespace

namespace {
// the message, with every byte outside printable ASCII (an echo of the file's
// own bytes, e.g. a malformed name) shown as '?', so that callers always
// receive plain text
void printable_error(char* error, size_t size, const std::string& msg) {
    if (!error || !size) return;
    std::string clean(msg);
    for (char& c : clean)
        if ((unsigned char)c < 0x20 || (unsigned char)c > 0x7e) c = '?';
    snprintf(error, size, "%s", clean.c_str());
}
}  // namespace

extern "C" int ptw_load_gltf_bytes(ptw_world* world, const void* bytes, size_t size, char* error,
                                   size_t error_size) {
    if (!world || !bytes) return PT_ERR_INVALID_ARG;
    Loader l;
    l.world = world;
    bool ok;
    try {
        const std::vector<uint8_t> file((const uint8_t*)bytes, (const uint8_t*)bytes + size);
        ok = l.open_bytes(file) && l.load();
    } catch (const std::bad_alloc&) {
        if (error && error_size) snprintf(error, error_size, "out of host memory");
        return PT_ERR_OOM;
    } catch (const std::exception& e) {  // nothing may leave the C ABI as an exception
        if (error && error_size) snprintf(error, error_size, "glTF import failed: %s", e.what());
        return PT_ERR_INVALID_ARG;
    }
    if (!ok) printable_error(error, error_size, l.error);
    return ok ? PT_OK : PT_ERR_INVALID_ARG;
}

extern "C" int ptw_load_gltf(ptw_world* world, const char* path, char* error, size_t error_size) {
    if (!world || !path) return PT_ERR_INVALID_ARG;
    Loader l;
    l.world = world;
    bool ok;
    try {
        ok = l.open(path) && l.load();
    } catch (const std::bad_alloc&) {
        if (error && error_size) snprintf(error, error_size, "out of host memory");
        return PT_ERR_OOM;
    } catch (const std::exception& e) {  // nothing may leave the C ABI as an exception
        if (error && error_size) snprintf(error, error_size, "glTF import failed: %s", e.what());
        return PT_ERR_INVALID_ARG;
    }
    if (!ok) printable_error(error, error_size, l.error);
    return ok ? PT_OK : PT_ERR_INVALID_ARG;
}
