// wide_bvh.cpp - host side of the precision form (include/pt_precision.h):
// the 8-wide BVH collapsed from the reference's binary BVH (world.rs:323-335,
// 1430-1591) with outward-rounded 8-bit child boxes, and the FP16 attribute
// conversion.
//
// Quantisation.  Per wide node and axis the frame origin is the minimum of
// the children's box minima and the scale a power of two s = 2^e; a child's
// lower bound becomes the largest q in [0, 255] with origin + q*s <= lo and
// its upper bound the smallest q with origin + q*s >= hi, both evaluated in
// FP32 exactly as the traversal kernel decodes them (q*s is exact, the one
// addition rounds to nearest).  e is the smallest exponent for which every
// child's upper bound fits in 8 bits.  Every decoded box therefore contains
// its binary node's box, and since the slab test is monotone in the box
// bounds, a wide box test accepts every ray the binary node's test accepts.
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/pt_precision.h"
#include "pt_abi_guard.h"
#include "pt_links.h"

namespace {

constexpr int kMinExp = -126;  // scale stays a normal float
constexpr int kMaxExp = 104;   // 2^(e + 23) stays finite (the kernel's exact decode)
constexpr uint32_t kMaxDepth = 64;

float decode(float origin, uint32_t q, float scale) {
    const float qs = (float)q * scale;  // exact
    return origin + qs;                 // one rounding, as in the kernel
}

double half_area(const pt_bvh_node& n) {
    const double dx = (double)n.aabb_max[0] - n.aabb_min[0];
    const double dy = (double)n.aabb_max[1] - n.aabb_min[1];
    const double dz = (double)n.aabb_max[2] - n.aabb_min[2];
    return dx * dy + dy * dz + dz * dx;
}

bool finite_box(const pt_bvh_node& n) {
    for (int a = 0; a < 3; ++a)
        if (!std::isfinite(n.aabb_min[a]) || !std::isfinite(n.aabb_max[a])) return false;
    return true;
}

// quantise one axis of up to 8 child boxes; false if no exponent fits
bool quantise_axis(float origin, const float* lo, const float* hi, int n, uint8_t* qlo, uint8_t* qhi, uint8_t* ebyte) {
    double ext = 0.0;
    for (int i = 0; i < n; ++i) ext = std::fmax(ext, (double)hi[i] - (double)origin);
    int e = kMinExp;
    if (ext > 0.0) {
        int ex = 0;
        std::frexp(ext / 255.0, &ex);  // ext / 255 < 2^ex
        e = ex - 1;
        if (e < kMinExp) e = kMinExp;
    }
    for (; e <= kMaxExp; ++e) {
        const float s = std::ldexp(1.0f, e);
        bool ok = true;
        for (int i = 0; i < n && ok; ++i) {
            double fl = std::floor(((double)lo[i] - (double)origin) / (double)s);
            int q = fl < 0.0 ? 0 : (fl > 255.0 ? 255 : (int)fl);
            while (q > 0 && decode(origin, (uint32_t)q, s) > lo[i]) --q;
            while (q < 255 && decode(origin, (uint32_t)q + 1u, s) <= lo[i]) ++q;
            if (decode(origin, (uint32_t)q, s) > lo[i]) ok = false;  // cannot happen: q = 0 decodes to origin
            double ce = std::ceil(((double)hi[i] - (double)origin) / (double)s);
            if (ce > 256.0) {
                ok = false;
                break;
            }
            int u = ce < 0.0 ? 0 : (int)ce;
            while (u <= 255 && decode(origin, (uint32_t)u, s) < hi[i]) ++u;
            if (u > 255) {
                ok = false;
                break;
            }
            while (u > 0 && decode(origin, (uint32_t)u - 1u, s) >= hi[i]) --u;
            qlo[i] = (uint8_t)q;
            qhi[i] = (uint8_t)u;
        }
        if (ok) {
            *ebyte = (uint8_t)(e + 127);
            return true;
        }
    }
    return false;
}

// Places the children of a wide node into slots 0..n-1 so that a ray whose
// direction has sign bits o (bit a set when d[a] < 0) meets them roughly
// nearest first when it visits slot i ^ o for i = 0, 1, ..., 7: slot s should
// hold the child lying furthest back along the direction of octant s, D(s) =
// (+-1, +-1, +-1) with a minus for each set bit of s.  Cost of child c in slot s
// = dot(centre(c) - centre(node), D(s)) over the decoded child boxes; pairs
// are taken greedily, lowest cost first (the assignment of Ylitie, Karras and
// Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs", HPG 2017).  A slot carries its box bytes, child index and triangle
// count, so the permutation keeps the tree; the order changes no result:
// every accepted child is still visited and exact-t ties are resolved by the
// binary traversal's order.
void order_by_octant(pt_wide_node& node) {
    const int n = node.child_count;
    if (n < 2) return;
    float cen[8][3], pc[3] = {0.0f, 0.0f, 0.0f};
    for (int a = 0; a < 3; ++a) {
        const float s = std::ldexp(1.0f, (int)node.exponent[a] - 127);
        for (int i = 0; i < n; ++i) {
            cen[i][a] = 0.5f * s * ((float)node.lo[a][i] + (float)node.hi[a][i]);  // relative to the origin
            pc[a] += cen[i][a];
        }
        pc[a] /= (float)n;
    }
    float cost[8][8];
    for (int i = 0; i < n; ++i)
        for (int s = 0; s < n; ++s) {
            float c = 0.0f;
            for (int a = 0; a < 3; ++a) c += ((s >> a) & 1 ? -1.0f : 1.0f) * (cen[i][a] - pc[a]);
            cost[i][s] = c;
        }
    int slot_of[8];
    bool child_done[8] = {}, slot_done[8] = {};
    for (int k = 0; k < n; ++k) {
        int bi = -1, bs = -1;
        for (int i = 0; i < n; ++i) {
            if (child_done[i]) continue;
            for (int s = 0; s < n; ++s)
                if (!slot_done[s] && (bi < 0 || cost[i][s] < cost[bi][bs])) {
                    bi = i;
                    bs = s;
                }
        }
        child_done[bi] = slot_done[bs] = true;
        slot_of[bi] = bs;
    }
    const pt_wide_node in = node;
    for (int i = 0; i < n; ++i) {
        const int s = slot_of[i];
        for (int a = 0; a < 3; ++a) {
            node.lo[a][s] = in.lo[a][i];
            node.hi[a][s] = in.hi[a][i];
        }
        node.child[s] = in.child[i];
        node.tri_count[s] = in.tri_count[i];
    }
}

// order_by_octant over all nodes, on up to 16 host threads (nodes are
// independent).  A host that refuses a new thread gets the remaining ranges
// done on the calling thread: no exception leaves the C ABI.
void order_all_by_octant(std::vector<pt_wide_node>& wide) {
    const size_t count = wide.size();
    unsigned threads = std::thread::hardware_concurrency();
    threads = threads == 0 ? 1 : (threads > 16 ? 16 : threads);
    if (count < 4096) threads = 1;
    const size_t per = (count + threads - 1) / threads;
    const auto range = [&wide](size_t lo, size_t hi) {
        for (size_t k = lo; k < hi; ++k) order_by_octant(wide[k]);
    };
    std::vector<std::thread> pool;
    size_t next = 0;  // first node no thread has taken
    for (unsigned t = 1; t < threads && next + per < count; ++t) {
        const size_t lo = next, hi = lo + per;
        try {
            pool.emplace_back(range, lo, hi);
        } catch (const std::system_error&) {
            break;
        }
        next = hi;
    }
    range(next, count);
    for (auto& th : pool) th.join();
}

struct Work {
    uint32_t bnode;  // binary node the wide node is collapsed from
    uint32_t wide;   // its index
    uint32_t depth;
};

}  // namespace

namespace {

// Frame origin and outward-rounded 8-bit child boxes of every wide node from
// its binary children (quantise_axis); nodes are independent, so up to 16
// host threads share them.  PT_ERR_INVALID_ARG if a child box is not finite
// or an axis fits no exponent.
int quantise_all(const pt_bvh_node* nodes, std::vector<pt_wide_node>& wide,
                 const std::vector<std::array<uint32_t, 8>>& kids_of) {
    if (kids_of.size() < wide.size()) return PT_ERR_INVALID_ARG;  // every wide node was reached by the walk
    std::atomic<bool> bad{false};
    const auto range = [&](size_t lo_k, size_t hi_k) {
        for (size_t k = lo_k; k < hi_k && !bad.load(std::memory_order_relaxed); ++k) {
            pt_wide_node& node = wide[k];
            const int n = node.child_count;
            float lo[3][8], hi[3][8];
            for (int i = 0; i < n; ++i) {
                const pt_bvh_node& c = nodes[kids_of[k][i]];
                if (!finite_box(c)) {
                    bad = true;
                    return;
                }
                for (int a = 0; a < 3; ++a) {
                    lo[a][i] = c.aabb_min[a];
                    hi[a][i] = c.aabb_max[a];
                }
            }
            for (int a = 0; a < 3; ++a) {
                float origin = lo[a][0];
                for (int i = 1; i < n; ++i) origin = std::fmin(origin, lo[a][i]);
                node.origin[a] = origin;
                if (!quantise_axis(origin, lo[a], hi[a], n, node.lo[a], node.hi[a], &node.exponent[a])) {
                    bad = true;
                    return;
                }
            }
        }
    };
    const size_t count = wide.size();
    unsigned threads = std::thread::hardware_concurrency();
    threads = threads == 0 ? 1 : (threads > 16 ? 16 : threads);
    if (count < 4096) threads = 1;
    const size_t per = (count + threads - 1) / threads;
    std::vector<std::thread> pool;
    size_t next = 0;  // first node no thread has taken
    for (unsigned t = 1; t < threads && next + per < count; ++t) {
        const size_t lo_k = next, hi_k = lo_k + per;
        try {
            pool.emplace_back(range, lo_k, hi_k);
        } catch (const std::system_error&) {
            break;  // the calling thread takes the rest
        }
        next = hi_k;
    }
    range(next, count);
    for (auto& th : pool) th.join();
    return bad ? PT_ERR_INVALID_ARG : PT_OK;
}

// the collapse proper, without the octant placement
int collapse(const pt_bvh_node* nodes, uint64_t node_count, uint32_t max_leaf_triangles,
             std::vector<pt_wide_node>& wide, uint32_t* wide_depth) {
    if (!nodes || node_count == 0 || node_count > 0xffffffffull) return PT_ERR_INVALID_ARG;
    // triangle range of every binary subtree (children follow their parent in
    // the reference's layout, so one backward pass suffices); a subtree of at
    // most max_leaf_triangles triangles in one contiguous range becomes a
    // single leaf child
    std::vector<uint32_t> sub_first, sub_count;
    if (max_leaf_triangles > 0) {
        sub_first.assign(node_count, 0);
        sub_count.assign(node_count, 0xffffffffu);  // not mergeable
        for (uint64_t k = node_count; k-- > 0;) {
            const pt_bvh_node& n = nodes[k];
            if (n.tri_count != 0) {
                sub_first[k] = n.left_first;
                sub_count[k] = n.tri_count;
                continue;
            }
            const uint64_t l = n.left_first, r = l + 1;
            if (l <= k || r >= node_count) continue;
            if (sub_count[l] == 0xffffffffu || sub_count[r] == 0xffffffffu) continue;
            if (sub_first[l] + sub_count[l] == sub_first[r]) {
                sub_first[k] = sub_first[l];
            } else if (sub_first[r] + sub_count[r] == sub_first[l]) {
                sub_first[k] = sub_first[r];
            } else {
                continue;
            }
            const uint64_t total = (uint64_t)sub_count[l] + sub_count[r];
            sub_count[k] = total > 0xffffu ? 0xffffffffu : (uint32_t)total;
        }
    }
    const auto as_leaf = [&](uint32_t b) {
        return nodes[b].tri_count != 0 || (max_leaf_triangles > 0 && sub_count[b] <= max_leaf_triangles);
    };
    wide.assign(1, pt_wide_node{});
    std::memset(wide.data(), 0, sizeof(pt_wide_node));
    std::vector<std::array<uint32_t, 8>> kids_of(1);  // binary children of each wide node, in slot order
    std::vector<Work> stack{{0u, 0u, 1u}};
    uint32_t max_depth = 0;
    const auto interior_ok = [&](uint32_t b) {
        const pt_bvh_node& n = nodes[b];
        return n.tri_count != 0 || (n.left_first >= 1 && (uint64_t)n.left_first + 1 < node_count);
    };
    while (!stack.empty()) {
        const Work wk = stack.back();
        stack.pop_back();
        if (wk.depth > kMaxDepth) return PT_ERR_INVALID_ARG;  // deeper than any traversal stack, or cyclic
        if (wk.depth > max_depth) max_depth = wk.depth;
        const pt_bvh_node& b = nodes[wk.bnode];
        if (!interior_ok(wk.bnode)) return PT_ERR_INVALID_ARG;
        uint32_t kids[8];
        int n = 0;
        if (b.tri_count != 0) {
            kids[n++] = wk.bnode;  // a leaf root: one leaf child
        } else {
            kids[n++] = b.left_first;
            kids[n++] = b.left_first + 1;
        }
        while (n < 8) {
            int best = -1;
            double best_area = -1.0;
            for (int i = 0; i < n; ++i) {
                if (as_leaf(kids[i])) continue;
                const double a = half_area(nodes[kids[i]]);
                if (a > best_area) {
                    best_area = a;
                    best = i;
                }
            }
            if (best < 0) break;
            const uint32_t open = kids[best];
            if (!interior_ok(open)) return PT_ERR_INVALID_ARG;
            for (int i = n; i > best + 1; --i) kids[i] = kids[i - 1];
            kids[best] = nodes[open].left_first;
            kids[best + 1] = nodes[open].left_first + 1;
            ++n;
        }
        for (int i = 0; i < n; ++i)
            if (nodes[kids[i]].tri_count > 0xffffu) return PT_ERR_INVALID_ARG;
        pt_wide_node node;
        std::memset(&node, 0, sizeof node);
        node.child_count = (uint8_t)n;
        node.source_node = wk.bnode;
        // the boxes are quantised after the walk (quantise_all), from these children
        std::array<uint32_t, 8> slots{};
        for (int i = 0; i < n; ++i) slots[i] = kids[i];
        if (kids_of.size() <= wk.wide) kids_of.resize((size_t)wk.wide + 1);
        kids_of[wk.wide] = slots;
        const uint32_t first_child = (uint32_t)wide.size();
        uint32_t next = first_child;
        for (int i = 0; i < n; ++i) {
            const pt_bvh_node& c = nodes[kids[i]];
            if (c.tri_count != 0) {
                node.child[i] = c.left_first;
                node.tri_count[i] = (uint16_t)c.tri_count;
            } else if (as_leaf(kids[i])) {
                node.child[i] = sub_first[kids[i]];
                node.tri_count[i] = (uint16_t)sub_count[kids[i]];
            } else {
                node.child[i] = next++;
                node.tri_count[i] = 0;
            }
        }
        if ((uint64_t)next > node_count) return PT_ERR_INVALID_ARG;  // more wide nodes than binary ones: not a tree
        wide[wk.wide] = node;
        wide.resize(next);
        // depth-first: the first interior child is expanded next, siblings stay contiguous
        for (int i = n - 1; i >= 0; --i)
            if (node.tri_count[i] == 0) stack.push_back({kids[i], node.child[i], wk.depth + 1});
    }
    if (wide_depth) *wide_depth = max_depth;
    return quantise_all(nodes, wide, kids_of);
}

}  // namespace

int ptw::build_wide_bvh(const pt_bvh_node* nodes, uint64_t node_count, uint32_t max_leaf_triangles,
                        std::vector<pt_wide_node>& wide, uint32_t* wide_depth) {
    const int rc = collapse(nodes, node_count, max_leaf_triangles, wide, wide_depth);
    if (rc == PT_OK) order_all_by_octant(wide);
    return rc;
}

extern "C" int pt_build_wide_bvh(const pt_bvh_node* nodes, uint64_t node_count, uint32_t max_leaf_triangles,
                                 pt_wide_node* out, uint64_t capacity, uint64_t* wide_count, uint32_t* wide_depth) try {
    std::vector<pt_wide_node> wide;
    const int rc = collapse(nodes, node_count, max_leaf_triangles, wide, wide_depth);
    if (rc != PT_OK) return rc;
    if (wide_count) *wide_count = wide.size();
    if (!out) return PT_OK;
    if (capacity < wide.size()) return PT_ERR_OUT_OF_LIMITS;
    order_all_by_octant(wide);
    std::memcpy(out, wide.data(), wide.size() * sizeof(pt_wide_node));
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

namespace {

// IEEE binary32 -> binary16, round to nearest even
uint16_t to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // >= 65520 rounds to infinity
    if (ax < 0x38800000u) {                                    // below 2^-14: subnormal or zero
        if (ax <= 0x33000000u) return (uint16_t)sign;           // <= 2^-25 rounds to zero
        const uint32_t e = ax >> 23, m = (ax & 0x7fffffu) | 0x800000u;
        const uint32_t shift = 126u - e;  // units of 2^-24
        uint32_t r = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
        if (rem > halfway || (rem == halfway && (r & 1u))) ++r;
        return (uint16_t)(sign | r);
    }
    uint32_t r = (ax >> 13) - ((127u - 15u) << 10);
    const uint32_t rem = ax & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) ++r;
    return (uint16_t)(sign | r);
}

}  // namespace

extern "C" void pt_half_attributes(const pt_triangle_attribute* in, uint64_t count, pt_half_attribute* out) {
    for (uint64_t i = 0; i < count; ++i) {
        const pt_triangle_attribute& a = in[i];
        pt_half_attribute& h = out[i];
        std::memset(&h, 0, sizeof h);
        for (int k = 0; k < 3; ++k) {
            h.n0[k] = to_half(a.n0[k]);
            h.n1[k] = to_half(a.n1[k]);
            h.n2[k] = to_half(a.n2[k]);
        }
        for (int k = 0; k < 4; ++k) {
            h.t0[k] = to_half(a.t0[k]);
            h.t1[k] = to_half(a.t1[k]);
            h.t2[k] = to_half(a.t2[k]);
        }
        for (int k = 0; k < 2; ++k) {
            h.uv0[k] = to_half(a.uv0[k]);
            h.uv1[k] = to_half(a.uv1[k]);
            h.uv2[k] = to_half(a.uv2[k]);
        }
        h.material_index = a.material_index;
    }
}

bool ptw::build_bvh_links(const pt_bvh_node* nodes, uint64_t node_count, uint64_t tri_count, uint32_t* parent,
                          uint32_t* leaf_of) {
    for (uint64_t i = 0; i < node_count; ++i) parent[i] = 0xffffffffu;
    for (uint64_t t = 0; t < tri_count; ++t) leaf_of[t] = 0xffffffffu;
    for (uint64_t i = 0; i < node_count; ++i) {
        const pt_bvh_node& n = nodes[i];
        if (n.tri_count == 0) {
            if ((uint64_t)n.left_first + 1 >= node_count) return false;
            parent[n.left_first] = (uint32_t)i;
            parent[n.left_first + 1] = (uint32_t)i;
        } else {
            if ((uint64_t)n.left_first + n.tri_count > tri_count) return false;
            for (uint32_t k = 0; k < n.tri_count; ++k) leaf_of[n.left_first + k] = (uint32_t)i;
        }
    }
    return true;
}
