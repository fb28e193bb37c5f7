// mikktspace.cpp - per-corner tangent frames by Morten Mikkelsen's MikkTSpace
// method, which the reference runs (through bevy_mikktspace 1.0.0,
// world.rs:1238-1260) for glTF primitives without usable tangents.
//
// A restatement of the published algorithm ("Simulation of Wrinkled
// Surfaces Revisited", 2008, and its reference implementation mikktspace.c)
// for triangles with the default 180-degree angular threshold:
//   1. corners with identical position, normal and texture coordinate are
//      welded into one vertex;
//   2. triangles with two equal corner positions are degenerate and set
//      aside;
//   3. every other triangle gets its texture-space derivatives: the unit
//      tangent and bitangent directions (signed by the triangle's texture
//      orientation) and their magnitudes; triangles with zero texture area
//      or zero magnitudes may join any group;
//   4. triangles are linked to the neighbours across their edges;
//   5. around every welded vertex, triangles of equal orientation reachable
//      through shared edges form a group;
//   6. within a group, the faces whose projected directions are not exactly
//      opposite form a subgroup whose tangent frame is the angle-weighted sum
//      of the members' derivatives projected into the vertex's tangent plane;
//   7. corners of degenerate triangles copy the frame of a good corner on
//      the same welded vertex.
// The output tangent of a corner is the subgroup's normalised tangent with
// w = +1 for orientation-preserving texture mapping, -1 otherwise.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <tuple>
#include <utility>
#include <vector>

#include "pt_mikktspace.h"

namespace ptw {

namespace {

struct V3 {
    float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 scale(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
bool not_zero(float v) { return std::fabs(v) > FLT_MIN; }
bool not_zero(V3 a) { return not_zero(a.x) || not_zero(a.y) || not_zero(a.z); }
V3 normalize(V3 a) { return scale(1.0f / length(a), a); }
bool equal(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
// the direction projected into the plane of unit normal n, normalised when not zero
V3 project(V3 n, V3 v) {
    V3 r = sub(v, scale(dot(n, v), n));
    return not_zero(r) ? normalize(r) : r;
}

constexpr int kOrientPreserving = 1, kGroupWithAny = 2;

struct Tri {
    int flag = 0;
    V3 os{0, 0, 0}, ot{0, 0, 0};  // unit texture-space tangent / bitangent directions
    float mag_s = 0, mag_t = 0;
    int neighbour[3] = {-1, -1, -1};  // across the edge from corner i to corner i + 1
    int group[3] = {-1, -1, -1};
};

struct Group {
    int vertex;  // welded vertex the group is around
    bool orient;
    std::vector<int> faces;
};

struct Frame {
    V3 os{1, 0, 0};
    bool orient = false;
};

float key_bits(float v) { return v == 0.0f ? 0.0f : v; }  // -0 welds with +0

}  // namespace

// corners: 3 per triangle, each with a position (3 floats), a unit normal
// (3) and a texture coordinate (2); writes 4 floats per corner
void mikktspace_tangents(size_t triangles, const float* pos, const float* nor, const float* uv, float* out) {
    const size_t corners = triangles * 3;
    const auto P = [&](int c) { return V3{pos[3 * c], pos[3 * c + 1], pos[3 * c + 2]}; };
    const auto N = [&](int c) { return V3{nor[3 * c], nor[3 * c + 1], nor[3 * c + 2]}; };
    // 1. weld: every corner points at the first corner with identical data
    std::vector<int> vert(corners);
    {
        std::map<std::tuple<float, float, float, float, float, float, float, float>, int> first;
        for (size_t c = 0; c < corners; ++c) {
            const auto key = std::make_tuple(key_bits(pos[3 * c]), key_bits(pos[3 * c + 1]), key_bits(pos[3 * c + 2]),
                                             key_bits(nor[3 * c]), key_bits(nor[3 * c + 1]), key_bits(nor[3 * c + 2]),
                                             key_bits(uv[2 * c]), key_bits(uv[2 * c + 1]));
            vert[c] = first.emplace(key, (int)c).first->second;
        }
    }
    // 2. good triangles first, degenerate ones after them, each in input order
    std::vector<int> order;
    std::vector<int> degenerate;
    for (size_t f = 0; f < triangles; ++f) {
        const V3 p0 = P(vert[3 * f]), p1 = P(vert[3 * f + 1]), p2 = P(vert[3 * f + 2]);
        (equal(p0, p1) || equal(p0, p2) || equal(p1, p2) ? degenerate : order).push_back((int)f);
    }
    const int good = (int)order.size();
    order.insert(order.end(), degenerate.begin(), degenerate.end());
    // triangle k of the processing order uses corners of input face order[k]
    const auto V = [&](int k, int i) { return vert[3 * (size_t)order[(size_t)k] + (size_t)i]; };
    // 3. texture-space derivatives
    std::vector<Tri> tri((size_t)good);
    for (int k = 0; k < good; ++k) {
        Tri& t = tri[(size_t)k];
        t.flag = kGroupWithAny;
        const int c0 = V(k, 0), c1 = V(k, 1), c2 = V(k, 2);
        const V3 v1 = P(c0), v2 = P(c1), v3 = P(c2);
        const float t21x = uv[2 * c1] - uv[2 * c0], t21y = uv[2 * c1 + 1] - uv[2 * c0 + 1];
        const float t31x = uv[2 * c2] - uv[2 * c0], t31y = uv[2 * c2 + 1] - uv[2 * c0 + 1];
        const V3 d1 = sub(v2, v1), d2 = sub(v3, v1);
        const float area2 = t21x * t31y - t21y * t31x;
        const V3 os = sub(scale(t31y, d1), scale(t21y, d2));
        const V3 ot = add(scale(-t31x, d1), scale(t21x, d2));
        if (area2 > 0) t.flag |= kOrientPreserving;
        if (not_zero(area2)) {
            const float abs_area = std::fabs(area2), len_s = length(os), len_t = length(ot);
            const float sign = (t.flag & kOrientPreserving) ? 1.0f : -1.0f;
            if (not_zero(len_s)) t.os = scale(sign / len_s, os);
            if (not_zero(len_t)) t.ot = scale(sign / len_t, ot);
            t.mag_s = len_s / abs_area;
            t.mag_t = len_t / abs_area;
            if (not_zero(t.mag_s) && not_zero(t.mag_t)) t.flag &= ~kGroupWithAny;
        }
    }
    // 4. neighbours: an edge pairs with the first unpaired edge running the other way
    {
        std::map<std::pair<int, int>, std::vector<std::pair<int, int>>> edges;  // (from, to) -> (triangle, edge)
        for (int k = 0; k < good; ++k)
            for (int i = 0; i < 3; ++i) edges[{V(k, i), V(k, (i + 1) % 3)}].push_back({k, i});
        for (int k = 0; k < good; ++k)
            for (int i = 0; i < 3; ++i) {
                if (tri[(size_t)k].neighbour[i] >= 0) continue;
                const auto it = edges.find({V(k, (i + 1) % 3), V(k, i)});
                if (it == edges.end()) continue;
                for (const auto& [g, e] : it->second)
                    if (g != k && tri[(size_t)g].neighbour[e] < 0) {
                        tri[(size_t)k].neighbour[i] = g;
                        tri[(size_t)g].neighbour[e] = k;
                        break;
                    }
            }
    }
    // 5. groups around welded vertices
    std::vector<Group> groups;
    // grows group gi from triangle k0 through edge neighbours around the group's vertex:
    // a triangle joins if its corner there is free and its orientation matches
    std::vector<std::pair<int, int>> stack;
    const auto assign = [&](int k0, int gi) {
        stack.assign(1, {k0, gi});
        while (!stack.empty()) {
            const int k = stack.back().first;
            stack.pop_back();
            Group& g = groups[(size_t)gi];
            Tri& t = tri[(size_t)k];
            int i = 0;
            while (i < 3 && V(k, i) != g.vertex) ++i;
            if (i == 3 || t.group[i] == gi || t.group[i] >= 0) continue;
            if ((t.flag & kGroupWithAny) && t.group[0] < 0 && t.group[1] < 0 && t.group[2] < 0)
                t.flag = (t.flag & ~kOrientPreserving) | (g.orient ? kOrientPreserving : 0);
            if (((t.flag & kOrientPreserving) != 0) != g.orient) continue;
            g.faces.push_back(k);
            t.group[i] = gi;
            const int left = t.neighbour[i], right = t.neighbour[i > 0 ? i - 1 : 2];
            // depth first, left before right
            if (right >= 0) stack.push_back({right, gi});
            if (left >= 0) stack.push_back({left, gi});
        }
    };
    for (int k = 0; k < good; ++k)
        for (int i = 0; i < 3; ++i) {
            if (tri[(size_t)k].group[i] >= 0) continue;
            const int gi = (int)groups.size();
            groups.push_back({V(k, i), (tri[(size_t)k].flag & kOrientPreserving) != 0, {k}});
            tri[(size_t)k].group[i] = gi;
            const int left = tri[(size_t)k].neighbour[i], right = tri[(size_t)k].neighbour[i > 0 ? i - 1 : 2];
            if (left >= 0) assign(left, gi);
            if (right >= 0) assign(right, gi);
        }
    // 6. frames per subgroup
    std::vector<Frame> frame(corners);  // by input corner
    const float thres_cos = (float)std::cos(180.0 * 3.14159265358979323846 / 180.0);
    std::vector<int> members;
    std::vector<std::pair<std::vector<int>, Frame>> subgroups;
    for (size_t gi = 0; gi < groups.size(); ++gi) {
        const Group& g = groups[gi];
        subgroups.clear();
        for (const int k : g.faces) {
            const Tri& t = tri[(size_t)k];
            int index = 0;
            while (t.group[index] != (int)gi) ++index;
            const V3 n = N(V(k, index));
            const V3 os = project(n, t.os), ot = project(n, t.ot);
            members.clear();
            for (const int m : g.faces) {
                const Tri& u = tri[(size_t)m];
                const V3 os2 = project(n, u.os), ot2 = project(n, u.ot);
                const bool any = ((t.flag | u.flag) & kGroupWithAny) != 0;
                if (any || m == k || (dot(os, os2) > thres_cos && dot(ot, ot2) > thres_cos)) members.push_back(m);
            }
            std::sort(members.begin(), members.end());
            size_t s = 0;
            while (s < subgroups.size() && subgroups[s].first != members) ++s;
            if (s == subgroups.size()) {
                // angle-weighted sum over the members that have valid derivatives
                V3 sum_s{0, 0, 0};
                for (const int m : members) {
                    const Tri& u = tri[(size_t)m];
                    if (u.flag & kGroupWithAny) continue;
                    int i = 0;
                    while (i < 3 && V(m, i) != g.vertex) ++i;
                    const V3 nn = N(V(m, i));
                    const V3 vs = project(nn, u.os);
                    const V3 p0 = P(V(m, i > 0 ? i - 1 : 2)), p1 = P(V(m, i)), p2 = P(V(m, i < 2 ? i + 1 : 0));
                    const V3 e1 = project(nn, sub(p0, p1)), e2 = project(nn, sub(p2, p1));
                    float c = dot(e1, e2);
                    c = c > 1.0f ? 1.0f : (c < -1.0f ? -1.0f : c);
                    const float angle = (float)std::acos((double)c);
                    sum_s = add(sum_s, scale(angle, vs));
                }
                Frame f;
                f.os = not_zero(sum_s) ? normalize(sum_s) : sum_s;
                subgroups.push_back({members, f});
            }
            Frame& out_frame = frame[3 * (size_t)order[(size_t)k] + (size_t)index];
            out_frame = subgroups[s].second;
            out_frame.orient = g.orient;
        }
    }
    // 7. corners of degenerate triangles take the frame of a good corner on the same vertex
    {
        std::map<int, size_t> good_corner;
        for (int k = 0; k < good; ++k)
            for (int i = 0; i < 3; ++i) good_corner.emplace(V(k, i), 3 * (size_t)order[(size_t)k] + (size_t)i);
        for (int k = good; k < (int)triangles; ++k)
            for (int i = 0; i < 3; ++i) {
                const auto it = good_corner.find(V(k, i));
                if (it != good_corner.end()) frame[3 * (size_t)order[(size_t)k] + (size_t)i] = frame[it->second];
            }
    }
    for (size_t c = 0; c < corners; ++c) {
        out[4 * c] = frame[c].os.x;
        out[4 * c + 1] = frame[c].os.y;
        out[4 * c + 2] = frame[c].os.z;
        out[4 * c + 3] = frame[c].orient ? 1.0f : -1.0f;
    }
}

}  // namespace ptw
