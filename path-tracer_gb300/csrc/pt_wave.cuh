// pt_wave.cuh - device building blocks shared by the wavefront kernels of one
// tile (trace_wavefront.cu) and of many jobs (batch.cu): the derived BVH and
// triangle layouts, the queue view, the per-lane traversal state machine and
// warp-aggregated queue appends.
#pragma once

#include <type_traits>

#include "pt_path.cuh"

namespace ptd {

struct Fast {
    const float4* pairs;  // node i at pairs[2i], pairs[2i+1]
    const float4* tri4;   // triangle i at tri4[kTriStride i .. kTriStride i + 2] (padded to 48 or 64 bytes)
    const float4* wide = nullptr;  // pt_wide_node i at wide[8i .. 8i+7] (precision form)
    const uint32_t* parent = nullptr;   // binary node -> its parent (root: 0xffffffff)
    const uint32_t* leaf_of = nullptr;  // triangle -> the binary leaf holding it
};


struct Queues {
    float4* o[2];
    float4* d[2];
    float4* T[2];
    float4* hit;
    float4* color;
    float4* so;
    float4* sd;
    float4* sc;
    uint32_t* hit_list;   // slots of the current queue whose ray hit a triangle
    uint32_t* miss_list;  // slots whose ray left the scene
    uint32_t* hit_sorted = nullptr;  // the hit list sorted by key (when cnt[7] != 0)
    // beside the hit list, each filed hit's triangle-bucket sort key (triangle
    // >> key_shift, at most the last bucket), written by the extend kernel so
    // that the sort reads its keys in order instead of gathering the hit
    // records; null: the sort computes the keys itself
    uint32_t* hit_keys = nullptr;
    uint32_t key_shift = 0;
    uint32_t* cnt;  // [0], [1] ray queue lengths, [2] shadow length, [3] extend fetch, [4] shadow fetch,
                    // [5] hit list length, [6] miss list length, [7] 1 if hit_sorted holds this bounce's hits,
                    // [8] 1 if hit_sorted holds the order of the current ray queue, [9] of the shadow queue
    Counters* rec;  // per path (recording variants)
    int32_t* rec_hits;
};

// the queues one stage reads and writes, with the ping-pong already resolved
struct Stage {
    float4* o;  // current ray queue
    float4* d;
    float4* T;
    float4* no;  // next ray queue
    float4* nd;
    float4* nT;
    uint32_t* count;       // length of the current queue
    uint32_t* next_count;  // length of the next queue
};

PTD Stage stage_of(const Queues& q, int cur) {
    Stage s;
    s.o = cur ? q.o[1] : q.o[0];
    s.d = cur ? q.d[1] : q.d[0];
    s.T = cur ? q.T[1] : q.T[0];
    s.no = cur ? q.o[0] : q.o[1];
    s.nd = cur ? q.d[0] : q.d[1];
    s.nT = cur ? q.T[0] : q.T[1];
    s.count = cur ? q.cnt + 1 : q.cnt;
    s.next_count = cur ? q.cnt : q.cnt + 1;
    return s;
}

// launch shapes (overridable at build time for tuning sweeps)
#ifndef PT_EXTEND_THREADS
#define PT_EXTEND_THREADS 128
#endif
// 9 resident blocks of the traversal kernels per SM: at most 56 registers, no spills
#ifndef PT_EXTEND_MIN_BLOCKS
#define PT_EXTEND_MIN_BLOCKS 9
#endif
// the shading kernel: one resident block of 1024 per SM, at most 64
// registers.  Its grid-stride loop hands consecutive slots of the (sorted)
// hit list to consecutive warps, so a block of 1024 keeps 1024 neighbouring
// hits - the same triangles, attributes and materials - in one SM's L1:
// measured 14 % less shading time than 8 blocks of 128 with the same
// registers
#ifndef PT_SHADE_THREADS
#define PT_SHADE_THREADS 1024
#endif
#ifndef PT_SHADE_MIN_BLOCKS
#define PT_SHADE_MIN_BLOCKS 1
#endif
#ifndef PT_STEPS_PER_REFILL
#define PT_STEPS_PER_REFILL 32
#endif
// idle lanes of a traversal warp take new rays once fewer than this many are busy
#ifndef PT_REFILL_BELOW
#define PT_REFILL_BELOW 32
#endif
// binary subtrees of at most this many triangles become one leaf of the 8-wide BVH
#ifndef PT_WIDE_LEAF_MERGE
#define PT_WIDE_LEAF_MERGE 0
#endif
// 1: a step of the 8-wide traversal tests one triangle of a leaf; 0: the whole leaf
#ifndef PT_WIDE_TRI_PER_STEP
#define PT_WIDE_TRI_PER_STEP 0
#endif
constexpr uint32_t kWideLeafMerge = PT_WIDE_LEAF_MERGE;
// 1: the 8-wide traversal visits a node's accepted children in the order of
// their slots XOR the ray's direction octant (the builder places children for
// that order), with three-input min/max in the child test; 0: it sorts the
// accepted children by entry distance
#ifndef PT_WIDE_OCTANT
#define PT_WIDE_OCTANT 1
#endif
// 1: the accepted children are collected in slot order and the 8-bit mask is
// permuted to octant order once per node; 0: each child sets its octant-order
// bit directly
#ifndef PT_WIDE_MASK_PERMUTE
#define PT_WIDE_MASK_PERMUTE 1
#endif
// resident blocks per SM the 8-wide traversal kernels are compiled for
#ifndef PT_WIDE_MIN_BLOCKS
#define PT_WIDE_MIN_BLOCKS 8
#endif
// 1: a traversal step tests one triangle of a leaf; 0: a whole leaf
#ifndef PT_TRI_PER_STEP
#define PT_TRI_PER_STEP 1
#endif
// the same for the binary shadow (any-hit) traversal, whose warps run the
// majority kind of step: there whole leaves per step measured 6 % faster
#ifndef PT_SHADOW_TRI_PER_STEP
#define PT_SHADOW_TRI_PER_STEP 0
#endif
// order the next bounce's rays / the shadow rays by direction octant before
// their traversal (when the hit sort is on and a queue holds at least its
// threshold); measured slower: the octant split breaks up the origin
// coherence the hit sort gives the next rays, so off by default
#ifndef PT_RAY_ORDER
#define PT_RAY_ORDER 0
#endif
#ifndef PT_SHADOW_ORDER
#define PT_SHADOW_ORDER 0
#endif
// 1: a pixel's samples are consecutive paths of a group / work item
// (camera rays of a warp share their first nodes); 0: sample-major
#ifndef PT_PIXEL_MAJOR
#define PT_PIXEL_MAJOR 1
#endif
constexpr int kExtendThreads = PT_EXTEND_THREADS;
constexpr int kShadeThreads = PT_SHADE_THREADS;
// entries at the top of each traversal lane's stack kept in shared memory
#ifndef PT_SMEM_STACK
#define PT_SMEM_STACK 8
#endif
constexpr uint32_t kSmemStack = PT_SMEM_STACK;
// the same for the 8-wide traversal kernels
#ifndef PT_WIDE_SMEM_STACK
#define PT_WIDE_SMEM_STACK 8
#endif
constexpr uint32_t kWideSmemStack = PT_WIDE_SMEM_STACK;

// 1: the shared-memory part of a traversal lane's stack holds its top
// entries (a ring); 0: its bottom entries.  Measured slower on the 2.1M
// triangle scene (extend 384 against 369 ms over three 64-spp images: the
// ring's extra shared accesses and branches cost more than the local-memory
// traffic they save), so off by default
#ifndef PT_STACK_RING
#define PT_STACK_RING 0
#endif

// The deferred stack of one traversal lane: 64 entries in the lane's local
// memory, kShared of them in the block's shared memory instead (one column
// per thread, so a warp touches consecutive words).  With PT_STACK_RING the
// shared column is a ring over the top of the stack: entries [lo, sp) live
// there, a push onto a full ring first moves the oldest ring entry to local
// memory, and a pop below lo reads it back from there, so the pushes and pops
// of a traversal moving about one depth stay in shared memory.  reset()
// before each traversal (an any-hit traversal may stop with entries left).
// Otherwise the shared column holds entries 0..kShared-1.
template <uint32_t kThreads, uint32_t kShared>
struct LaneStack {
    uint2* col;  // &shared[threadIdx.x]; ring slot j at col[j * kThreads]
    uint2 deep[64];
#if PT_STACK_RING
    uint32_t lo = 0u;
    PTD void reset() { lo = 0u; }
    PTD void put(uint32_t i, uint2 e) {
        if (kShared == 0u) {
            deep[i & 63u] = e;
            return;
        }
        if (i - lo >= kShared) {  // the ring is full: its oldest entry moves out
            deep[lo & 63u] = col[(lo % kShared) * kThreads];
            lo += 1u;
        }
        col[(i % kShared) * kThreads] = e;
    }
    PTD uint2 get(uint32_t i) {
        if (kShared > 0u && i >= lo) return col[(i % kShared) * kThreads];
        lo = i;
        return deep[i & 63u];
    }
#else
    PTD void reset() {}
    PTD void put(uint32_t i, uint2 e) {
        if (kShared > 0u && i < kShared)
            col[i * kThreads] = e;
        else
            deep[i & 63u] = e;
    }
    PTD uint2 get(uint32_t i) const {
        if (kShared > 0u && i < kShared) return col[i * kThreads];
        return deep[i & 63u];
    }
#endif
};

// the whole stack in local memory
struct LocalStack {
    uint2 deep[64];
    PTD void reset() {}
    PTD void put(uint32_t i, uint2 e) { deep[i & 63u] = e; }
    PTD uint2 get(uint32_t i) const { return deep[i & 63u]; }
};

// 256-bit loads of a child pair (two 32-byte nodes, 64-byte aligned): one
// ld.global.nc.v8 per node instead of two 128-bit loads
#ifndef PT_V8_PAIRS
#define PT_V8_PAIRS 1
#endif
PTD void load_node(const float4* p, float4& lo, float4& hi) {
#if PT_V8_PAIRS
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z), "=f"(hi.w)
        : "l"(p));
#else
    lo = __ldg(p);
    hi = __ldg(p + 1);
#endif
}

// a padded triangle (48 bytes) as one 256-bit and one 128-bit load: the
// 32-byte aligned half comes first for even triangles, second for odd ones
#ifndef PT_V8_TRIS
#define PT_V8_TRIS 0
#endif
// 1: a traversal step that tests one triangle (PT_TRI_PER_STEP) reads its
// data - a child pair, or a triangle padded to 64 bytes - with the same two
// 256-bit loads whichever kind of step the lane runs, so a warp whose lanes
// run both kinds waits for one load, not for two in turn
#ifndef PT_UNIFIED_STEP
#define PT_UNIFIED_STEP 1
#endif
// float4s per padded triangle: 3 (48 bytes), or 4 (64 bytes: one 256-bit and
// one 128-bit load, both aligned; the shape of a child pair, which the
// unified step needs)
#ifndef PT_TRI_STRIDE
#if PT_UNIFIED_STEP
#define PT_TRI_STRIDE 4
#else
#define PT_TRI_STRIDE 3
#endif
#endif
static_assert(!PT_UNIFIED_STEP || PT_TRI_STRIDE == 4, "the unified traversal step reads triangles padded to 64 bytes");
constexpr uint32_t kTriStride = PT_TRI_STRIDE;
PTD Tri load_tri4(const Fast& f, uint32_t tri) {
    const float4* p = f.tri4 + kTriStride * (size_t)tri;
#if PT_TRI_STRIDE == 4
    float4 a, b;
    load_node(p, a, b);
    const float4 c = __ldg(p + 2);
#elif PT_V8_TRIS
    const bool odd = tri & 1u;
    float4 w0, w1;
    load_node(p + (odd ? 1 : 0), w0, w1);
    const float4 x = __ldg(p + (odd ? 0 : 2));
    const float4 a = odd ? x : w0, b = odd ? w0 : w1, c = odd ? w1 : x;
#else
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
#endif
    Tri t;
    t.v0 = mk(a.x, a.y, a.z);
    t.v1 = mk(b.x, b.y, b.z);
    t.v2 = mk(c.x, c.y, c.z);
    return t;
}

// 1: after a closest-hit traversal step that did not finish, the lane
// prefetches into L1 what its next step loads (the next child pair or
// triangle), and a shadow lane that waits a majority step prefetches its
// next step's data: the load is issued while the warp runs the other branch
// for its other lanes.  The address is the one the next step reads, so it
// is always inside the arrays.  Measured slower on the 2.1M-triangle scene
// (1920x1080x64: 1648 against 1691 Mrays/s, extend +2.7 %, shadow +7 %; the
// L1 is already busy with the loads themselves), so off by default
#ifndef PT_PREFETCH
#define PT_PREFETCH 0
#endif
PTD void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

PTD float box_test(float4 lo, float4 hi, f3 nod, f3 rcp, float hit_t) {
    const float bmin[3] = {lo.x, lo.y, lo.z}, bmax[3] = {hi.x, hi.y, hi.z};
    return intersect_aabb(bmin, bmax, nod, rcp, hit_t);
}

// One ray's traversal (trace.slang:764-884 closest hit, or 614-717 any hit
// when kShadow) on the aligned child-pair layout, as a state machine advanced
// one node visit per step().  The deferred stack holds the (left_first,
// tri_count) of each node, so a pop needs no memory access.  Node visits
// happen in exactly the reference's order.  The stacks live outside the
// object so its scalar state can stay in registers.
template <bool kRec, bool kAlpha, bool kShadow, bool kTri36 = false, bool kTriStep = (PT_TRI_PER_STEP != 0)>
struct Traverser {
    f3 o, d, rcp, nod;
    Shear s;
    float hit_t, hv, hw;
    int32_t hit, light_tri;
    uint32_t lf, tc, sp, idx;
    uint32_t tri_left;  // triangles of the current leaf still to test (PT_TRI_PER_STEP)
    Rng<kRec> rng;
    Counters c;
    Rec<kRec> rec;

    PTD void init(const Fast& f, f3 origin, f3 dir, float t_max, int32_t light) {
        o = origin;
        d = dir;
        rcp = 1.0f / d;
        s = make_shear(d, rcp);
        nod = -o * rcp;
        hit_t = t_max;
        hv = hw = 0.0f;
        hit = -1;
        light_tri = light;
        sp = 0u;
        idx = 0u;
        tri_left = 0u;
        lf = __float_as_uint(__ldg(&f.pairs[0].w));
        tc = __float_as_uint(__ldg(&f.pairs[1].w));
        if constexpr (kRec) {
            rec.c = &c;
            rng.rec.c = &c;
            if constexpr (kShadow) {
                rec.shadow = true;
                c.shadow_rays += 1;
            } else {
                c.extend_rays += 1;
            }
        }
    }

    template <class S>
    PTD bool pop(S& stack, uint32_t* istack) {
        if (sp == 0u) return true;
        sp -= 1u;
        const uint2 e = stack.get(sp);
        lf = e.x;
        tc = e.y;
        if constexpr (kRec) idx = istack[sp & 63u];
        return false;
    }

    // the watertight test of one triangle against the ray; for kShadow true
    // when the triangle occludes
    PTD bool test_triangle(const World& w, const Fast& f, uint32_t tri) {
        Tri tv;
        if constexpr (kTri36)
            tv = load_tri(w, tri);  // the caller's 36-byte triangles
        else
            tv = load_tri4(f, tri);
        return test_loaded(w, tri, tv);
    }
    // the same with the triangle's vertices already loaded
    PTD bool test_loaded(const World& w, uint32_t tri, const Tri& tv) {
        rec.tri();
        float t, v, wb;
        if (!triangle_test(tv, o, s, &t, &v, &wb)) return false;
        if (t > 0.0f && t < hit_t) {
            if constexpr (kAlpha) {
                if (passes_through(w, tri, v, wb, rng)) return false;
            }
            if constexpr (kShadow) {
                hit = 1;
                return true;
            } else {
                hit_t = t;
                hit = (int32_t)tri;
                hv = v;
                hw = wb;
            }
        }
        return false;
    }

    // whether the next step() is an interior visit (else a triangle test, or
    // a whole leaf)
    PTD bool next_is_interior() const { return kTriStep ? (tri_left == 0u && tc == 0u) : tc == 0u; }

    // kTriStep: one interior visit or one triangle of a leaf per step, else
    // one interior visit or a whole leaf
    // prefetch what the next step loads: a leaf under way or about to start:
    // its next triangle; else the next child pair (only while the traversal
    // has not finished, so lf indexes a node pair or a triangle of a leaf)
    PTD void prefetch_next(const Fast& f) const {
#if PT_PREFETCH
        if constexpr (!kTri36) {
            if (tri_left > 0u || tc > 0u)
                prefetch_l1(f.tri4 + kTriStride * (size_t)lf);
            else
                prefetch_l1(f.pairs + 2 * (size_t)lf);
        }
#endif
    }

    template <class S>
    PTD bool step(const World& w, const Fast& f, S& stack, uint32_t* istack) {
        if constexpr (kTriStep && PT_UNIFIED_STEP && !kTri36) {
            return step_unified(w, f, stack, istack);
        } else if constexpr (kTriStep) {
            const bool done = step_tri(w, f, stack, istack);
            if (!done) prefetch_next(f);
            return done;
        } else {
            return step_leaf(w, f, stack, istack);
        }
    }


    // one interior node visit or one triangle test; true when the traversal
    // has finished (for kShadow, hit == 1 marks an occluder).  Testing a
    // leaf's triangles one per step keeps the two divergent paths of a warp
    // (box pair vs triangle) about equally long.
    template <class S>
    PTD bool step_tri(const World& w, const Fast& f, S& stack, uint32_t* istack) {
        if (tri_left == 0u) {
            rec.visit(idx);
            if (tc == 0u) {
                rec.interior();
                const float4* p = f.pairs + 2 * (size_t)lf;
                float4 l0, l1, r0, r1;
                load_node(p, l0, l1);
                load_node(p + 2, r0, r1);
                const float dl = box_test(l0, l1, nod, rcp, hit_t);
                const float dr = box_test(r0, r1, nod, rcp, hit_t);
                const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
                if (hl || hr) {
                    const bool go_left = hl && (!hr || dl < dr);
                    if (hl && hr) {
                        const float4 f0 = go_left ? r0 : l0, f1 = go_left ? r1 : l1;
                        stack.put(sp, make_uint2(__float_as_uint(f0.w), __float_as_uint(f1.w)));
                        if constexpr (kRec) istack[sp & 63u] = go_left ? lf + 1u : lf;
                        sp += 1u;
                    }
                    const float4 n0 = go_left ? l0 : r0, n1 = go_left ? l1 : r1;
                    if constexpr (kRec) idx = go_left ? lf : lf + 1u;
                    lf = __float_as_uint(n0.w);
                    tc = __float_as_uint(n1.w);
                    return false;
                }
                return pop(stack, istack);
            }
            rec.leaf();
            tri_left = tc;  // lf walks the leaf's triangles
        }
        const uint32_t tri = lf;
        lf += 1u;
        tri_left -= 1u;
        bool skip = false;
        if constexpr (kShadow) skip = (int32_t)tri == light_tri;
        if (!skip && test_triangle(w, f, tri)) return true;
        if (tri_left > 0u) return false;
        return pop(stack, istack);
    }
    // step_tri with one load for both kinds of step: the lane's next child
    // pair (interior) or next triangle (64-byte padded layout) is read by the
    // same two 256-bit loads before the branch, so the warp's interior lanes
    // and triangle lanes wait for memory together.  The same visits, tests
    // and stack operations as step_tri, in the same order.
    template <class S>
    PTD bool step_unified(const World& w, const Fast& f, S& stack, uint32_t* istack) {
        if (tri_left == 0u) {
            rec.visit(idx);
            if (tc != 0u) {
                rec.leaf();
                tri_left = tc;  // lf walks the leaf's triangles
            } else {
                rec.interior();
            }
        }
        const bool interior = tri_left == 0u;
        const float4* p = interior ? f.pairs + 2 * (size_t)lf : f.tri4 + kTriStride * (size_t)lf;
        float4 a0, a1, b0, b1;
        load_node(p, a0, a1);
        load_node(p + 2, b0, b1);
        if (interior) {
            const float dl = box_test(a0, a1, nod, rcp, hit_t);
            const float dr = box_test(b0, b1, nod, rcp, hit_t);
            const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
            if (hl || hr) {
                const bool go_left = hl && (!hr || dl < dr);
                if (hl && hr) {
                    const float4 f0 = go_left ? b0 : a0, f1 = go_left ? b1 : a1;
                    stack.put(sp, make_uint2(__float_as_uint(f0.w), __float_as_uint(f1.w)));
                    if constexpr (kRec) istack[sp & 63u] = go_left ? lf + 1u : lf;
                    sp += 1u;
                }
                const float4 n0 = go_left ? a0 : b0, n1 = go_left ? a1 : b1;
                if constexpr (kRec) idx = go_left ? lf : lf + 1u;
                lf = __float_as_uint(n0.w);
                tc = __float_as_uint(n1.w);
                return false;
            }
            return pop(stack, istack);
        }
        const uint32_t tri = lf;
        lf += 1u;
        tri_left -= 1u;
        bool skip = false;
        if constexpr (kShadow) skip = (int32_t)tri == light_tri;
        Tri tv;
        tv.v0 = mk(a0.x, a0.y, a0.z);
        tv.v1 = mk(a1.x, a1.y, a1.z);
        tv.v2 = mk(b0.x, b0.y, b0.z);
        if (!skip && test_loaded(w, tri, tv)) return true;
        if (tri_left > 0u) return false;
        return pop(stack, istack);
    }

    // one node visit; true when the traversal has finished (for kShadow,
    // hit == 1 marks an occluder)
    template <class S>
    PTD bool step_leaf(const World& w, const Fast& f, S& stack, uint32_t* istack) {
        rec.visit(idx);
        if (tc > 0u) {
            rec.leaf();
            for (uint32_t i = 0; i < tc; ++i) {
                const uint32_t tri = lf + i;
                if constexpr (kShadow) {
                    if ((int32_t)tri == light_tri) continue;
                }
                rec.tri();
                float t, v, wb;
                Tri tv;
                if constexpr (kTri36)
                    tv = load_tri(w, tri);  // the caller's 36-byte triangles
                else
                    tv = load_tri4(f, tri);
                if (!triangle_test(tv, o, s, &t, &v, &wb)) continue;
                if (t > 0.0f && t < hit_t) {
                    if constexpr (kAlpha) {
                        if (passes_through(w, tri, v, wb, rng)) continue;
                    }
                    if constexpr (kShadow) {
                        hit = 1;
                        return true;
                    } else {
                        hit_t = t;
                        hit = (int32_t)tri;
                        hv = v;
                        hw = wb;
                    }
                }
            }
        } else {
            rec.interior();
            const float4* p = f.pairs + 2 * (size_t)lf;
            float4 l0, l1, r0, r1;
            load_node(p, l0, l1);
            load_node(p + 2, r0, r1);
            const float dl = box_test(l0, l1, nod, rcp, hit_t);
            const float dr = box_test(r0, r1, nod, rcp, hit_t);
            const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
            if (hl || hr) {
                const bool go_left = hl && (!hr || dl < dr);
                if (hl && hr) {
                    const float4 f0 = go_left ? r0 : l0, f1 = go_left ? r1 : l1;
                    stack.put(sp, make_uint2(__float_as_uint(f0.w), __float_as_uint(f1.w)));
                    if constexpr (kRec) istack[sp & 63u] = go_left ? lf + 1u : lf;
                    sp += 1u;
                }
                const float4 n0 = go_left ? l0 : r0, n1 = go_left ? l1 : r1;
                if constexpr (kRec) idx = go_left ? lf : lf + 1u;
                lf = __float_as_uint(n0.w);
                tc = __float_as_uint(n1.w);
                return false;
            }
        }
        return pop(stack, istack);
    }
};

// Sort 8 keys ascending (a 19-comparator network: no dynamic indexing, so the
// keys stay in registers).
PTD void sort8(uint32_t (&k)[8]) {
#define PT_CE(a, b)                                  \
    {                                                \
        const uint32_t lo_ = umin(k[a], k[b]);       \
        const uint32_t hi_ = umax(k[a], k[b]);       \
        k[a] = lo_;                                  \
        k[b] = hi_;                                  \
    }
    PT_CE(0, 2) PT_CE(1, 3) PT_CE(4, 6) PT_CE(5, 7)
    PT_CE(0, 4) PT_CE(1, 5) PT_CE(2, 6) PT_CE(3, 7)
    PT_CE(0, 1) PT_CE(2, 3) PT_CE(4, 5) PT_CE(6, 7)
    PT_CE(2, 4) PT_CE(3, 5)
    PT_CE(1, 4) PT_CE(3, 6)
    PT_CE(1, 2) PT_CE(3, 4) PT_CE(5, 6)
#undef PT_CE
}

// Whether the reference's binary traversal (trace.slang:786-884) reaches
// triangle a before triangle b on this ray: in one leaf the lower index
// first; otherwise at their lowest common ancestor the child the traversal
// enters first (the nearer accepted child box, ties to the right).  Used
// only to break exact-t ties the way the reference does (its `t < hit_t`
// keeps the first triangle found).
PTD bool binary_first(const Fast& f, f3 o, f3 d, uint32_t a, uint32_t b) {
    uint32_t la = __ldg(f.leaf_of + a), lb = __ldg(f.leaf_of + b);
    if (la == lb) return a < b;
    const auto depth = [&](uint32_t n) {
        uint32_t k = 0;
        while (n != 0u && k < 64u) {
            n = __ldg(f.parent + n);
            ++k;
        }
        return k;
    };
    uint32_t da = depth(la), db = depth(lb);
    for (; da > db; --da) la = __ldg(f.parent + la);
    for (; db > da; --db) lb = __ldg(f.parent + lb);
    for (uint32_t k = 0; k < 64u; ++k) {
        const uint32_t pa = __ldg(f.parent + la), pb = __ldg(f.parent + lb);
        if (pa == pb) break;
        la = pa;
        lb = pb;
    }
    // la, lb: the two children of the common ancestor, la on a's side
    const uint32_t left = la < lb ? la : lb;
    const f3 rcp = 1.0f / d, nod = -o * rcp;
    const float4* p = f.pairs + 2 * (size_t)left;
    const float inf = __int_as_float(0x7f800000);
    const float dl = box_test(__ldg(p), __ldg(p + 1), nod, rcp, inf);
    const float dr = box_test(__ldg(p + 2), __ldg(p + 3), nod, rcp, inf);
    const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
    const bool go_left = hl && (!hr || dl < dr);
    return (la == left) == go_left;
}

// One ray's traversal of the 8-wide BVH of the precision form
// (include/pt_precision.h), with the same step()/result interface as
// Traverser.  A visit decodes the node's child boxes exactly as the host
// quantised them (origin + q * 2^e: the product exact, one rounding) and runs
// the reference's slab test (trace.slang:597-609) on them; an axis whose
// direction component is zero constrains nothing (the binary test's value is
// then not a bound: 0 * inf).  The accepted children are visited in the
// order of their slots XOR the ray's direction octant (the builder places
// them for that order; PT_WIDE_OCTANT 0 sorts them by entry distance
// instead); the deferred stack holds (node, children still to visit), one
// entry per level.  A leaf's triangles are tested with the reference's
// watertight test, so a hit's (t, v, w) are the binary traversal's for the
// same triangle.  Opaque scenes only.
// One axis of a wide node in the ray's frame.  A child bound q (8 bits) is
// placed into the float v = 1 + q 2^-15 with one byte permute, and its slab
// distance is t = fma(v, a15, c): a15 = 2^(e+15) rcp and c = B - a15 with
// B = fma(origin, rcp, -o rcp), so t = B + q 2^e rcp up to rounding.  The
// near bound (the box minimum when rcp >= 0, else the maximum) uses
// c - eps, the far bound c + eps, with eps = 2^-19 (|B| + |a15| + |o rcp|):
// more than the sum of the rounding errors of this form, of the
// reference's slab test on the binary box (trace.slang:597-609), and of the
// box decode (each at most a few units of 2^-24 of those magnitudes).  So the
// wide interval contains the interval the reference computes for every
// binary node under the child, and a box the reference accepts is accepted.
// An axis the ray does not move along (rcp = 0 here) constrains nothing.
struct AxisFrame {
    float a15, c_near, c_far;
    uint32_t near0, near1, far0, far1;  // bound bytes of children 0-3 / 4-7
};
PTD AxisFrame axis_frame(float origin, uint32_t ebyte, float rcp_a, float nod_a, uint32_t lo0, uint32_t lo1,
                         uint32_t hi0, uint32_t hi1) {
    AxisFrame f;
    const bool neg = rcp_a < 0.0f;
    f.near0 = neg ? hi0 : lo0;
    f.near1 = neg ? hi1 : lo1;
    f.far0 = neg ? lo0 : hi0;
    f.far1 = neg ? lo1 : hi1;
    if (rcp_a == 0.0f) {
        const float inf = __int_as_float(0x7f800000);
        f.a15 = 0.0f;
        f.c_near = -inf;
        f.c_far = inf;
        return f;
    }
    const float s15 = __uint_as_float((ebyte + 15u) << 23);  // 2^(e + 15)
    f.a15 = s15 * rcp_a;
    const float b = fmaf(origin, rcp_a, nod_a);
    const float c0 = b - f.a15;
    const float eps = (fabsf(b) + fabsf(f.a15) + fabsf(nod_a)) * 0x1p-19f;
    f.c_near = c0 - eps;
    f.c_far = c0 + eps;
    return f;
}
// v = 1 + q 2^-15 for the bound byte of child i (bytes: 0, q, 0x80, 0x3F)
template <int i>
PTD float bound_v(uint32_t w0, uint32_t w1) {
    return __uint_as_float(__byte_perm(i < 4 ? w0 : w1, 0x3F800000u, 0x7604u | ((unsigned)(i & 3) << 4)));
}

// 1: the 8-wide child test evaluates a child's near and far slab distance
// on one axis with one packed FP32 fma (fma.rn.f32x2, sm_100 and later: each
// half rounds as one fma.rn, so the distances are the same bits); 0: one fma
// per distance.  Measured slower on the 2.1M-triangle scene (compressed form,
// 1920x1080x64: 1514 against 1535 Mrays/s, wide extend 442 against 429 ms
// over three images; the packed operands cost registers and 40 B of spills),
// so off by default
#ifndef PT_WIDE_FMA2
#define PT_WIDE_FMA2 0
#endif
PTD unsigned long long pack2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
PTD float2 unpack2(unsigned long long v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
PTD unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

template <bool kShadow, bool kTri36 = false>
struct WideTraverser {
    f3 o, d, rcp, nod;
    Shear s;
    float hit_t, hv, hw;
    int32_t hit, light_tri;
    // list: the accepted children still to visit in the current node (with
    // PT_WIDE_OCTANT a mask in bits 0..7 and the ray's direction octant, bit a
    // set when d[a] < 0, in bits 8..10)
    uint32_t node, list, lf, tri_left, sp;
    Rng<false> rng;  // unused (no alpha draws in the wide form)
    Counters c;      // unused (no records in the wide form)

    PTD void init(const Fast& f, f3 origin, f3 dir, float t_max, int32_t light) {
        o = origin;
        d = dir;
        rcp = 1.0f / d;
        s = make_shear(d, rcp);
        nod = -o * rcp;
        // an axis the ray does not move along: the slab test's 0 * inf is not a
        // bound, so the axis is left unconstrained
        const float inf = __int_as_float(0x7f800000);
        if (fabsf(rcp.x) == inf) { rcp.x = 0.0f; nod.x = 0.0f; }
        if (fabsf(rcp.y) == inf) { rcp.y = 0.0f; nod.y = 0.0f; }
        if (fabsf(rcp.z) == inf) { rcp.z = 0.0f; nod.z = 0.0f; }
        hit_t = t_max;
        hv = hw = 0.0f;
        hit = -1;
        light_tri = light;
        sp = 0u;
        tri_left = 0u;
        node = 0u;
#if PT_WIDE_OCTANT
        const uint32_t oct =
            (__float_as_uint(d.x) >> 31) | ((__float_as_uint(d.y) >> 31) << 1) | ((__float_as_uint(d.z) >> 31) << 2);
        list = visit(f, 0u, oct) | (oct << 8);
#else
        list = visit(f, 0u);
#endif
    }

#if PT_WIDE_OCTANT
    // the accepted children of node n as a mask: child slot i sets bit i ^ oct,
    // so the lowest set bit is the next child in the octant order.  A child is
    // accepted when max(near bounds, 0) <= min(far bounds, hit_t): every ray
    // the slab test of trace.slang:597-609 accepts on the binary box (plus the
    // boundary cases t_far = 0 and t_near = hit_t, which change no result)
    PTD uint32_t visit(const Fast& f, uint32_t n, uint32_t oct) const {
        const float4* p = f.wide + 8 * (size_t)n;
        float4 h0, h1, h2, h3;
        load_node(p, h0, h1);
        load_node(p + 2, h2, h3);
        const uint32_t meta = __float_as_uint(h0.w);
        const uint32_t count = meta >> 24;
        const AxisFrame X = axis_frame(h0.x, meta & 0xffu, rcp.x, nod.x, __float_as_uint(h1.x), __float_as_uint(h1.y),
                                       __float_as_uint(h2.z), __float_as_uint(h2.w));
        const AxisFrame Y = axis_frame(h0.y, (meta >> 8) & 0xffu, rcp.y, nod.y, __float_as_uint(h1.z),
                                       __float_as_uint(h1.w), __float_as_uint(h3.x), __float_as_uint(h3.y));
        const AxisFrame Z = axis_frame(h0.z, (meta >> 16) & 0xffu, rcp.z, nod.z, __float_as_uint(h2.x),
                                       __float_as_uint(h2.y), __float_as_uint(h3.z), __float_as_uint(h3.w));
        uint32_t mask = 0u;
#if PT_WIDE_FMA2
        // the accept test of one child from its six slab distances
        const auto accept = [&](int i, float nx, float ny, float nz, float fx, float fy, float fz) {
#if PT_WIDE_MINMAX3
            const float t_near = max3f(nx, ny, fmaxf(nz, 0.0f));
            const float t_far = min3f(fx, fy, fminf(fz, hit_t));
#else
            const float t_near = fmaxf(fmaxf(nx, ny), fmaxf(nz, 0.0f));
            const float t_far = fminf(fminf(fx, fy), fminf(fz, hit_t));
#endif
            if (t_near <= t_far) mask |= 1u << i;
        };
        // per axis (a15, a15) and (c_near, c_far): one packed fma gives a child's near and far distance
        const unsigned long long xa = pack2(X.a15, X.a15), xc = pack2(X.c_near, X.c_far);
        const unsigned long long ya = pack2(Y.a15, Y.a15), yc = pack2(Y.c_near, Y.c_far);
        const unsigned long long za = pack2(Z.a15, Z.a15), zc = pack2(Z.c_near, Z.c_far);
        const auto child = [&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const float2 x = unpack2(fma2(pack2(bound_v<i>(X.near0, X.near1), bound_v<i>(X.far0, X.far1)), xa, xc));
            const float2 y = unpack2(fma2(pack2(bound_v<i>(Y.near0, Y.near1), bound_v<i>(Y.far0, Y.far1)), ya, yc));
            const float2 z = unpack2(fma2(pack2(bound_v<i>(Z.near0, Z.near1), bound_v<i>(Z.far0, Z.far1)), za, zc));
            accept(i, x.x, y.x, z.x, x.y, y.y, z.y);
        };
        child(std::integral_constant<int, 0>());
        child(std::integral_constant<int, 1>());
        child(std::integral_constant<int, 2>());
        child(std::integral_constant<int, 3>());
        child(std::integral_constant<int, 4>());
        child(std::integral_constant<int, 5>());
        child(std::integral_constant<int, 6>());
        child(std::integral_constant<int, 7>());
#else
        const auto child = [&](auto ic) {
            constexpr int i = decltype(ic)::value;
            const float nx = fmaf(bound_v<i>(X.near0, X.near1), X.a15, X.c_near);
            const float ny = fmaf(bound_v<i>(Y.near0, Y.near1), Y.a15, Y.c_near);
            const float nz = fmaf(bound_v<i>(Z.near0, Z.near1), Z.a15, Z.c_near);
            const float fx = fmaf(bound_v<i>(X.far0, X.far1), X.a15, X.c_far);
            const float fy = fmaf(bound_v<i>(Y.far0, Y.far1), Y.a15, Y.c_far);
            const float fz = fmaf(bound_v<i>(Z.far0, Z.far1), Z.a15, Z.c_far);
#if PT_WIDE_MINMAX3
            const float t_near = max3f(nx, ny, fmaxf(nz, 0.0f));
            const float t_far = min3f(fx, fy, fminf(fz, hit_t));
#else
            const float t_near = fmaxf(fmaxf(nx, ny), fmaxf(nz, 0.0f));
            const float t_far = fminf(fminf(fx, fy), fminf(fz, hit_t));
#endif
#if PT_WIDE_MASK_PERMUTE
            if (t_near <= t_far) mask |= 1u << i;
#else
            if ((uint32_t)i < count && t_near <= t_far) mask |= 1u << ((uint32_t)i ^ oct);
#endif
        };
        child(std::integral_constant<int, 0>());
        child(std::integral_constant<int, 1>());
        child(std::integral_constant<int, 2>());
        child(std::integral_constant<int, 3>());
        child(std::integral_constant<int, 4>());
        child(std::integral_constant<int, 5>());
        child(std::integral_constant<int, 6>());
        child(std::integral_constant<int, 7>());
#endif
#if PT_WIDE_MASK_PERMUTE || PT_WIDE_FMA2
        // slot order -> octant order: bit i moves to bit i ^ oct
        mask &= (1u << count) - 1u;
        if (oct & 1u) mask = ((mask & 0x55u) << 1) | ((mask >> 1) & 0x55u);
        if (oct & 2u) mask = ((mask & 0x33u) << 2) | ((mask >> 2) & 0x33u);
        if (oct & 4u) mask = ((mask & 0x0fu) << 4) | ((mask >> 4) & 0x0fu);
#endif
        return mask;
    }
#else
    // the hit children of node n as 3-bit indices (nearest first unless
    // kShadow) in bits 0..23, their count in bits 24..27
    PTD uint32_t visit(const Fast& f, uint32_t n) const {
        const float4* p = f.wide + 8 * (size_t)n;
        float4 h0, h1, h2, h3;
        load_node(p, h0, h1);
        load_node(p + 2, h2, h3);
        const uint32_t meta = __float_as_uint(h0.w);
        const uint32_t count = meta >> 24;
        const AxisFrame X = axis_frame(h0.x, meta & 0xffu, rcp.x, nod.x, __float_as_uint(h1.x), __float_as_uint(h1.y),
                                       __float_as_uint(h2.z), __float_as_uint(h2.w));
        const AxisFrame Y = axis_frame(h0.y, (meta >> 8) & 0xffu, rcp.y, nod.y, __float_as_uint(h1.z),
                                       __float_as_uint(h1.w), __float_as_uint(h3.x), __float_as_uint(h3.y));
        const AxisFrame Z = axis_frame(h0.z, (meta >> 16) & 0xffu, rcp.z, nod.z, __float_as_uint(h2.x),
                                       __float_as_uint(h2.y), __float_as_uint(h3.z), __float_as_uint(h3.w));
        uint32_t k[8];
        const auto child = [&](auto ic) {
            constexpr int i = decltype(ic)::value;
            k[i] = 0xffffffffu;
            if ((uint32_t)i >= count) return;
            const float nx = fmaf(bound_v<i>(X.near0, X.near1), X.a15, X.c_near);
            const float ny = fmaf(bound_v<i>(Y.near0, Y.near1), Y.a15, Y.c_near);
            const float nz = fmaf(bound_v<i>(Z.near0, Z.near1), Z.a15, Z.c_near);
            const float fx = fmaf(bound_v<i>(X.far0, X.far1), X.a15, X.c_far);
            const float fy = fmaf(bound_v<i>(Y.far0, Y.far1), Y.a15, Y.c_far);
            const float fz = fmaf(bound_v<i>(Z.far0, Z.far1), Z.a15, Z.c_far);
            const float t_near = fmaxf(fmaxf(nx, ny), nz);
            const float t_far = fminf(fminf(fx, fy), fz);
            if (t_near <= t_far && t_far > 0.0f && t_near < hit_t) {
                if constexpr (kShadow)
                    k[i] = (uint32_t)i;
                else
                    k[i] = (__float_as_uint(fmaxf(0.0f, t_near)) & ~7u) | (uint32_t)i;
            }
        };
        child(std::integral_constant<int, 0>());
        child(std::integral_constant<int, 1>());
        child(std::integral_constant<int, 2>());
        child(std::integral_constant<int, 3>());
        child(std::integral_constant<int, 4>());
        child(std::integral_constant<int, 5>());
        child(std::integral_constant<int, 6>());
        child(std::integral_constant<int, 7>());
        if constexpr (!kShadow) sort8(k);
        uint32_t l = 0u, cnt = 0u;
#pragma unroll
        for (int i = 7; i >= 0; --i)
            if (k[i] != 0xffffffffu) {
                l = (l << 3) | (k[i] & 7u);
                ++cnt;
            }
        return l | (cnt << 24);
    }
#endif

    PTD bool test_triangle(const World& w, const Fast& f, uint32_t tri) {
        float t, v, wb;
        Tri tv;
        if constexpr (kTri36)
            tv = load_tri(w, tri);
        else
            tv = load_tri4(f, tri);
        if (!triangle_test(tv, o, s, &t, &v, &wb)) return false;
        if (t > 0.0f && t < hit_t) {
            if constexpr (kShadow) {
                hit = 1;
                return true;
            } else {
                hit_t = t;
                hit = (int32_t)tri;
                hv = v;
                hw = wb;
            }
        } else if (!kShadow && t == hit_t && hit >= 0 && binary_first(f, o, d, tri, (uint32_t)hit)) {
            // an exact tie: keep the triangle the binary traversal finds first
            hit = (int32_t)tri;
            hv = v;
            hw = wb;
        }
        return false;
    }

    // one node visit or one triangle test; true when the traversal has finished
    template <class S>
    PTD bool step(const World& w, const Fast& f, S& stack, uint32_t*) {
        if (tri_left == 0u) {
#if PT_WIDE_OCTANT
            if ((list & 0xffu) == 0u) {
                if (sp == 0u) return true;
                sp -= 1u;
                const uint2 e = stack.get(sp);
                node = e.x;
                list = e.y;
            }
            const uint32_t oct = list >> 8;
            const uint32_t k = (uint32_t)(__ffs(list) - 1) ^ oct;
            list &= list - 1u;  // the lowest set bit is in the mask: it is not empty
            const bool more = (list & 0xffu) != 0u;
#else
            uint32_t cnt = list >> 24;
            if (cnt == 0u) {
                if (sp == 0u) return true;
                sp -= 1u;
                const uint2 e = stack.get(sp);
                node = e.x;
                list = e.y;
                cnt = list >> 24;
            }
            const uint32_t k = list & 7u;
            list = ((list & 0xffffffu) >> 3) | ((cnt - 1u) << 24);
            const bool more = cnt > 1u;
#endif
            const float4* p = f.wide + 8 * (size_t)node;
            const uint32_t child = __ldg(reinterpret_cast<const uint32_t*>(p + 4) + k);
            const uint32_t tc = __ldg(reinterpret_cast<const unsigned short*>(p + 6) + k);
            if (tc == 0u) {
                if (more) {
                    stack.put(sp, make_uint2(node, list));
                    sp += 1u;
                }
                node = child;
#if PT_WIDE_OCTANT
                list = visit(f, child, oct) | (oct << 8);
#else
                list = visit(f, child);
#endif
                return false;
            }
            lf = child;
            tri_left = tc;
        }
#if PT_WIDE_TRI_PER_STEP
        const uint32_t tri = lf;
        lf += 1u;
        tri_left -= 1u;
        bool skip = false;
        if constexpr (kShadow) skip = (int32_t)tri == light_tri;
        return !skip && test_triangle(w, f, tri);
#else
        for (; tri_left > 0u; --tri_left, ++lf) {
            if (kShadow && (int32_t)lf == light_tri) continue;
            if (test_triangle(w, f, lf)) return true;
        }
        return false;
#endif
    }
};

constexpr int kStepsPerRefill = PT_STEPS_PER_REFILL;
// steps between refills of the 8-wide traversal (its steps are longer)
#ifndef PT_WIDE_STEPS_PER_REFILL
#define PT_WIDE_STEPS_PER_REFILL 8
#endif
constexpr int kWideStepsPerRefill = PT_WIDE_STEPS_PER_REFILL;
constexpr unsigned kRefillBelow = PT_REFILL_BELOW;

PTD unsigned lane_id() {
    unsigned l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

// warp-aggregated append: one atomic per warp, slots in lane order
PTD uint32_t warp_append(bool want, uint32_t* counter, unsigned mask) {
    const unsigned ballot = __ballot_sync(mask, want);
    if (ballot == 0u) return 0xffffffffu;
    const unsigned lane = lane_id();
    const unsigned leader = (unsigned)(__ffs(ballot) - 1);
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(ballot));
    base = __shfl_sync(mask, base, leader);
    return want ? base + (uint32_t)__popc(ballot & ((1u << lane) - 1u)) : 0xffffffffu;
}

// Files finished extend rays' queue slots under hits or misses, so that the
// shading kernel runs warps of hits only and warps of misses only.  Lanes
// finish at different steps, so a finishing lane only appends to its warp's
// buffer in shared memory; the warp flushes the buffer to the global lists
// once per refill round (one global atomic per list and round).  A lane
// finishes at most one ray per round, so 32 entries per list suffice.
struct ResultFiler {
    uint32_t* buf;   // this warp's [3][32] in shared memory: hits, misses, the hits' sort keys
    uint32_t* fill;  // this warp's [2] entry counts
    PTD void file(uint32_t slot, bool is_hit, uint32_t key = 0u) {
        const uint32_t b = is_hit ? 0u : 1u;
        const uint32_t j = atomicAdd(&fill[b], 1u);
        buf[b * 32u + j] = slot;
        if (is_hit) buf[64u + j] = key;
    }
    // all 32 lanes, converged
    PTD void flush(const Queues& q, unsigned lane) {
        __syncwarp();
        const uint32_t nh = fill[0], nm = fill[1];
        uint32_t bh = 0, bm = 0;
        if (lane == 0u) {
            if (nh) bh = atomicAdd(&q.cnt[5], nh);
            if (nm) bm = atomicAdd(&q.cnt[6], nm);
        }
        bh = __shfl_sync(0xffffffffu, bh, 0);
        bm = __shfl_sync(0xffffffffu, bm, 0);
        if (lane < nh) {
            q.hit_list[bh + lane] = buf[lane];
            if (q.hit_keys) q.hit_keys[bh + lane] = buf[64u + lane];
        }
        if (lane < nm) q.miss_list[bm + lane] = buf[32u + lane];
        __syncwarp();
        if (lane == 0u) fill[0] = fill[1] = 0u;
        __syncwarp();
    }
};

// shared-memory buffers of the ResultFilers of one extend block
template <int kThreads>
struct FilerSlots {
    uint32_t buf[kThreads / 32][96];
    uint32_t fill[kThreads / 32][2];
    PTD ResultFiler of_warp(unsigned lane) {
        const unsigned wi = threadIdx.x >> 5;
        if (lane == 0u) fill[wi][0] = fill[wi][1] = 0u;
        __syncwarp();
        return ResultFiler{buf[wi], fill[wi]};
    }
};

struct NoRound {
    PTD void operator()() const {}
};

// 1: in opaque scenes a shading step adds exactly one radiance term to its
// path's colour (the sky at a miss, trace.slang:925; emission at a hit,
// :991; the next-event light of :1204 arrives later through the shadow
// kernel), so the shading kernel starts from zero, and reads and rewrites
// the path's colour only when that term is not zero.  Same bits: the colour
// starts at +0 and is only ever a sum, so it is never -0, and
// colour + (+-0) = colour.  Non-opaque scenes add the unoccluded light in
// the same step (two terms), so they keep the read-modify-write of the
// running colour.
#ifndef PT_COLOR_DELTA
#define PT_COLOR_DELTA 1
#endif
template <bool kAlpha>
constexpr bool kColorDelta = PT_COLOR_DELTA && !kAlpha;

// the path's colour after a shading step: `c` is the new colour, or with
// kColorDelta the term the step added (0 + term)
template <bool kAlpha>
PTD void store_color(float4* color, uint32_t p, f3 c) {
    if constexpr (kColorDelta<kAlpha>) {
        if (c.x != 0.0f || c.y != 0.0f || c.z != 0.0f) {
            const float4 old = color[p];
            color[p] = make_float4(old.x + c.x, old.y + c.y, old.z + c.z, 0.0f);
        }
    } else {
        color[p] = make_float4(c.x, c.y, c.z, 0.0f);
    }
}

// The shading kernels' view of the filed results: misses first, padded to
// whole warps, then hits.  Entry j of that range maps to a queue slot.
struct ShadeRange {
    uint32_t n_hit, n_miss, miss_span;
    const uint32_t* hits;
    PTD ShadeRange(const Queues& q)
        : n_hit(q.cnt[5]), n_miss(q.cnt[6]), miss_span((q.cnt[6] + 31u) & ~31u),
          hits(q.cnt[7] ? q.hit_sorted : q.hit_list) {}
    PTD uint32_t count() const { return miss_span + n_hit; }
    // queue slot of entry j, or 0xffffffff for the padding after the misses and past the end
    PTD uint32_t slot(const Queues& q, uint32_t j) const {
        if (j < miss_span) return j < n_miss ? q.miss_list[j] : 0xffffffffu;
        const uint32_t k = j - miss_span;
        return k < n_hit ? hits[k] : 0xffffffffu;
    }
};

// ---- hit sorting before shading: a counting sort of the hit list into
// kSortBuckets keys, so that neighbouring lanes shade hits of the same
// material (key mode 0: material index) or of nearby triangles (mode 1:
// triangle index >> shift; triangles are in BVH order, so nearby in space,
// and mostly of one mesh).  Three passes: block histograms into global
// counts; one block scans the counts into bucket offsets (and clears the
// counts for the next bounce); blocks recount their chunk, reserve each
// key's range with one global atomic and scatter.  Skipped (cnt[7] = 0)
// below min_hits.
#ifndef PT_SORT_BUCKETS
#define PT_SORT_BUCKETS 4096
#endif
constexpr uint32_t kSortBuckets = PT_SORT_BUCKETS;  // a multiple of 1024, at most 8192 (shared memory)
static_assert(kSortBuckets % 1024 == 0 && kSortBuckets <= 8192, "sort buckets: 1024 .. 8192 in steps of 1024");
constexpr uint32_t kSortPerThread = kSortBuckets / 1024;
constexpr int kSortThreads = 256, kSortItems = 8;

template <int kMode>
PTD uint32_t hit_key(const World& w, const Queues& q, uint32_t slot, uint32_t tri_shift) {
    const uint32_t tri = __float_as_uint(__ldg(&q.hit[slot].y));
    if constexpr (kMode == 0) return attr_material(w, tri) & (kSortBuckets - 1u);
    const uint32_t k = tri >> tri_shift;
    return k < kSortBuckets ? k : kSortBuckets - 1u;
}

template <int kMode>
__global__ void __launch_bounds__(kSortThreads) sort_count_kernel(World w, Queues q, uint32_t* counts,
                                                                   uint32_t min_hits, uint32_t tri_shift) {
    __shared__ uint32_t hist[kSortBuckets];
    const uint32_t n = q.cnt[5];
    if (n < min_hits) return;
    for (uint32_t i = threadIdx.x; i < kSortBuckets; i += blockDim.x) hist[i] = 0u;
    __syncthreads();
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        atomicAdd(&hist[kMode == 1 && q.hit_keys ? q.hit_keys[j] : hit_key<kMode>(w, q, q.hit_list[j], tri_shift)],
                  1u);
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kSortBuckets; i += blockDim.x)
        if (hist[i]) atomicAdd(&counts[i], hist[i]);
}

// Ray ordering: the slots of a ray queue (the next bounce's rays, or the
// shadow rays) grouped by direction octant, written to `order`; within an
// octant, slots keep roughly their queue order (which follows the sorted
// hits, so origins stay close).  A warp of the traversal then holds rays
// whose near-child choices agree more often.  Only the processing order
// changes.  `flag` (a counter slot) is 1 when `order` is valid.
PTD uint32_t octant(float4 d) { return (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u); }

// (templates, as the other sort kernels, so that both translation units may include them)
template <int kUnused>
__global__ void __launch_bounds__(kSortThreads) ray_count_kernel(const float4* d, const uint32_t* count,
                                                                 uint32_t* counts, uint32_t min_rays) {
    __shared__ uint32_t hist[8];
    const uint32_t n = *count;
    if (n < min_rays) return;
    if (threadIdx.x < 8) hist[threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
        atomicAdd(&hist[octant(d[j])], 1u);
    __syncthreads();
    if (threadIdx.x < 8 && hist[threadIdx.x]) atomicAdd(&counts[threadIdx.x], hist[threadIdx.x]);
}

template <int kUnused>
__global__ void ray_scan_kernel(const uint32_t* count, uint32_t* counts, uint32_t* offsets, uint32_t* flag,
                                uint32_t min_rays) {
    if (*count < min_rays) {
        *flag = 0u;
        return;
    }
    uint32_t base = 0;
    for (int k = 0; k < 8; ++k) {
        offsets[k] = base;
        base += counts[k];
        counts[k] = 0u;
    }
    *flag = 1u;
}

template <int kUnused>
__global__ void __launch_bounds__(kSortThreads) ray_scatter_kernel(const float4* d, const uint32_t* count,
                                                                   uint32_t* offsets, uint32_t* order,
                                                                   uint32_t min_rays) {
    __shared__ uint32_t hist[8];
    const uint32_t n = *count;
    if (n < min_rays) return;
    const uint32_t chunk = kSortThreads * kSortItems;
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        if (threadIdx.x < 8) hist[threadIdx.x] = 0u;
        __syncthreads();
        uint32_t keys[kSortItems];
#pragma unroll
        for (int k = 0; k < kSortItems; ++k) {
            const uint32_t j = c0 + (uint32_t)k * kSortThreads + threadIdx.x;
            keys[k] = 0xffffffffu;
            if (j < n) {
                keys[k] = octant(d[j]);
                atomicAdd(&hist[keys[k]], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x < 8 && hist[threadIdx.x]) hist[threadIdx.x] = atomicAdd(&offsets[threadIdx.x], hist[threadIdx.x]);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortItems; ++k)
            if (keys[k] != 0xffffffffu) order[atomicAdd(&hist[keys[k]], 1u)] = c0 + (uint32_t)k * kSortThreads + threadIdx.x;
        __syncthreads();
    }
}

// one block of 1024 threads, kSortPerThread buckets each
template <int kUnused>
__global__ void __launch_bounds__(1024) sort_scan_kernel(Queues q, uint32_t* counts, uint32_t* offsets,
                                                          uint32_t min_hits) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x;
    if (q.cnt[5] < min_hits) {
        if (t == 0) q.cnt[7] = 0u;
        return;
    }
    uint32_t c[kSortPerThread], sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kSortPerThread; ++k) {
        c[k] = counts[kSortPerThread * t + k];
        counts[kSortPerThread * t + k] = 0u;
        sum += c[k];
    }
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024u; off <<= 1) {
        const uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t base = part[t] - sum;
#pragma unroll
    for (uint32_t k = 0; k < kSortPerThread; ++k) {
        offsets[kSortPerThread * t + k] = base;
        base += c[k];
    }
    if (t == 0) q.cnt[7] = 1u;
}

template <int kMode>
__global__ void __launch_bounds__(kSortThreads) sort_scatter_kernel(World w, Queues q, uint32_t* offsets,
                                                                     uint32_t min_hits, uint32_t tri_shift) {
    __shared__ uint32_t hist[kSortBuckets];
    const uint32_t n = q.cnt[5];
    if (n < min_hits) return;
    const uint32_t chunk = kSortThreads * kSortItems;
    for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
        for (uint32_t i = threadIdx.x; i < kSortBuckets; i += blockDim.x) hist[i] = 0u;
        __syncthreads();
        uint32_t keys[kSortItems], slots[kSortItems];
#pragma unroll
        for (int k = 0; k < kSortItems; ++k) {
            const uint32_t j = c0 + (uint32_t)k * kSortThreads + threadIdx.x;
            keys[k] = 0xffffffffu;
            if (j < n) {
                slots[k] = q.hit_list[j];
                keys[k] = kMode == 1 && q.hit_keys ? q.hit_keys[j] : hit_key<kMode>(w, q, slots[k], tri_shift);
                atomicAdd(&hist[keys[k]], 1u);
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < kSortBuckets; i += blockDim.x)
            if (hist[i]) hist[i] = atomicAdd(&offsets[i], hist[i]);  // this block's range of key i
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortItems; ++k)
            if (keys[k] != 0xffffffffu) q.hit_sorted[atomicAdd(&hist[keys[k]], 1u)] = slots[k];
        __syncthreads();
    }
}

// The persistent traversal loop of one warp; every lane holds at most one ray.
// Each round the warp counts its busy lanes: when fewer than refill_below are
// busy and the queue still has rays, the idle lanes take the next ones (one
// atomic per warp, queue slots in lane order).  Busy lanes then advance their
// ray by up to `steps` traversal steps.  start(i) loads queue entry i into the
// lane; advance() runs one step and returns true once the ray has finished
// and its result is written.  round() runs with the warp converged at the top
// of every round (and so after the last one).  A warp leaves only when the
// queue is exhausted and none of its lanes is busy, so every entry below
// `count` is traced once.
//
// With a `kind` functor (true when the lane's next step is an interior visit,
// false when it is a triangle test), each step runs only the kind that the
// majority of the warp's busy lanes needs and the other lanes wait one step,
// instead of the warp running both branches with part of its lanes each;
// every ray still takes its own steps in its own order.
struct NoKind {};

// the majority-step functor of a traversal, or none.  Used by the binary
// shadow traversal (any hit): −11 % shadow time on the 2.1M-triangle bench
// scene; the closest-hit extend traversal lost 7 % with it and runs both
// branches per step
#ifndef PT_MAJORITY_EXTEND
#define PT_MAJORITY_EXTEND 0
#endif
#ifndef PT_MAJORITY_SHADOW
#define PT_MAJORITY_SHADOW 1
#endif
template <class T, class G>
struct StepKind {
    const T* t;
    G fast;  // the lane's current scene layouts: () -> const Fast&
    PTD bool operator()() const { return t->next_is_interior(); }
    // a lane that waits this step fetches its next step's data meanwhile (PT_PREFETCH)
    PTD void wait() const { t->prefetch_next(fast()); }
};
template <bool kUse, class T, class G>
PTD auto step_kind(const T& t, G fast) {
    if constexpr (kUse)
        return StepKind<T, G>{&t, fast};
    else
        return NoKind{};
}

template <class Start, class Advance, class Round = NoRound, class Kind = NoKind>
PTD void lane_refill_loop(uint32_t* fetch, uint32_t count, uint32_t steps, unsigned refill_below, Start&& start,
                          Advance&& advance, Round&& round = Round(), Kind&& kind = Kind()) {
    constexpr bool kMajority = !std::is_same<typename std::decay<Kind>::type, NoKind>::value;
    const unsigned lane = lane_id();
    if (refill_below < 1u) refill_below = 1u;
    bool active = false, exhausted = false;
    for (;;) {
        round();
        unsigned busy = __ballot_sync(0xffffffffu, active);
        if (!exhausted && (unsigned)__popc(busy) < refill_below) {
            const unsigned idle = ~busy;
            const unsigned leader = (unsigned)(__ffs(idle) - 1);
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(fetch, (uint32_t)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
                const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < count) {
                    start(i);
                    active = true;
                }
            }
            if (base + (uint32_t)__popc(idle) >= count) exhausted = true;
            busy = __ballot_sync(0xffffffffu, active);
        }
        if (busy == 0u) break;  // exhausted: a refill above found nothing left
        if constexpr (kMajority) {
            // every lane of the warp runs the same number of rounds of this loop
#pragma unroll 1
            for (uint32_t k = 0; k < steps; ++k) {
                bool interior = false;
                if (active) interior = kind();
                const unsigned alive = __ballot_sync(0xffffffffu, active);
                if (alive == 0u) break;
                const unsigned want = __ballot_sync(0xffffffffu, interior);
                const bool run_interior = 2 * __popc(want) >= __popc(alive);
                if (active) {
                    if (interior == run_interior) {
                        if (advance()) active = false;
                    } else {
                        kind.wait();
                    }
                }
            }
        } else {
            if (active) {
#pragma unroll 1
                for (uint32_t k = 0; k < steps; ++k) {
                    if (advance()) {
                        active = false;
                        break;
                    }
                }
            }
        }
    }
}


}  // namespace ptd
