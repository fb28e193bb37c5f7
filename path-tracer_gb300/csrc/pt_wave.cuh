// pt_wave.cuh - device building blocks shared by the wavefront kernels of one
// tile (trace_wavefront.cu) and of many jobs (batch.cu): the derived BVH and
// triangle layouts, the queue view, the per-lane traversal state machine and
// warp-aggregated queue appends.
#pragma once

#include "pt_path.cuh"

namespace ptd {

struct Fast {
    const float4* pairs;  // node i at pairs[2i], pairs[2i+1]
    const float4* tri4;   // triangle i at tri4[3i .. 3i+2]
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
    uint32_t* cnt;  // [0], [1] ray queue lengths, [2] shadow length, [3] extend fetch, [4] shadow fetch
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
#ifndef PT_EXTEND_MIN_BLOCKS
#define PT_EXTEND_MIN_BLOCKS 1
#endif
#ifndef PT_SHADE_THREADS
#define PT_SHADE_THREADS 128
#endif
#ifndef PT_SHADE_MIN_BLOCKS
#define PT_SHADE_MIN_BLOCKS 8
#endif
#ifndef PT_STEPS_PER_REFILL
#define PT_STEPS_PER_REFILL 32
#endif
// idle lanes of a traversal warp take new rays once fewer than this many are busy
#ifndef PT_REFILL_BELOW
#define PT_REFILL_BELOW 32
#endif
// 1: a traversal step tests one triangle of a leaf; 0: a whole leaf
#ifndef PT_TRI_PER_STEP
#define PT_TRI_PER_STEP 1
#endif
constexpr int kExtendThreads = PT_EXTEND_THREADS;
constexpr int kShadeThreads = PT_SHADE_THREADS;

PTD Tri load_tri4(const Fast& f, uint32_t tri) {
    const float4* p = f.tri4 + 3 * (size_t)tri;
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    Tri t;
    t.v0 = mk(a.x, a.y, a.z);
    t.v1 = mk(b.x, b.y, b.z);
    t.v2 = mk(c.x, c.y, c.z);
    return t;
}

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
template <bool kRec, bool kAlpha, bool kShadow, bool kTri36 = false>
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

    PTD bool pop(uint2* stack, uint32_t* istack) {
        if (sp == 0u) return true;
        sp -= 1u;
        const uint2 e = stack[sp & 63u];
        lf = e.x;
        tc = e.y;
        if constexpr (kRec) idx = istack[sp & 63u];
        return false;
    }

    // the watertight test of one triangle against the ray; for kShadow true
    // when the triangle occludes
    PTD bool test_triangle(const World& w, const Fast& f, uint32_t tri) {
        rec.tri();
        float t, v, wb;
        Tri tv;
        if constexpr (kTri36)
            tv = load_tri(w, tri);  // the caller's 36-byte triangles
        else
            tv = load_tri4(f, tri);
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

#if PT_TRI_PER_STEP
    // one interior node visit or one triangle test; true when the traversal
    // has finished (for kShadow, hit == 1 marks an occluder).  Testing a
    // leaf's triangles one per step keeps the two divergent paths of a warp
    // (box pair vs triangle) about equally long.
    PTD bool step(const World& w, const Fast& f, uint2* stack, uint32_t* istack) {
        if (tri_left == 0u) {
            rec.visit(idx);
            if (tc == 0u) {
                rec.interior();
                const float4* p = f.pairs + 2 * (size_t)lf;
                const float4 l0 = __ldg(p), l1 = __ldg(p + 1), r0 = __ldg(p + 2), r1 = __ldg(p + 3);
                const float dl = box_test(l0, l1, nod, rcp, hit_t);
                const float dr = box_test(r0, r1, nod, rcp, hit_t);
                const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
                if (hl || hr) {
                    const bool go_left = hl && (!hr || dl < dr);
                    if (hl && hr) {
                        const float4 f0 = go_left ? r0 : l0, f1 = go_left ? r1 : l1;
                        stack[sp & 63u] = make_uint2(__float_as_uint(f0.w), __float_as_uint(f1.w));
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
#else
    // one node visit; true when the traversal has finished (for kShadow,
    // hit == 1 marks an occluder)
    PTD bool step(const World& w, const Fast& f, uint2* stack, uint32_t* istack) {
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
            const float4 l0 = __ldg(p), l1 = __ldg(p + 1), r0 = __ldg(p + 2), r1 = __ldg(p + 3);
            const float dl = box_test(l0, l1, nod, rcp, hit_t);
            const float dr = box_test(r0, r1, nod, rcp, hit_t);
            const bool hl = dl >= 0.0f, hr = dr >= 0.0f;
            if (hl || hr) {
                const bool go_left = hl && (!hr || dl < dr);
                if (hl && hr) {
                    const float4 f0 = go_left ? r0 : l0, f1 = go_left ? r1 : l1;
                    stack[sp & 63u] = make_uint2(__float_as_uint(f0.w), __float_as_uint(f1.w));
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
#endif
};

constexpr int kStepsPerRefill = PT_STEPS_PER_REFILL;
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

// The persistent traversal loop of one warp; every lane holds at most one ray.
// Each round the warp counts its busy lanes: when fewer than refill_below are
// busy and the queue still has rays, the idle lanes take the next ones (one
// atomic per warp, queue slots in lane order).  Busy lanes then advance their
// ray by up to `steps` traversal steps.  start(i) loads queue entry i into the
// lane; advance() runs one step and returns true once the ray has finished
// and its result is written.  A warp leaves only when the queue is exhausted
// and none of its lanes is busy, so every entry below `count` is traced once.
template <class Start, class Advance>
PTD void lane_refill_loop(uint32_t* fetch, uint32_t count, uint32_t steps, unsigned refill_below, Start&& start,
                          Advance&& advance) {
    const unsigned lane = lane_id();
    if (refill_below < 1u) refill_below = 1u;
    bool active = false, exhausted = false;
    for (;;) {
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


}  // namespace ptd
