// batch.cu - the batched render engine of include/pt_batch.h.
//
// Device side: a ring of work items (job, tile, sample range); per wave a
// planner kernel packs queued items into the wave's path budget, then raygen
// -> (extend -> shade -> shadow) x 17 rounds -> accumulate run over every
// path of the wave, each path looking up its job and scene.  The whole wave
// is one captured CUDA graph.  Host side: the scene cache (content hash, HBM
// budget, LRU eviction), jobs and their resident accumulation buffers, the
// ring producer, wave launching and completion polling, and the autotuner.
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <system_error>
#include <thread>
#include <vector>

#include <type_traits>

#include "../../include/pt_batch.h"
#include "../../include/pt_precision.h"
#include "pt_abi_guard.h"
#include "pt_links.h"
#include "pt_wave.cuh"
#include "pt_wavefront.h"

namespace ptb {

using namespace ptd;

struct SceneDev {
    World w;  // camera unused: each job carries its own
    Fast f;
};

struct JobDev {
    uint32_t scene;
    uint32_t width, height, max_bounces;
    pt_camera camera;
    float4* accum;
    float4* image;
    float4* comp;  // Kahan compensation (precision form), else null
};

struct ItemDev {
    uint32_t slot;  // job slot
    uint32_t x0, y0, w, h;
    uint32_t first_sample;  // 1-based sample index n of the first sample
    uint32_t samples;
    uint32_t pad;
};

struct Ctrl {
    unsigned long long head, tail;  // ring positions (items)
    uint32_t wave_items, wave_paths;
    unsigned long long waves;
};

struct WaveBufs {
    Queues q;
    uint32_t* tag;        // per path: job slot << 8 | scene slot
    uint32_t* wave_item;  // ring index of each item of the wave
    uint32_t* wave_off;   // first path of each item (+ total at [n])
};

constexpr uint32_t kMaxScenes = 256;
constexpr uint32_t kMaxSlots = 1u << 16;
constexpr uint32_t kRounds = PT_MAX_BOUNCES_LIMIT + 1;
constexpr uint32_t kEngineSortShift = 10;  // sort bucket = triangle index / 1024

// ---------------------------------------------------------------- kernels

__global__ void plan_kernel(Ctrl* ctrl, const ItemDev* ring, uint64_t ring_cap, uint32_t budget, uint32_t max_items,
                            WaveBufs b) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long head = ctrl->head;
    const unsigned long long tail = ctrl->tail;
    uint32_t n = 0, paths = 0;
    while (head < tail && n < max_items) {
        const ItemDev it = ring[head % ring_cap];
        const uint32_t np = it.w * it.h * it.samples;
        if (n > 0 && paths + np > budget) break;
        b.wave_item[n] = (uint32_t)(head % ring_cap);
        b.wave_off[n] = paths;
        paths += np;
        ++n;
        ++head;
    }
    b.wave_off[n] = paths;
    ctrl->head = head;
    ctrl->wave_items = n;
    ctrl->wave_paths = paths;
    ctrl->waves += 1;
    b.q.cnt[0] = paths;
    b.q.cnt[1] = 0u;
}

// one block per item (grid-stride over the wave's items)
// path order within a work item: the wavefront kernels' order (PT_PIXEL_MAJOR)
PTD uint32_t item_path(uint32_t s, uint32_t pix, uint32_t px_count, uint32_t samples) {
#if PT_PIXEL_MAJOR
    return pix * samples + s;
#else
    return s * px_count + pix;
#endif
}

__global__ void __launch_bounds__(256) raygen_kernel(const Ctrl* ctrl, const ItemDev* ring, const JobDev* jobs,
                                                     WaveBufs b) {
    const uint32_t n_items = ctrl->wave_items;
    for (uint32_t k = blockIdx.x; k < n_items; k += gridDim.x) {
        const ItemDev it = ring[b.wave_item[k]];
        const JobDev& job = jobs[it.slot];
        const uint32_t off = b.wave_off[k];
        const uint32_t px_count = it.w * it.h;
        const uint32_t paths = px_count * it.samples;
        const uint32_t tag = (it.slot << 8) | job.scene;
        for (uint32_t i = threadIdx.x; i < paths; i += blockDim.x) {
#if PT_PIXEL_MAJOR
            const uint32_t pix = i / it.samples, s = i - pix * it.samples;  // a pixel's samples adjacent
#else
            const uint32_t s = i / px_count, pix = i - s * px_count;
#endif
            const uint32_t gy = pix / it.w, gx = pix - gy * it.w;
            const uint32_t px = it.x0 + gx, py = it.y0 + gy;
            const uint32_t p = off + i;
            Rng<false> rng;
            rng.s = seed(px, py, it.first_sample + s);
            PathState ps;
            camera_ray(job.camera, px, py, job.width, job.height, rng, ps);
            b.q.o[0][p] = make_float4(ps.o.x, ps.o.y, ps.o.z, __uint_as_float(p));
            b.q.d[0][p] = make_float4(ps.d.x, ps.d.y, ps.d.z, __uint_as_float(rng.s));
            b.q.T[0][p] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            b.q.color[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            b.tag[p] = tag;
        }
    }
}

__global__ void reset_kernel(uint32_t* cnt, int next) {
    cnt[next] = 0u;
    cnt[2] = 0u;
    cnt[3] = 0u;
    cnt[4] = 0u;
    cnt[5] = 0u;
    cnt[6] = 0u;
    cnt[7] = 0u;  // set again by the sort when it runs
}

// resident blocks per SM a kernel of kThreads threads is compiled for: the
// same registers per thread as kMinBlocks blocks of kBaseThreads threads
static_assert((kExtendThreads == 64 || kExtendThreads == 128 || kExtendThreads == 256) &&
                  (kShadeThreads == 128 || kShadeThreads == 256 || kShadeThreads == 512 || kShadeThreads == 1024),
              "the engine's default block shapes must be among its compiled ones");
constexpr int blocks_for(int kMinBlocks, int kBaseThreads, int kThreads) {
    return kMinBlocks * kBaseThreads / kThreads > 0 ? kMinBlocks * kBaseThreads / kThreads : 1;
}

template <bool kAlpha, bool kWide, int kThreads = kExtendThreads>
__global__ void __launch_bounds__(kThreads, blocks_for(kWide ? PT_WIDE_MIN_BLOCKS : PT_EXTEND_MIN_BLOCKS, kExtendThreads, kThreads))
    extend_kernel(const SceneDev* scenes, WaveBufs b, int cur, uint32_t steps_per_refill) {
    static_assert(!(kAlpha && kWide), "the wide form runs opaque scenes only");
    const Stage st = stage_of(b.q, cur);
    const uint32_t count = *st.count;
    typename std::conditional<kWide, WideTraverser<false>, Traverser<false, kAlpha, false>>::type tr;
    constexpr uint32_t kShared = kWide ? kWideSmemStack : kSmemStack;
    __shared__ uint2 stack_top[kShared > 0u ? kShared * kThreads : 1u];
    LaneStack<kThreads, kShared> stack;
    stack.col = stack_top + threadIdx.x;
    uint32_t istack[1];
    const SceneDev* sc = scenes;
    uint32_t slot = 0;
    __shared__ FilerSlots<kThreads> filer_slots;
    ResultFiler filer = filer_slots.of_warp(lane_id());
    lane_refill_loop(
        &b.q.cnt[3], count, kWide ? (uint32_t)kWideStepsPerRefill : steps_per_refill, kRefillBelow,
        [&](uint32_t i) {
            slot = i;
            const float4 o4 = st.o[i], d4 = st.d[i];
            sc = scenes + (b.tag[__float_as_uint(o4.w)] & 0xffu);
            tr.rng.s = __float_as_uint(d4.w);
            stack.reset();
            tr.init(sc->f, mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z), kFltMax, -1);
        },
        [&]() {
            if (!tr.step(sc->w, sc->f, stack, istack)) return false;
            b.q.hit[slot] = make_float4(tr.hit_t, __int_as_float(tr.hit), tr.hv, tr.hw);
            if constexpr (kAlpha) st.d[slot].w = __uint_as_float(tr.rng.s);
            filer.file(slot, tr.hit != -1);
            return true;
        },
        [&]() { filer.flush(b.q, lane_id()); });
}

template <bool kAlpha, int kThreads = kShadeThreads>
__global__ void __launch_bounds__(kThreads, blocks_for(PT_SHADE_MIN_BLOCKS, kShadeThreads, kThreads))
    shade_kernel(const SceneDev* scenes, const JobDev* jobs, WaveBufs b, int cur, uint32_t bounce) {
    const Stage st = stage_of(b.q, cur);
    const ShadeRange range(b.q);
    const uint32_t count = range.count();
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const unsigned lane = lane_id();
    for (uint32_t base = warp * 32u; base < count; base += warps * 32u) {
        const uint32_t i = range.slot(b.q, base + lane);
        bool cont = false;
        ShadowRay sr;
        sr.valid = false;
        PathState ps;
        uint32_t p = 0, rs = 0;
        if (i != 0xffffffffu) {
            // the entries before miss_span are misses (the extend kernel filed them so): no hit record to read
            const bool miss = base + lane < range.miss_span;
            const float4 o4 = st.o[i], d4 = st.d[i], t4 = st.T[i];
            const float4 h4 = miss ? make_float4(0.0f, __int_as_float(-1), 0.0f, 0.0f) : b.q.hit[i];
            p = __float_as_uint(o4.w);
            const uint32_t tag = b.tag[p];
            const World& w = scenes[tag & 0xffu].w;
            const uint32_t max_bounces = jobs[tag >> 8].max_bounces;
            ps.o = mk(o4.x, o4.y, o4.z);
            ps.d = mk(d4.x, d4.y, d4.z);
            ps.throughput = mk(t4.x, t4.y, t4.z);
            ps.prev_pdf = t4.w;
            if constexpr (kColorDelta<kAlpha>) {
                ps.color = mk(0.0f, 0.0f, 0.0f);
            } else {
                const float4 c4 = b.q.color[p];
                ps.color = mk(c4.x, c4.y, c4.z);
            }
            Rng<false> rng;
            rng.s = __float_as_uint(d4.w);
            const int32_t hit = __float_as_int(h4.y);
            if (bounce <= max_bounces) {
                if (hit == -1) {
                    shade_miss(w, bounce, ps);
                } else {
                    cont = shade_hit<false, kAlpha>(w, bounce, max_bounces, ps, h4.x, (uint32_t)hit, h4.z, h4.w, rng,
                                                    nullptr, &sr);
                }
            }
            store_color<kAlpha>(b.q.color, p, ps.color);
            rs = rng.s;
        }
        const uint32_t slot = warp_append(cont, st.next_count, 0xffffffffu);
        if (cont) {
            st.no[slot] = make_float4(ps.o.x, ps.o.y, ps.o.z, __uint_as_float(p));
            st.nd[slot] = make_float4(ps.d.x, ps.d.y, ps.d.z, __uint_as_float(rs));
            st.nT[slot] = make_float4(ps.throughput.x, ps.throughput.y, ps.throughput.z, ps.prev_pdf);
        }
        if constexpr (!kAlpha) {
            const uint32_t sslot = warp_append(sr.valid, &b.q.cnt[2], 0xffffffffu);
            if (sr.valid) {
                b.q.so[sslot] = make_float4(sr.o.x, sr.o.y, sr.o.z, __uint_as_float(p));
                b.q.sd[sslot] = make_float4(sr.d.x, sr.d.y, sr.d.z, sr.dist);
                b.q.sc[sslot] = make_float4(sr.contribution.x, sr.contribution.y, sr.contribution.z, __int_as_float(sr.light_tri));
            }
        }
    }
}

template <bool kWide, int kThreads = kExtendThreads>
__global__ void __launch_bounds__(kThreads, blocks_for(kWide ? PT_WIDE_MIN_BLOCKS : PT_EXTEND_MIN_BLOCKS, kExtendThreads, kThreads))
    shadow_kernel(const SceneDev* scenes, WaveBufs b, uint32_t steps_per_refill) {
    const uint32_t count = b.q.cnt[2];
    typename std::conditional<kWide, WideTraverser<true>, Traverser<false, false, true, false, PT_SHADOW_TRI_PER_STEP != 0>>::type tr;
    constexpr uint32_t kShared = kWide ? kWideSmemStack : kSmemStack;
    __shared__ uint2 stack_top[kShared > 0u ? kShared * kThreads : 1u];
    LaneStack<kThreads, kShared> stack;
    stack.col = stack_top + threadIdx.x;
    uint32_t istack[1];
    const SceneDev* sc = scenes;
    uint32_t path = 0;
    float4 contribution = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    lane_refill_loop(
        &b.q.cnt[4], count, kWide ? (uint32_t)kWideStepsPerRefill : steps_per_refill, kRefillBelow,
        [&](uint32_t i) {
            const float4 o4 = b.q.so[i], d4 = b.q.sd[i];
            contribution = b.q.sc[i];
            path = __float_as_uint(o4.w);
            sc = scenes + (b.tag[path] & 0xffu);
            stack.reset();
            tr.init(sc->f, mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z), d4.w, __float_as_int(contribution.w));
        },
        [&]() {
            if (!tr.step(sc->w, sc->f, stack, istack)) return false;
            if (tr.hit != 1) {
                const float4 col = b.q.color[path];
                const f3 sum = mk(col.x, col.y, col.z) + mk(contribution.x, contribution.y, contribution.z);
                b.q.color[path] = make_float4(sum.x, sum.y, sum.z, 0.0f);
            }
            return true;
        },
        NoRound(), step_kind<PT_MAJORITY_SHADOW && !kWide>(tr, [&]() -> const Fast& { return sc->f; }));
}

// accumulate, trace.slang:1299-1308: one block per item, samples in order;
// then count the item as finished for its job slot
__global__ void __launch_bounds__(256) accumulate_kernel(const Ctrl* ctrl, const ItemDev* ring, const JobDev* jobs,
                                                         WaveBufs b, uint32_t* items_done) {
    const uint32_t n_items = ctrl->wave_items;
    for (uint32_t k = blockIdx.x; k < n_items; k += gridDim.x) {
        const ItemDev it = ring[b.wave_item[k]];
        const JobDev& job = jobs[it.slot];
        const uint32_t off = b.wave_off[k];
        const uint32_t px_count = it.w * it.h;
        for (uint32_t pix = threadIdx.x; pix < px_count; pix += blockDim.x) {
            const uint32_t gy = pix / it.w, gx = pix - gy * it.w;
            const size_t idx = (size_t)(it.y0 + gy) * job.width + (it.x0 + gx);
            f3 acc = mk(0.0f, 0.0f, 0.0f);
            if (it.first_sample > 1u) {
                const float4 a = job.accum[idx];
                acc = mk(a.x, a.y, a.z);
            }
            uint32_t n = it.first_sample;
            if (job.comp) {
                // Kahan-compensated sums; the first sample is 0 + L with zero compensation
                f3 comp = mk(0.0f, 0.0f, 0.0f);
                if (it.first_sample > 1u) {
                    const float4 k = job.comp[idx];
                    comp = mk(k.x, k.y, k.z);
                }
                for (uint32_t s = 0; s < it.samples; ++s, ++n) {
                    const float4 c = b.q.color[off + item_path(s, pix, px_count, it.samples)];
                    const f3 y = mk(c.x, c.y, c.z) - comp;
                    const f3 sum = acc + y;
                    comp = (sum - acc) - y;
                    acc = sum;
                }
                job.comp[idx] = make_float4(comp.x, comp.y, comp.z, 0.0f);
            } else {
                for (uint32_t s = 0; s < it.samples; ++s, ++n) {
                    const float4 c = b.q.color[off + item_path(s, pix, px_count, it.samples)];
                    acc = (n > 1u ? acc : mk(0.0f, 0.0f, 0.0f)) + mk(c.x, c.y, c.z);
                }
            }
            n -= 1u;
            job.accum[idx] = make_float4(acc.x, acc.y, acc.z, 1.0f);
            const f3 out = kExposure * acc / (float)n;
            job.image[idx] = make_float4(out.x, out.y, out.z, 1.0f);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&items_done[it.slot], 1u);
        }
        __syncthreads();
    }
}

__global__ void pad_triangles_kernel(const pt_triangle_geometry* geo, uint64_t n, float4* tri4) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = geo[i].v0;
    tri4[kTriStride * i + 0] = make_float4(v[0], v[1], v[2], 0.0f);
    tri4[kTriStride * i + 1] = make_float4(v[3], v[4], v[5], 0.0f);
    tri4[kTriStride * i + 2] = make_float4(v[6], v[7], v[8], 0.0f);
    if (kTriStride == 4) tri4[kTriStride * i + 3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // read, never used
}

// ---------------------------------------------------------------- host

struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t alloc(size_t n) {
        release();
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e == cudaSuccess) bytes = n ? n : 16;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    ~Buf() { release(); }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// A device buffer allocated and freed in stream order from the engine's
// memory pool: neither call synchronises the device, so per-job buffers come
// and go while waves run (cudaFree would wait for the whole GPU).
struct StreamBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    cudaError_t alloc(size_t n, cudaMemPool_t pool, cudaStream_t s) {
        release();
        stream = s;
        cudaError_t e = cudaMallocFromPoolAsync(&p, n ? n : 16, pool, s);
        if (e == cudaSuccess) bytes = n ? n : 16;
        return e;
    }
    void release() {
        if (p) cudaFreeAsync(p, stream);
        p = nullptr;
        bytes = 0;
    }
    ~StreamBuf() { release(); }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct Scene {
    uint64_t id = 0;
    uint64_t check = 0;  // second content hash (see hash_buffers)
    uint32_t slot = 0;
    uint64_t bytes = 0;
    bool any_alpha = false;
    int caller_refs = 0;  // pte_scene_add minus pte_scene_release
    int job_refs = 0;     // accumulations using it
    uint64_t last_use = 0;
    Buf geo, attr, mat, nodes, srgb, linear, sky, sky_alias, scene_alias, lut, pairs, tri4;
    Buf wide, links, attr_h, sky_h;  // precision form (links: parent per node, leaf per triangle)
};

struct Accumulation {
    uint32_t slot = 0;
    uint64_t scene = 0;
    uint32_t width = 0, height = 0, max_bounces = 0;
    uint32_t samples_done = 0;
    bool busy = false;
    uint64_t bytes = 0;
    int job_refs = 0;
    StreamBuf accum, image, comp;
    std::deque<uint64_t> waiting;  // jobs queued behind the running pass
};

struct Job {
    uint64_t id = 0;
    std::shared_ptr<Accumulation> acc;
    pt_camera camera{};
    uint32_t samples = 0;
    int status = PT_JOB_QUEUED;
    uint64_t items_target = 0;  // cumulative item count of the slot at which this job is done
    std::deque<ItemDev> pending;  // work items not yet handed to a wave
    uint64_t pending_paths = 0;
    uint32_t rounds = 0;  // bounce rounds its paths can take (max_bounces + 1)
    bool alpha = false;   // its scene has non-opaque materials
    std::chrono::steady_clock::time_point submitted;
};

struct Flight {
    cudaEvent_t start, stop;
};

int hbm_fail(std::string& err, const char* what, uint64_t need, uint64_t used, uint64_t budget) {
    char msg[256];
    snprintf(msg, sizeof msg, "%s needs %llu bytes but only %llu of the %llu-byte HBM budget are free", what,
             (unsigned long long)need, (unsigned long long)(budget > used ? budget - used : 0),
             (unsigned long long)budget);
    err = msg;
    return PT_ERR_OOM;
}

// Content identity of a scene: two independent 64-bit hashes over every
// uploaded byte.  The first names the scene in the cache; a cache hit also
// needs the second to match, so two different uploads share a cache entry
// only if both hashes collide at once.
struct Digest {
    uint64_t a = 0x5EED5EEDull, b = 0x243F6A8885A308D3ull;
};

inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

// both hashes of one byte range: a multiply-xorshift chain and an
// add-multiply-rotate chain with different constants
Digest hash_range(const unsigned char* p, size_t n) {
    Digest d;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        memcpy(&w, p + i, 8);
        d.a ^= w;
        d.a *= 0x9E3779B97F4A7C15ull;
        d.a ^= d.a >> 29;
        d.b = rotl64(d.b + w * 0xC2B2AE3D27D4EB4Full, 31) * 0x165667B19E3779F9ull;
    }
    for (; i < n; ++i) {
        d.a ^= p[i];
        d.a *= 0x100000001B3ull;
        d.b = rotl64(d.b + p[i] * 0x27D4EB2F165667C5ull, 23) * 0x9E3779B185EBCA87ull;
    }
    d.a ^= (uint64_t)n;
    d.b ^= rotl64((uint64_t)n, 17);
    return d;
}

// Digest of a sequence of buffers: each is cut into 8 MiB chunks hashed in
// parallel on up to 16 host threads, and the chunk digests are folded in
// order together with each buffer's length, so the result depends on every
// byte, the order of the buffers and their boundaries.
Digest hash_buffers(const std::vector<std::pair<const void*, size_t>>& bufs) {
    constexpr size_t kChunk = 8u << 20;
    struct Piece {
        const unsigned char* p;
        size_t n;
        size_t buffer;
    };
    std::vector<Piece> pieces;
    for (size_t k = 0; k < bufs.size(); ++k) {
        const unsigned char* p = static_cast<const unsigned char*>(bufs[k].first);
        const size_t n = bufs[k].second;
        if (n == 0) pieces.push_back({p, 0, k});
        for (size_t o = 0; o < n; o += kChunk) pieces.push_back({p + o, n - o < kChunk ? n - o : kChunk, k});
    }
    std::vector<Digest> parts(pieces.size());
    std::atomic<size_t> next{0};
    const auto worker = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < pieces.size();) parts[i] = hash_range(pieces[i].p, pieces[i].n);
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t threads = std::min<size_t>(pieces.size(), std::max(1u, std::min(hw, 16u)));
    std::vector<std::thread> pool;
    for (size_t t = 1; t < threads; ++t) {
        try {
            pool.emplace_back(worker);
        } catch (const std::system_error&) {
            break;  // the calling thread takes the remaining chunks
        }
    }
    worker();
    for (auto& th : pool) th.join();
    Digest d;
    for (size_t i = 0; i < pieces.size(); ++i) {
        d.a = (d.a ^ parts[i].a ^ (pieces[i].buffer << 48)) * 0x9E3779B97F4A7C15ull;
        d.a ^= d.a >> 31;
        d.b = rotl64(d.b + parts[i].b + pieces[i].buffer, 27) * 0xC2B2AE3D27D4EB4Full;
    }
    for (const auto& b : bufs) {
        d.a = (d.a ^ (uint64_t)b.second) * 0xFF51AFD7ED558CCDull;
        d.b = rotl64(d.b ^ (uint64_t)b.second, 13) * 0xC4CEB9FE1A85EC53ull;
    }
    return d;
}

}  // namespace ptb

using namespace ptb;

struct pt_engine {
    pt_engine_config cfg{};
    std::string error;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;  // per-job buffers, kept cached (release threshold: never)
    int sms = 0;
    uint64_t budget = 0, used = 0;
    // scenes
    std::map<uint64_t, std::unique_ptr<Scene>> scenes;
    std::vector<uint64_t> scene_slots;  // slot -> scene id (0 = free)
    Buf d_scenes;
    uint64_t use_clock = 0;
    // accumulations / jobs
    std::vector<std::shared_ptr<Accumulation>> slots;  // job slot -> accumulation
    std::vector<uint64_t> slot_items;                  // items ever queued per slot
    Buf d_jobs, d_done;
    uint32_t* h_done = nullptr;  // pinned mirror of the per-slot finished-item counters
    Ctrl* h_ctrl = nullptr;      // pinned mirror of the ring control block
    std::map<uint64_t, Job> jobs;
    uint64_t next_job = 1;
    std::deque<uint64_t> done_unreported;
    // ring and wave
    Buf d_ring, d_ctrl;
    uint64_t ring_cap = 1ull << 20;
    uint64_t tail = 0;  // host copy of the producer position
    uint64_t head_seen = 0;
    Buf wave[13];
    Buf d_tag, d_wave_item, d_wave_off;
    uint32_t* sort_counts = nullptr;  // kSortBuckets counts, then kSortBuckets offsets (inside wave[12])
    ptb::WaveBufs wb{};
    uint32_t max_items = 0;
    bool wave_ready = false;
    // one captured wave per kind (opaque / non-opaque) and number of bounce rounds
    cudaGraphExec_t graph[2][kRounds] = {};
    std::deque<Flight> flights;
    std::vector<cudaEvent_t> event_pool;
    pt_engine_stats stats{};
    // a background thread keeps waves queued on the stream (harvest + pump)
    // whatever the caller's thread is doing; every entry point takes `mu`
    mutable std::recursive_mutex mu;
    std::thread pumper;
    std::atomic<bool> stop{false};
    int sticky = PT_OK;  // first error of the background thread, returned by later calls

    int fail(int code, const std::string& m) {
        error = m;
        return code;
    }
    int cuda(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return PT_OK;
        error = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? PT_ERR_OOM : PT_ERR_CUDA;
    }
    cudaEvent_t event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
};

namespace {

uint64_t wave_bytes(uint32_t paths) {
    return (uint64_t)paths * (11 * 16 + 4 + 12) + 2ull * (paths / 64 + 2) * 4 + 2 * kSortBuckets * 4 + 4096;
}

void drop_graphs(pt_engine* e) {
    for (auto& kind : e->graph)
        for (auto& g : kind)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
}

int setup_wave(pt_engine* e) {
    drop_graphs(e);
    for (Buf& b : e->wave) b.release();
    e->d_tag.release();
    e->d_wave_item.release();
    e->d_wave_off.release();
    if (e->wave_ready) e->used -= wave_bytes(e->cfg.wave_paths);
    e->wave_ready = false;
    const uint32_t W = e->cfg.wave_paths;
    const uint64_t need = wave_bytes(W);
    if (e->used + need > e->budget) return hbm_fail(e->error, "the wave buffers", need, e->used, e->budget);
    e->max_items = W / 64 + 1;
    int rc = PT_OK;
    for (int k = 0; k < 11 && !rc; ++k) rc = e->cuda(e->wave[k].alloc((size_t)W * 16), "wave buffers");
    if (!rc) rc = e->cuda(e->wave[11].alloc(64), "wave counters");
    if (!rc) rc = e->cuda(e->wave[12].alloc((size_t)W * 12 + 2 * kSortBuckets * 4), "wave hit lists");
    if (!rc) rc = e->cuda(cudaMemset(e->wave[12].as<uint32_t>() + 3 * (size_t)W, 0, kSortBuckets * 4), "sort counts");
    if (!rc) rc = e->cuda(e->d_tag.alloc((size_t)W * 4), "wave buffers");
    if (!rc) rc = e->cuda(e->d_wave_item.alloc((size_t)(e->max_items + 1) * 4), "wave buffers");
    if (!rc) rc = e->cuda(e->d_wave_off.alloc((size_t)(e->max_items + 1) * 4), "wave buffers");
    if (rc) return rc;
    Queues& q = e->wb.q;
    q.o[0] = e->wave[0].as<float4>();
    q.o[1] = e->wave[1].as<float4>();
    q.d[0] = e->wave[2].as<float4>();
    q.d[1] = e->wave[3].as<float4>();
    q.T[0] = e->wave[4].as<float4>();
    q.T[1] = e->wave[5].as<float4>();
    q.hit = e->wave[6].as<float4>();
    q.color = e->wave[7].as<float4>();
    q.so = e->wave[8].as<float4>();
    q.sd = e->wave[9].as<float4>();
    q.sc = e->wave[10].as<float4>();
    q.cnt = e->wave[11].as<uint32_t>();
    q.hit_list = e->wave[12].as<uint32_t>();
    q.miss_list = q.hit_list + W;
    q.hit_sorted = q.miss_list + W;
    e->sort_counts = q.hit_sorted + W;
    q.rec = nullptr;
    q.rec_hits = nullptr;
    e->wb.tag = e->d_tag.as<uint32_t>();
    e->wb.wave_item = e->d_wave_item.as<uint32_t>();
    e->wb.wave_off = e->d_wave_off.as<uint32_t>();
    e->used += need;
    e->wave_ready = true;
    return PT_OK;
}

template <class K>
int occupancy(K kernel, int threads) {
    int blocks = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, 0);
    return blocks > 0 ? blocks : 1;
}

// one launch of a persistent stage kernel: the blocks that stay resident on every SM
template <class... P, class... A>
void launch_persistent(void (*kernel)(P...), pt_engine* e, int threads, A&&... args) {
    kernel<<<e->sms * occupancy(kernel, threads), threads, 0, e->stream>>>(std::forward<A>(args)...);
}

// the launches of one wave (captured into a graph, or issued directly)
template <bool kAlpha, bool kWideBvh>
cudaError_t issue_wave(pt_engine* e, uint32_t rounds) {
    const cudaStream_t s = e->stream;
    const ItemDev* ring = e->d_ring.as<const ItemDev>();
    Ctrl* ctrl = e->d_ctrl.as<Ctrl>();
    const SceneDev* scenes = e->d_scenes.as<const SceneDev>();
    const JobDev* jobs = e->d_jobs.as<const JobDev>();
    const int per_wave_blocks = e->sms * 8;
    plan_kernel<<<1, 32, 0, s>>>(ctrl, ring, e->ring_cap, e->cfg.wave_paths, e->max_items, e->wb);
    raygen_kernel<<<per_wave_blocks, 256, 0, s>>>(ctrl, ring, jobs, e->wb);
    constexpr bool kWide = kWideBvh && !kAlpha;
    const uint32_t tt = e->cfg.traversal_threads, st = e->cfg.shade_threads;
    // persistent launches: as many blocks as stay resident, for the block shape of the configuration
    const auto extend = [&](int cur) {
        if (tt == 64u) return launch_persistent(extend_kernel<kAlpha, kWide, 64>, e, 64, scenes, e->wb, cur, e->cfg.steps_per_refill);
        if (tt == 256u) return launch_persistent(extend_kernel<kAlpha, kWide, 256>, e, 256, scenes, e->wb, cur, e->cfg.steps_per_refill);
        return launch_persistent(extend_kernel<kAlpha, kWide, 128>, e, 128, scenes, e->wb, cur, e->cfg.steps_per_refill);
    };
    const auto shade = [&](int cur, uint32_t bounce) {
        if (st == 128u) return launch_persistent(shade_kernel<kAlpha, 128>, e, 128, scenes, jobs, e->wb, cur, bounce);
        if (st == 256u) return launch_persistent(shade_kernel<kAlpha, 256>, e, 256, scenes, jobs, e->wb, cur, bounce);
        if (st == 512u) return launch_persistent(shade_kernel<kAlpha, 512>, e, 512, scenes, jobs, e->wb, cur, bounce);
        return launch_persistent(shade_kernel<kAlpha, 1024>, e, 1024, scenes, jobs, e->wb, cur, bounce);
    };
    const auto shadow = [&]() {
        if (tt == 64u) return launch_persistent(shadow_kernel<kWide, 64>, e, 64, scenes, e->wb, e->cfg.steps_per_refill);
        if (tt == 256u) return launch_persistent(shadow_kernel<kWide, 256>, e, 256, scenes, e->wb, e->cfg.steps_per_refill);
        return launch_persistent(shadow_kernel<kWide, 128>, e, 128, scenes, e->wb, e->cfg.steps_per_refill);
    };
    int cur = 0;
    for (uint32_t bounce = 0; bounce < rounds; ++bounce) {
        reset_kernel<<<1, 1, 0, s>>>(e->wb.q.cnt, cur ^ 1);
        extend(cur);
        if (e->cfg.sort_min_hits != 0xffffffffu) {
            // hits of all jobs by triangle bucket (1024 triangles per bucket)
            sort_count_kernel<1><<<e->sms * 4, kSortThreads, 0, s>>>(World{}, e->wb.q, e->sort_counts,
                                                                   e->cfg.sort_min_hits, kEngineSortShift);
            sort_scan_kernel<0><<<1, 1024, 0, s>>>(e->wb.q, e->sort_counts, e->sort_counts + kSortBuckets,
                                                   e->cfg.sort_min_hits);
            sort_scatter_kernel<1><<<e->sms * 4, kSortThreads, 0, s>>>(World{}, e->wb.q, e->sort_counts + kSortBuckets,
                                                                     e->cfg.sort_min_hits, kEngineSortShift);
        }
        shade(cur, bounce);
        if constexpr (!kAlpha) shadow();
        cur ^= 1;
    }
    accumulate_kernel<<<per_wave_blocks, 256, 0, s>>>(ctrl, ring, jobs, e->wb, e->d_done.as<uint32_t>());
    cudaMemcpyAsync(e->h_ctrl, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(e->h_done, e->d_done.p, kMaxSlots * 4, cudaMemcpyDeviceToHost, s);
    return cudaGetLastError();
}

cudaError_t issue_any_wave(pt_engine* e, bool alpha, uint32_t rounds) {
    const bool wide = (e->cfg.precision & PT_PRECISION_WIDE_BVH) != 0;
    if (alpha) return issue_wave<true, false>(e, rounds);
    return wide ? issue_wave<false, true>(e, rounds) : issue_wave<false, false>(e, rounds);
}

// one wave of `rounds` bounce rounds (the deepest job of the wave needs
// max_bounces + 1; a path never takes more, so shallower waves skip the
// launches of rounds that would find empty queues)
int launch_wave(pt_engine* e, bool alpha, uint32_t rounds) {
    const int gi = alpha ? 1 : 0;
    if (rounds < 1 || rounds > kRounds) rounds = kRounds;
    cudaGraphExec_t& exec = e->graph[gi][rounds - 1];
    if (e->cfg.use_graphs && !exec) {
        cudaGraph_t g = nullptr;
        int rc = e->cuda(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        if (rc) return rc;
        const cudaError_t le = issue_any_wave(e, alpha, rounds);
        const cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
        if ((rc = e->cuda(le, "wave capture"))) return rc;
        if ((rc = e->cuda(ce, "graph capture"))) return rc;
        rc = e->cuda(cudaGraphInstantiate(&exec, g, 0), "graph instantiate");
        cudaGraphDestroy(g);
        if (rc) return rc;
    }
    Flight f{e->event(), e->event()};
    cudaEventRecord(f.start, e->stream);
    int rc;
    if (e->cfg.use_graphs)
        rc = e->cuda(cudaGraphLaunch(exec, e->stream), "graph launch");
    else
        rc = e->cuda(issue_any_wave(e, alpha, rounds), "wave launch");
    if (rc) return rc;
    cudaEventRecord(f.stop, e->stream);
    e->flights.push_back(f);
    return PT_OK;
}

// queue the work items of a job whose accumulation is free
int start_job(pt_engine* e, Job& j) {
    Accumulation& a = *j.acc;
    a.busy = true;
    j.status = PT_JOB_RUNNING;
    // device job record (camera of this pass)
    auto& sc = e->scenes.at(a.scene);
    JobDev jd;
    jd.scene = sc->slot;
    jd.width = a.width;
    jd.height = a.height;
    jd.max_bounces = a.max_bounces;
    jd.camera = j.camera;
    jd.accum = a.accum.as<float4>();
    jd.image = a.image.as<float4>();
    jd.comp = a.comp.p ? a.comp.as<float4>() : nullptr;
    int rc = e->cuda(cudaMemcpyAsync(e->d_jobs.as<JobDev>() + a.slot, &jd, sizeof jd, cudaMemcpyHostToDevice, e->stream),
                     "job record");
    if (rc) return rc;
    // the job's work items wait on the host until feed_wave hands them to a wave
    const uint32_t T = e->cfg.tile_size;
    size_t count = 0;
    for (uint32_t y = 0; y < a.height; y += T)
        for (uint32_t x = 0; x < a.width; x += T) {
            ItemDev it;
            it.slot = a.slot;
            it.x0 = x;
            it.y0 = y;
            it.w = std::min(T, a.width - x);
            it.h = std::min(T, a.height - y);
            it.first_sample = a.samples_done + 1u;
            it.samples = j.samples;
            it.pad = 0;
            j.pending.push_back(it);
            j.pending_paths += (uint64_t)it.w * it.h * it.samples;
            ++count;
        }
    j.rounds = a.max_bounces + 1u;
    j.alpha = sc->any_alpha;
    e->slot_items[a.slot] += count;
    j.items_target = e->slot_items[a.slot];
    e->stats.items += count;
    return PT_OK;
}

// Scheduling weight of a job's pending work: its remaining paths, shrunk as
// it waits (halved after kAgeMs), so short jobs go first (shortest remaining
// work first) and a long job's wait stays bounded.
constexpr double kAgeMs = 50.0;
double feed_key(const Job& j, std::chrono::steady_clock::time_point now) {
    const double age_ms = std::chrono::duration<double, std::milli>(now - j.submitted).count();
    return (double)j.pending_paths / (1.0 + age_ms / kAgeMs);
}

// Hands the next wave its work items: jobs in feed_key order, each giving
// its pending items in tile order while they fit the wave's path budget and
// item limit.  Writes them to the ring and the ring's tail, so the wave's
// planner (which takes every item up to the budget) consumes exactly these.
// Returns the number of items fed; *alpha and *rounds describe the wave.
int feed_wave(pt_engine* e, size_t* fed, bool* alpha, uint32_t* rounds) {
    *fed = 0;
    *alpha = false;
    *rounds = 1;
    const auto now = std::chrono::steady_clock::now();
    std::vector<std::pair<double, Job*>> order;
    for (auto& [id, j] : e->jobs)
        if (!j.pending.empty()) order.emplace_back(feed_key(j, now), &j);
    if (order.empty()) return PT_OK;
    std::stable_sort(order.begin(), order.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<ItemDev> wave;
    uint64_t paths = 0;
    const uint64_t budget = e->cfg.wave_paths;
    for (auto& [key, j] : order) {
        while (!j->pending.empty() && wave.size() < e->max_items) {
            const ItemDev& it = j->pending.front();
            const uint64_t np = (uint64_t)it.w * it.h * it.samples;
            if (!wave.empty() && paths + np > budget) break;
            wave.push_back(it);
            paths += np;
            j->pending_paths -= np;
            j->pending.pop_front();
            *alpha |= j->alpha;
            *rounds = std::max(*rounds, j->rounds);
        }
        if (paths >= budget || wave.size() >= e->max_items) break;
    }
    if (e->tail + wave.size() - e->head_seen > e->ring_cap) return e->fail(PT_ERR_OUT_OF_LIMITS, "work ring full");
    // copy into the ring (two pieces across the wrap); the copies read
    // pageable host memory, so they have taken it before they return
    size_t done = 0;
    while (done < wave.size()) {
        const uint64_t pos = (e->tail + done) % e->ring_cap;
        const size_t n = std::min<size_t>(wave.size() - done, e->ring_cap - pos);
        int rc = e->cuda(cudaMemcpyAsync(e->d_ring.as<ItemDev>() + pos, wave.data() + done, n * sizeof(ItemDev),
                                         cudaMemcpyHostToDevice, e->stream), "ring write");
        if (rc) return rc;
        done += n;
    }
    e->tail += wave.size();
    const unsigned long long t = e->tail;
    int rc = e->cuda(cudaMemcpyAsync(&e->d_ctrl.as<Ctrl>()->tail, &t, sizeof t, cudaMemcpyHostToDevice, e->stream),
                     "ring tail");
    if (rc) return rc;
    *fed = wave.size();
    return PT_OK;
}

void free_accumulation(pt_engine* e, Accumulation& a) {
    e->used -= a.bytes;
    a.accum.release();
    a.image.release();
    a.comp.release();
    e->slots[a.slot].reset();
    auto it = e->scenes.find(a.scene);
    if (it != e->scenes.end()) it->second->job_refs -= 1;
}

// harvest finished waves: job completion from the per-slot item counters
int harvest(pt_engine* e, bool block) {
    while (!e->flights.empty()) {
        Flight& f = e->flights.front();
        cudaError_t q = block ? cudaEventSynchronize(f.stop) : cudaEventQuery(f.stop);
        if (q == cudaErrorNotReady) return PT_OK;
        int rc = e->cuda(q, "wave");
        if (rc) return rc;
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, f.start, f.stop) == cudaSuccess) e->stats.gpu_ms += ms;
        e->event_pool.push_back(f.start);
        e->event_pool.push_back(f.stop);
        e->flights.pop_front();
        e->stats.waves += 1;
        e->stats.paths += e->h_ctrl->wave_paths;
        e->head_seen = e->h_ctrl->head;
        block = false;
        for (auto& [id, j] : e->jobs) {
            if (j.status != PT_JOB_RUNNING) continue;
            if (e->h_done[j.acc->slot] >= j.items_target) {
                j.status = PT_JOB_DONE;
                j.acc->samples_done += j.samples;
                j.acc->busy = false;
                e->stats.jobs_done += 1;
                e->done_unreported.push_back(id);
            }
        }
        // passes waiting on now-free accumulations
        for (auto& [id, j] : e->jobs) {
            if (j.status != PT_JOB_DONE) continue;
            Accumulation& a = *j.acc;
            while (!a.busy && !a.waiting.empty()) {
                const uint64_t next = a.waiting.front();
                a.waiting.pop_front();
                auto it = e->jobs.find(next);
                if (it == e->jobs.end()) continue;
                if ((rc = start_job(e, it->second))) return rc;
            }
        }
    }
    return PT_OK;
}

// waves queued on the stream at once: each wave's items are chosen when it
// is queued, so a newly submitted job waits at most for the waves already
// queued; one keeps that wait to the wave on the GPU, and the background
// thread queues the next wave within ~0.1 ms of its end
#ifndef PT_ENGINE_FLIGHTS
#define PT_ENGINE_FLIGHTS 1
#endif
int pump(pt_engine* e) {
    while (e->flights.size() < PT_ENGINE_FLIGHTS) {
        size_t fed = 0;
        bool alpha = false;
        uint32_t rounds = 1;
        int rc = feed_wave(e, &fed, &alpha, &rounds);
        if (rc) return rc;
        if (fed == 0) break;
        if ((rc = launch_wave(e, alpha, rounds))) return rc;
    }
    return PT_OK;
}

// which derived copies a cached scene keeps: the binary BVH always (waves
// with non-opaque jobs traverse it), the wide BVH for opaque scenes of a wide
// engine, and FP16 attributes / BF16 skybox in place of the FP32 ones
struct SceneForm {
    bool wide, half;
};
SceneForm scene_form(const pt_engine* e, bool any_alpha);

int upload_scene(pt_engine* e, Scene& s, const pt_world_updates* u) {
    const pt_scene_upload* sc = u->scene;
    const pt_skybox_upload* sk = u->skybox;
    const size_t layer = (size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
    const SceneForm form = scene_form(e, s.any_alpha);
    const uint64_t texels = (uint64_t)sk->uniforms.width * sk->uniforms.height;
    auto put = [&](Buf& b, const void* src, size_t n, const char* what) {
        int rc = e->cuda(b.alloc(n), what);
        if (!rc && n) rc = e->cuda(cudaMemcpyAsync(b.p, src, n, cudaMemcpyHostToDevice, e->stream), what);
        return rc;
    };
    int rc = put(s.geo, sc->geometries, sc->triangle_count * 36, "geometries");
    if (!rc) rc = put(s.attr, sc->attributes, sc->triangle_count * 112, "attributes");
    if (!rc) rc = put(s.mat, sc->materials, sc->material_count * 224, "materials");
    if (!rc) rc = put(s.nodes, sc->bvh_nodes, sc->node_count * 32, "BVH");
    if (!rc) rc = put(s.srgb, sc->srgb_texture_atlases, sc->srgb_atlas_count * layer, "atlases");
    if (!rc) rc = put(s.linear, sc->linear_texture_atlases, sc->linear_atlas_count * layer, "atlases");
    if (!rc) rc = put(s.sky, sk->rgba, texels * 16, "skybox");
    if (!rc && form.half) {
        // narrow copies on the device; the FP32 ones are dropped once converted
        rc = e->cuda(s.attr_h.alloc(sc->triangle_count * sizeof(pt_half_attribute)), "FP16 attributes");
        if (!rc) rc = e->cuda(ptw::convert_half_attributes(s.attr.as<pt_triangle_attribute>(), sc->triangle_count,
                                                           s.attr_h.as<uint2>(), e->stream), "FP16 attributes");
        if (!rc) rc = e->cuda(s.sky_h.alloc(texels * 8), "BF16 skybox");
        if (!rc) rc = e->cuda(ptw::convert_bf16_sky(s.sky.as<float4>(), texels, s.sky_h.as<uint2>(), e->stream),
                              "BF16 skybox");
        if (!rc) rc = e->cuda(cudaStreamSynchronize(e->stream), "narrow copies");
        if (!rc) {
            s.attr.release();
            s.sky.release();
        }
    }
    if (!rc && form.wide) {
        uint32_t depth = 0;
        std::vector<pt_wide_node> wide;
        if (ptw::build_wide_bvh(sc->bvh_nodes, sc->node_count, kWideLeafMerge, wide, &depth) != PT_OK)
            return e->fail(PT_ERR_INVALID_ARG, "the BVH cannot be collapsed into 8-wide nodes");
        const uint64_t count = wide.size();
        std::vector<uint32_t> links(sc->node_count + sc->triangle_count);
        if (!ptw::build_bvh_links(sc->bvh_nodes, sc->node_count, sc->triangle_count, links.data(),
                                  links.data() + sc->node_count))
            return e->fail(PT_ERR_INVALID_ARG, "BVH child or triangle range out of bounds");
        rc = put(s.wide, wide.data(), count * sizeof(pt_wide_node), "wide BVH");
        if (!rc) rc = put(s.links, links.data(), links.size() * 4, "BVH links");
        if (!rc) rc = e->cuda(cudaStreamSynchronize(e->stream), "wide BVH");  // the host copies go out of scope
    }
    if (!rc) rc = put(s.sky_alias, sk->alias_table, sk->alias_count * 12, "skybox aliases");
    if (!rc) rc = put(s.scene_alias, u->scene_alias_table, u->scene_alias_count * 16, "scene aliases");
    float lut[256];
    for (int i = 0; i < 256; ++i) {
        const double v = (double)i / 255.0;
        lut[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
    if (!rc) rc = put(s.lut, lut, sizeof lut, "sRGB table");
    if (!rc) rc = e->cuda(s.pairs.alloc((sc->node_count + 1) * 32 + 256), "BVH layout");
    if (!rc)
        rc = e->cuda(cudaMemcpyAsync(static_cast<char*>(s.pairs.p) + 32, s.nodes.p, sc->node_count * 32,
                                     cudaMemcpyDeviceToDevice, e->stream), "BVH layout");
    if (!rc) rc = e->cuda(s.tri4.alloc(sc->triangle_count * 16 * ptd::kTriStride), "triangle layout");
    if (!rc) {
        pad_triangles_kernel<<<(unsigned)((sc->triangle_count + 255) / 256), 256, 0, e->stream>>>(
            s.geo.as<pt_triangle_geometry>(), sc->triangle_count, s.tri4.as<float4>());
        rc = e->cuda(cudaGetLastError(), "triangle layout");
    }
    if (rc) return rc;
    SceneDev d{};
    World& w = d.w;
    w.geo = s.geo.as<pt_triangle_geometry>();
    w.attr = s.attr.p ? s.attr.as<pt_triangle_attribute>() : nullptr;
    w.attr_h = s.attr_h.p ? s.attr_h.as<uint2>() : nullptr;
    w.mat = s.mat.as<pt_material>();
    w.nodes = s.nodes.as<pt_bvh_node>();
    w.srgb = sc->srgb_atlas_count ? s.srgb.as<uint8_t>() : nullptr;
    w.linear = sc->linear_atlas_count ? s.linear.as<uint8_t>() : nullptr;
    w.srgb_count = sc->srgb_atlas_count;
    w.linear_count = sc->linear_atlas_count;
    w.sky = s.sky.p ? s.sky.as<float4>() : nullptr;
    w.sky_h = s.sky_h.p ? s.sky_h.as<uint2>() : nullptr;
    w.sky_alias = s.sky_alias.as<pt_skybox_alias_entry>();
    w.scene_alias = s.scene_alias.as<pt_scene_alias_entry>();
    w.sky_u = *u->skybox_uniforms;
    w.scene = *u->scene_uniforms;
    w.srgb_lut = s.lut.as<float>();
    w.any_alpha = s.any_alpha ? 1 : 0;
    w.attr16 = 1;  // a device allocation
    if (ptd::kTriStride == 4) w.tri64 = s.tri4.as<float4>();  // the shading frame's vertices
    d.f.pairs = reinterpret_cast<const float4*>(static_cast<const char*>(s.pairs.p) + 32);
    d.f.tri4 = s.tri4.as<float4>();
    d.f.wide = s.wide.p ? s.wide.as<float4>() : nullptr;
    d.f.parent = s.links.p ? s.links.as<uint32_t>() : nullptr;
    d.f.leaf_of = s.links.p ? s.links.as<uint32_t>() + sc->node_count : nullptr;
    rc = e->cuda(cudaMemcpyAsync(e->d_scenes.as<SceneDev>() + s.slot, &d, sizeof d, cudaMemcpyHostToDevice, e->stream),
                 "scene record");
    if (!rc) rc = e->cuda(cudaStreamSynchronize(e->stream), "scene upload");
    return rc;
}

SceneForm scene_form(const pt_engine* e, bool any_alpha) {
    SceneForm f;
    f.wide = (e->cfg.precision & PT_PRECISION_WIDE_BVH) != 0 && !any_alpha;
    f.half = (e->cfg.precision & PT_PRECISION_HALF_ATTRIBUTES) != 0;
    return f;
}

bool evict_one(pt_engine* e) {
    Scene* victim = nullptr;
    for (auto& [id, s] : e->scenes)
        if (s->caller_refs <= 0 && s->job_refs <= 0 && (!victim || s->last_use < victim->last_use)) victim = s.get();
    if (!victim) return false;
    e->used -= victim->bytes;
    e->scene_slots[victim->slot] = 0;
    e->stats.scenes_evicted += 1;
    e->scenes.erase(victim->id);
    return true;
}

}  // namespace

// The background pump: while a wave runs, every ~20 us finished waves are
// harvested and the next one queued, so the stream stays busy while the
// caller is busy between calls (PT_ENGINE_FLIGHTS waves in flight at most).
static void pump_loop(pt_engine* e) {
    cudaSetDevice(e->cfg.device);
    while (!e->stop.load(std::memory_order_relaxed)) {
        bool idle;
        {
            std::lock_guard<std::recursive_mutex> g(e->mu);
            if (e->sticky == PT_OK) {
                int rc;
                try {
                    rc = harvest(e, false);
                    if (!rc) rc = pump(e);
                } catch (...) {  // an exception leaving this thread would end the process
                    rc = pt_abi_current_status(&e->error);
                }
                if (rc) e->sticky = rc;
            }
            idle = e->flights.empty();  // nothing on the GPU and nothing queued by pump()
        }
        // while idle, a submit queues its own first wave, so a slower poll costs no latency
        std::this_thread::sleep_for(std::chrono::microseconds(idle ? 1000 : 20));
    }
}

namespace {
// inside a catch handler of an engine entry point: the status, with the
// message kept as the engine's last error under its lock (the engine's
// thread writes it too)
int engine_abi_status(pt_engine* e) noexcept {
    if (!e) return pt_abi_current_status(nullptr);
    try {
        std::lock_guard<std::recursive_mutex> lock(e->mu);
        return pt_abi_current_status(&e->error);
    } catch (...) {
        return pt_abi_current_status(nullptr);
    }
}
}  // namespace

extern "C" {

int pte_create(const pt_engine_config* cfg, pt_engine** out) try {
    if (!out) return PT_ERR_INVALID_ARG;
    *out = nullptr;
    pt_engine* e = new pt_engine();
    if (cfg) e->cfg = *cfg;
    if (!cfg) e->cfg.use_graphs = 1;
    if (e->cfg.wave_paths == 0) e->cfg.wave_paths = 1u << 22;
    if (e->cfg.tile_size == 0) e->cfg.tile_size = 32;
    if (e->cfg.steps_per_refill == 0) e->cfg.steps_per_refill = 32;
    if (e->cfg.sort_min_hits == 0) e->cfg.sort_min_hits = 65536u;
    if (e->cfg.traversal_threads == 0) e->cfg.traversal_threads = kExtendThreads;
    if (e->cfg.shade_threads == 0) e->cfg.shade_threads = kShadeThreads;
    e->budget = e->cfg.hbm_budget_bytes ? e->cfg.hbm_budget_bytes : 150ull << 30;
    int rc = PT_OK;
    if (e->cfg.tile_size > 256 || e->cfg.wave_paths < (1u << 12) || e->cfg.wave_paths > (1u << 28))
        rc = e->fail(PT_ERR_INVALID_ARG, "tile_size must be at most 256 and wave_paths in [4096, 2^28]");
    if (!rc && (e->cfg.precision & ~PT_PRECISION_COMPRESSED))
        rc = e->fail(PT_ERR_INVALID_ARG, "unknown precision bits");
    const uint32_t tt = e->cfg.traversal_threads, st = e->cfg.shade_threads;
    if (!rc && !((tt == 64u || tt == 128u || tt == 256u) && (st == 128u || st == 256u || st == 512u || st == 1024u)))
        rc = e->fail(PT_ERR_INVALID_ARG, "traversal_threads must be 64, 128 or 256 and shade_threads 128, 256, 512 or 1024");
    if (!rc) rc = e->cuda(cudaSetDevice(e->cfg.device), "cudaSetDevice");
    if (!rc) rc = e->cuda(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "stream");
    if (!rc) rc = e->cuda(cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, e->cfg.device), "SM count");
    if (!rc) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = e->cfg.device;
        rc = e->cuda(cudaMemPoolCreate(&e->pool, &props), "memory pool");
        uint64_t keep = ~0ull;
        if (!rc) rc = e->cuda(cudaMemPoolSetAttribute(e->pool, cudaMemPoolAttrReleaseThreshold, &keep), "memory pool");
    }
    if (!rc) rc = e->cuda(e->d_scenes.alloc(kMaxScenes * sizeof(SceneDev)), "scene table");
    if (!rc) rc = e->cuda(e->d_jobs.alloc((size_t)kMaxSlots * sizeof(JobDev)), "job table");
    if (!rc) rc = e->cuda(e->d_done.alloc((size_t)kMaxSlots * 4), "job counters");
    if (!rc) rc = e->cuda(cudaMemset(e->d_done.p, 0, (size_t)kMaxSlots * 4), "job counters");
    if (!rc) rc = e->cuda(e->d_ring.alloc(e->ring_cap * sizeof(ItemDev)), "work ring");
    if (!rc) rc = e->cuda(e->d_ctrl.alloc(sizeof(Ctrl)), "ring control");
    if (!rc) rc = e->cuda(cudaMemset(e->d_ctrl.p, 0, sizeof(Ctrl)), "ring control");
    if (!rc) rc = e->cuda(cudaHostAlloc((void**)&e->h_done, (size_t)kMaxSlots * 4, cudaHostAllocDefault), "pinned counters");
    if (!rc) rc = e->cuda(cudaHostAlloc((void**)&e->h_ctrl, sizeof(Ctrl), cudaHostAllocDefault), "pinned counters");
    if (!rc) {
        memset(e->h_done, 0, (size_t)kMaxSlots * 4);
        memset(e->h_ctrl, 0, sizeof(Ctrl));
        e->used = kMaxScenes * sizeof(SceneDev) + (size_t)kMaxSlots * (sizeof(JobDev) + 4) + e->ring_cap * sizeof(ItemDev);
        e->scene_slots.assign(kMaxScenes, 0);
        e->slots.resize(kMaxSlots);
        e->slot_items.assign(kMaxSlots, 0);
        rc = setup_wave(e);
    }
    if (rc) {
        fprintf(stderr, "pte_create: %s\n", e->error.c_str());
        pte_destroy(e);
        return rc;
    }
    try {
        e->pumper = std::thread(pump_loop, e);
    } catch (const std::system_error&) {
        fprintf(stderr, "pte_create: the engine's background thread could not be started\n");
        pte_destroy(e);
        return PT_ERR_STATE;
    }
    *out = e;
    return PT_OK;
} catch (...) {
    return pt_abi_current_status(nullptr);
}

void pte_destroy(pt_engine* e) {
    if (!e) return;
    e->stop.store(true);
    if (e->pumper.joinable()) e->pumper.join();
    cudaSetDevice(e->cfg.device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    for (auto& f : e->flights) {
        cudaEventDestroy(f.start);
        cudaEventDestroy(f.stop);
    }
    for (cudaEvent_t ev : e->event_pool) cudaEventDestroy(ev);
    e->jobs.clear();
    for (auto& s : e->slots) s.reset();
    e->scenes.clear();
    if (e->stream) cudaStreamSynchronize(e->stream);  // the stream-ordered frees above
    if (e->pool) cudaMemPoolDestroy(e->pool);
    if (e->h_done) cudaFreeHost(e->h_done);
    if (e->h_ctrl) cudaFreeHost(e->h_ctrl);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

const char* pte_last_error(const pt_engine* e) {
    if (!e) return "null engine";
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    return e->error.c_str();
}

int pte_scene_add(pt_engine* e, const pt_world_updates* u, uint64_t* scene_id) try {
    if (!e || !u || !scene_id) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    if (!u->scene || !u->skybox || !u->scene_uniforms || !u->skybox_uniforms || !u->scene_alias_table)
        return e->fail(PT_ERR_INVALID_ARG, "a scene needs a full upload (scene, skybox, uniforms, alias table)");
    cudaSetDevice(e->cfg.device);
    // the same checks pt_create applies, through a throwaway context would cost an
    // upload; check the structural invariants the kernels rely on here
    const pt_scene_upload* sc = u->scene;
    if (!sc->geometries || !sc->attributes || !sc->materials || !sc->bvh_nodes || sc->triangle_count == 0 ||
        sc->node_count == 0 || sc->material_count == 0)
        return e->fail(PT_ERR_INVALID_ARG, "scene upload is incomplete");
    for (uint64_t i = 0; i < sc->triangle_count; ++i)
        if (sc->attributes[i].material_index >= sc->material_count)
            return e->fail(PT_ERR_INVALID_ARG, "triangle material index outside the material buffer");
    {
        std::vector<uint8_t> seen(sc->node_count, 0);
        std::vector<std::pair<uint64_t, uint32_t>> st{{0, 0}};
        while (!st.empty()) {
            auto [i, depth] = st.back();
            st.pop_back();
            if (seen[i]) return e->fail(PT_ERR_INVALID_ARG, "BVH node reached twice (not a tree)");
            seen[i] = 1;
            const pt_bvh_node& n = sc->bvh_nodes[i];
            if (n.tri_count > 0) {
                if ((uint64_t)n.left_first + n.tri_count > sc->triangle_count)
                    return e->fail(PT_ERR_INVALID_ARG, "BVH leaf triangle range outside the triangle buffer");
            } else {
                if (depth >= 64) return e->fail(PT_ERR_OUT_OF_LIMITS, "BVH deeper than the 64-entry traversal stack");
                if ((uint64_t)n.left_first + 1 >= sc->node_count || n.left_first == 0)
                    return e->fail(PT_ERR_INVALID_ARG, "BVH child index outside the node buffer");
                st.push_back({n.left_first, depth + 1});
                st.push_back({(uint64_t)n.left_first + 1, depth + 1});
            }
        }
    }
    const pt_skybox_upload* sk = u->skybox;
    const pt_scene_uniforms& su = *u->scene_uniforms;
    const float p0 = su.light_probabilities[0], p1 = su.light_probabilities[1];
    if (!(p0 >= 0.0f && p1 >= 0.0f) || su.emissive_triangles_count > u->scene_alias_count ||
        (p0 > 0.0f && su.emissive_triangles_count == 0) ||
        ((p1 > 0.0f || (p0 + p1 > 0.0f && p0 < 1.0f)) &&
         (sk->alias_count == 0 || sk->alias_count != (uint64_t)sk->uniforms.width * sk->uniforms.height)))
        return e->fail(PT_ERR_INVALID_ARG, "light tables are inconsistent with the light probabilities");
    for (uint64_t i = 0; i < u->scene_alias_count; ++i)
        if (u->scene_alias_table[i].triangle_index >= sc->triangle_count ||
            u->scene_alias_table[i].alias_index >= u->scene_alias_count)
            return e->fail(PT_ERR_INVALID_ARG, "scene alias entry out of range");
    for (uint64_t i = 0; i < sk->alias_count; ++i)
        if (sk->alias_table[i].alias_index >= sk->alias_count)
            return e->fail(PT_ERR_INVALID_ARG, "skybox alias index out of range");
    // content identity
    const size_t layer = (size_t)PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
    const Digest dg = hash_buffers({
        {sc->geometries, sc->triangle_count * 36},
        {sc->attributes, sc->triangle_count * 112},
        {sc->materials, sc->material_count * 224},
        {sc->bvh_nodes, sc->node_count * 32},
        {sc->srgb_texture_atlases, sc->srgb_atlas_count * layer},
        {sc->linear_texture_atlases, sc->linear_atlas_count * layer},
        {sk->rgba, (size_t)sk->uniforms.width * sk->uniforms.height * 16},
        {sk->alias_table, sk->alias_count * 12},
        {u->scene_alias_table, u->scene_alias_count * 16},
        {u->scene_uniforms, 16},
        {u->skybox_uniforms, 16},
    });
    e->use_clock += 1;
    // the first hash names the scene; an entry whose second hash differs is a
    // different scene, so probe on to the next free name (ids are never 0)
    uint64_t h = dg.a ? dg.a : 1;
    for (auto it = e->scenes.find(h); it != e->scenes.end(); it = e->scenes.find(h)) {
        if (it->second->check == dg.b) {
            it->second->caller_refs += 1;
            it->second->last_use = e->use_clock;
            e->stats.scene_hits += 1;
            *scene_id = h;
            return PT_OK;
        }
        h = h + 1 ? h + 1 : 1;
    }
    bool any_alpha = false;
    for (uint64_t i = 0; i < sc->material_count; ++i) any_alpha |= sc->materials[i].alpha_mode != PT_ALPHA_MODE_OPAQUE;
    const SceneForm form = scene_form(e, any_alpha);
    const uint64_t texels = (uint64_t)sk->uniforms.width * sk->uniforms.height;
    uint64_t bytes = sc->triangle_count * (36 + 16 * ptd::kTriStride) + sc->material_count * 224 + 512 +
                     (sc->srgb_atlas_count + sc->linear_atlas_count) * layer + sk->alias_count * 12 +
                     u->scene_alias_count * 16 + 1024;
    bytes += form.half ? sc->triangle_count * 64 + texels * 8 : sc->triangle_count * 112 + texels * 16;
    bytes += sc->node_count * 64 + 256;             // binary nodes + child-pair copy
    bytes += form.wide ? sc->node_count * (64 + 4) + sc->triangle_count * 4 : 0;  // wide nodes (at most one per
                                                                                   // two binary nodes) + links
    while (e->used + bytes > e->budget && evict_one(e)) {
    }
    if (e->used + bytes > e->budget) return hbm_fail(e->error, "the scene", bytes, e->used, e->budget);
    uint32_t slot = kMaxScenes;
    for (uint32_t i = 0; i < kMaxScenes; ++i)
        if (e->scene_slots[i] == 0) {
            slot = i;
            break;
        }
    if (slot == kMaxScenes) {
        if (!evict_one(e)) return e->fail(PT_ERR_OUT_OF_LIMITS, "scene table full (256 scenes)");
        for (uint32_t i = 0; i < kMaxScenes; ++i)
            if (e->scene_slots[i] == 0) {
                slot = i;
                break;
            }
    }
    auto s = std::make_unique<Scene>();
    s->id = h;
    s->check = dg.b;
    s->slot = slot;
    s->bytes = bytes;
    s->caller_refs = 1;
    s->last_use = e->use_clock;
    s->any_alpha = any_alpha;
    int rc = upload_scene(e, *s, u);
    if (rc) return rc;
    e->scene_slots[slot] = h;
    e->used += bytes;
    e->scenes[h] = std::move(s);
    e->stats.scenes_cached = e->scenes.size();
    *scene_id = h;
    return PT_OK;
} catch (...) {
    return engine_abi_status(e);
}

int pte_scene_release(pt_engine* e, uint64_t scene_id) try {
    if (!e) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    auto it = e->scenes.find(scene_id);
    if (it == e->scenes.end()) return e->fail(PT_ERR_INVALID_ARG, "unknown scene");
    it->second->caller_refs -= 1;
    return PT_OK;
} catch (...) {
    return engine_abi_status(e);
}

int pte_submit(pt_engine* e, const pt_job_desc* d, uint64_t* job_id) try {
    if (!e || !d || !job_id) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    cudaSetDevice(e->cfg.device);
    if (d->samples == 0 || d->max_bounces > PT_MAX_BOUNCES_LIMIT)
        return e->fail(PT_ERR_INVALID_ARG, "samples must be positive and max_bounces at most 16");
    Job j;
    j.camera = d->camera;
    j.samples = d->samples;
    j.submitted = std::chrono::steady_clock::now();
    if (d->continue_job) {
        auto it = e->jobs.find(d->continue_job);
        if (it == e->jobs.end() || !it->second.acc) return e->fail(PT_ERR_INVALID_ARG, "unknown job to continue");
        j.acc = it->second.acc;
        if (j.acc->scene != d->scene_id || j.acc->width != d->width || j.acc->height != d->height ||
            j.acc->max_bounces != d->max_bounces)
            return e->fail(PT_ERR_INVALID_ARG, "a continued job must keep its scene, size and max_bounces");
    } else {
        auto sit = e->scenes.find(d->scene_id);
        if (sit == e->scenes.end()) return e->fail(PT_ERR_INVALID_ARG, "unknown scene");
        if (d->width == 0 || d->height == 0 || d->width > 16384 || d->height > 16384)
            return e->fail(PT_ERR_OUT_OF_LIMITS, "image size must be within 1..16384");
        uint32_t slot = kMaxSlots;
        for (uint32_t i = 0; i < kMaxSlots; ++i)
            if (!e->slots[i]) {
                slot = i;
                break;
            }
        if (slot == kMaxSlots) return e->fail(PT_ERR_OUT_OF_LIMITS, "too many live jobs");
        const bool kahan = (e->cfg.precision & PT_PRECISION_KAHAN) != 0;
        const uint64_t bytes = (uint64_t)d->width * d->height * (kahan ? 48 : 32);
        while (e->used + bytes > e->budget && evict_one(e)) {
        }
        if (e->used + bytes > e->budget) return hbm_fail(e->error, "the job's accumulation", bytes, e->used, e->budget);
        auto a = std::make_shared<Accumulation>();
        a->slot = slot;
        a->scene = d->scene_id;
        a->width = d->width;
        a->height = d->height;
        a->max_bounces = d->max_bounces;
        a->bytes = bytes;
        const size_t plane = (size_t)d->width * d->height * 16;
        int rc = e->cuda(a->accum.alloc(plane, e->pool, e->stream), "accumulation buffer");
        if (!rc) rc = e->cuda(a->image.alloc(plane, e->pool, e->stream), "image buffer");
        if (!rc && kahan) rc = e->cuda(a->comp.alloc(plane, e->pool, e->stream), "Kahan compensation");
        if (rc) return rc;
        e->used += bytes;
        e->slots[slot] = a;
        sit->second->job_refs += 1;
        sit->second->last_use = ++e->use_clock;
        j.acc = a;
    }
    const uint64_t tile_px = (uint64_t)e->cfg.tile_size * e->cfg.tile_size;
    if (tile_px * d->samples > e->cfg.wave_paths)
        return e->fail(PT_ERR_OUT_OF_LIMITS, "samples per pass times the tile area exceed the wave budget; split into continued jobs");
    j.id = e->next_job++;
    e->jobs[j.id] = j;
    e->stats.jobs_submitted += 1;
    Job& stored = e->jobs[j.id];
    stored.acc->job_refs += 1;
    int rc = PT_OK;
    if (stored.acc->busy)
        stored.acc->waiting.push_back(j.id);
    else
        rc = start_job(e, stored);
    if (rc) return rc;
    *job_id = j.id;
    return pump(e);
} catch (...) {
    return engine_abi_status(e);
}

int pte_poll(pt_engine* e, uint32_t timeout_ms, uint64_t* done, uint32_t capacity, uint32_t* count) try {
    if (!e || !count || (capacity && !done)) return PT_ERR_INVALID_ARG;
    cudaSetDevice(e->cfg.device);
    *count = 0;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        {
            std::lock_guard<std::recursive_mutex> lock(e->mu);
            if (e->sticky) return e->sticky;
            int rc = harvest(e, false);
            if (!rc) rc = pump(e);
            if (rc) return rc;
            while (*count < capacity && !e->done_unreported.empty()) {
                done[(*count)++] = e->done_unreported.front();
                e->done_unreported.pop_front();
            }
            if (*count > 0 || e->flights.empty() || std::chrono::steady_clock::now() >= deadline) return PT_OK;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
} catch (...) {
    return engine_abi_status(e);
}

int pte_wait_idle(pt_engine* e, uint32_t timeout_ms) try {
    if (!e) return PT_ERR_INVALID_ARG;
    cudaSetDevice(e->cfg.device);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        {
            std::lock_guard<std::recursive_mutex> lock(e->mu);
            if (e->sticky) return e->sticky;
            int rc = harvest(e, false);
            if (!rc) rc = pump(e);
            if (rc) return rc;
            bool busy = !e->flights.empty();
            for (auto& [id, j] : e->jobs) busy |= j.status != PT_JOB_DONE;
            if (!busy) return PT_OK;
            if (timeout_ms && std::chrono::steady_clock::now() >= deadline)
                return e->fail(PT_ERR_TIMEOUT, "engine still busy");
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
} catch (...) {
    return engine_abi_status(e);
}

int pte_job_status(pt_engine* e, uint64_t id, int* status, uint32_t* samples_done) try {
    if (!e) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    auto it = e->jobs.find(id);
    if (it == e->jobs.end()) return e->fail(PT_ERR_INVALID_ARG, "unknown job");
    if (status) *status = it->second.status;
    if (samples_done) *samples_done = it->second.acc ? it->second.acc->samples_done : 0;
    return PT_OK;
} catch (...) {
    return engine_abi_status(e);
}

int pte_job_read(pt_engine* e, uint64_t id, int which, float* host) try {
    if (!e || !host || (which != PT_TILE_IMAGE && which != PT_TILE_ACCUMULATION && which != PT_TILE_COMPENSATION))
        return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    cudaSetDevice(e->cfg.device);
    auto it = e->jobs.find(id);
    if (it == e->jobs.end() || !it->second.acc) return e->fail(PT_ERR_INVALID_ARG, "unknown job");
    if (it->second.status != PT_JOB_DONE) return e->fail(PT_ERR_STATE, "job not finished");
    Accumulation& a = *it->second.acc;
    if (which == PT_TILE_COMPENSATION && !a.comp.p) {
        memset(host, 0, (size_t)a.width * a.height * 16);
        return PT_OK;
    }
    const StreamBuf& b = which == PT_TILE_IMAGE ? a.image : (which == PT_TILE_ACCUMULATION ? a.accum : a.comp);
    int rc = e->cuda(cudaMemcpyAsync(host, b.p, (size_t)a.width * a.height * 16, cudaMemcpyDeviceToHost, e->stream), "job readback");
    if (!rc) rc = e->cuda(cudaStreamSynchronize(e->stream), "job readback");
    return rc;
} catch (...) {
    return engine_abi_status(e);
}

int pte_job_release(pt_engine* e, uint64_t id) try {
    if (!e) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    cudaSetDevice(e->cfg.device);
    auto it = e->jobs.find(id);
    if (it == e->jobs.end()) return e->fail(PT_ERR_INVALID_ARG, "unknown job");
    if (it->second.status != PT_JOB_DONE) return e->fail(PT_ERR_STATE, "job not finished");
    std::shared_ptr<Accumulation> a = it->second.acc;
    e->jobs.erase(it);
    if (a) {
        a->job_refs -= 1;
        if (a->job_refs == 0 && !a->busy && a->waiting.empty()) {
            // no wave can still touch the buffers: the job is done and nothing is queued on them
            free_accumulation(e, *a);
        }
    }
    return PT_OK;
} catch (...) {
    return engine_abi_status(e);
}

int pte_stats(pt_engine* e, pt_engine_stats* s) try {
    if (!e || !s) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    *s = e->stats;
    s->scenes_cached = e->scenes.size();
    s->hbm_used = e->used;
    s->hbm_budget = e->budget;
    s->wave_paths = e->cfg.wave_paths;
    s->tile_size = e->cfg.tile_size;
    s->steps_per_refill = e->cfg.steps_per_refill;
    s->precision = e->cfg.precision;
    s->sort_min_hits = e->cfg.sort_min_hits;
    s->use_graphs = e->cfg.use_graphs;
    s->traversal_threads = e->cfg.traversal_threads;
    s->shade_threads = e->cfg.shade_threads;
    return PT_OK;
} catch (...) {
    return engine_abi_status(e);
}

int pte_autotune(pt_engine* e, const pt_job_desc* jobs, uint32_t count, pt_engine_config* chosen) try {
    if (!e || !jobs || count == 0) return PT_ERR_INVALID_ARG;
    std::lock_guard<std::recursive_mutex> lock(e->mu);
    if (e->sticky) return e->sticky;
    cudaSetDevice(e->cfg.device);
    int rc = pte_wait_idle(e, 0);
    if (rc) return rc;
    const uint32_t waves[] = {1u << 20, 1u << 21, 1u << 22, 1u << 23};
    const uint32_t tiles[] = {16, 32, 64};
    const uint32_t steps[] = {16, 32};
    const uint32_t sorts[] = {0xffffffffu, 65536u};
    const uint32_t traversal_shapes[] = {64, 128, 256};
    const uint32_t shade_shapes[] = {128, 256, 512, 1024};
    pt_engine_config best = e->cfg;
    double best_rate = -1.0;
    // renders the jobs under e->cfg: one untimed pass to capture graphs, then the timed pass
    const auto measure = [&]() -> int {
        drop_graphs(e);
        for (int pass = 0; pass < 2; ++pass) {
            const double ms0 = e->stats.gpu_ms;
            const uint64_t paths0 = e->stats.paths;
            std::vector<uint64_t> ids;
            for (uint32_t k = 0; k < count; ++k) {
                pt_job_desc d = jobs[k];
                d.continue_job = 0;
                uint64_t id = 0;
                if (int r = pte_submit(e, &d, &id)) return r;
                ids.push_back(id);
            }
            if (int r = pte_wait_idle(e, 0)) return r;
            for (uint64_t id : ids) pte_job_release(e, id);
            e->done_unreported.clear();
            const double ms = e->stats.gpu_ms - ms0;
            const double rate = (double)(e->stats.paths - paths0) / (ms > 0 ? ms : 1e-9);
            if (pass == 1 && rate > best_rate) {
                best_rate = rate;
                best = e->cfg;
            }
        }
        return PT_OK;
    };
    for (uint32_t W : waves)
        for (uint32_t T : tiles)
            for (uint32_t S : steps)
            for (uint32_t H : sorts) {
                bool fits = true;
                for (uint32_t k = 0; k < count; ++k) fits &= (uint64_t)T * T * jobs[k].samples <= W;
                if (!fits) continue;
                if (W != e->cfg.wave_paths) {
                    e->cfg.wave_paths = W;
                    if ((rc = setup_wave(e))) return rc;
                }
                e->cfg.tile_size = T;
                e->cfg.steps_per_refill = S;
                e->cfg.sort_min_hits = H;
                if ((rc = measure())) return rc;
            }
    // block shapes, with the best of the above
    if (best.wave_paths != e->cfg.wave_paths) {
        e->cfg.wave_paths = best.wave_paths;
        if ((rc = setup_wave(e))) return rc;
    }
    const pt_engine_config base = best;
    for (uint32_t TT : traversal_shapes)
        for (uint32_t ST : shade_shapes) {
            if (TT == base.traversal_threads && ST == base.shade_threads) continue;  // measured above
            e->cfg = base;
            e->cfg.traversal_threads = TT;
            e->cfg.shade_threads = ST;
            if ((rc = measure())) return rc;
        }
    if (best.wave_paths != e->cfg.wave_paths) {
        e->cfg.wave_paths = best.wave_paths;
        if ((rc = setup_wave(e))) return rc;
    }
    e->cfg = best;
    drop_graphs(e);
    if (chosen) *chosen = best;
    return PT_OK;
} catch (...) {
    return engine_abi_status(e);
}

}  // extern "C"
