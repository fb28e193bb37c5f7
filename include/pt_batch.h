/*
 * pt_batch.h - C ABI of the batched, continuously fed render engine.
 *
 * The reference renders one job at a time: one tile, at most 16 samples per
 * submit, the host waiting between submits (headless.rs:207-285,
 * path_tracer.rs:316-351).  This engine serves many render jobs of uneven
 * size, sample count, depth and scene on one GPU at once:
 *
 *   - scenes are uploaded once and cached on the device under a hash of
 *     their content, within an HBM budget (least recently used scenes that no
 *     job uses are evicted first);
 *   - a job is (scene, camera, width x height, samples, max_bounces); its
 *     accumulation buffer stays on the device, so a later job can add samples
 *     to it (progressive refinement, the accumulation rule of
 *     trace.slang:1299-1308 continued across passes);
 *   - jobs are cut into work items (tile x sample range) placed in a device
 *     ring; every wave a planner kernel packs queued items into a fixed path
 *     budget and the wavefront kernels trace them together, whatever job they
 *     belong to; work submitted while a wave runs joins the next wave;
 *   - each wave is replayed from a captured CUDA graph;
 *   - a background thread of the engine harvests finished waves and queues
 *     the next ones every 100 us, so the GPU stays fed while the caller's
 *     thread is busy between calls (at most two waves in flight).
 * Every path computes exactly what pt_trace computes for the same pixel and
 * sample, and each pixel accumulates its samples in order, so a job's result
 * is bit-identical whether it runs alone or mixed with others.
 *
 * All functions return PT_OK or an error code from pt.h; pte_last_error gives
 * the message.  Calls on one engine may come from several threads; they are
 * serialised with the background thread by a lock.  An error of the
 * background thread is returned by every later call.
 */
#ifndef PT_BATCH_H
#define PT_BATCH_H

#include "pt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pt_engine pt_engine;

typedef struct pt_engine_config {
    int device;
    uint64_t hbm_budget_bytes;  /* scenes + job buffers + wave buffers; 0 = 150 GB */
    uint32_t wave_paths;        /* paths traced per wave; 0 = 4 Mi */
    uint32_t tile_size;         /* work-item tile side in pixels; 0 = 32 */
    uint32_t steps_per_refill;  /* node visits between traversal lane refills; 0 = 32 */
    uint32_t use_graphs;        /* 1 = replay waves from a captured CUDA graph (default), 0 = plain launches */
    uint32_t precision;         /* PT_PRECISION_* bits of include/pt_precision.h; 0 = the reference's FP32
                                   buffers.  With PT_PRECISION_HALF_ATTRIBUTES a cached scene keeps only
                                   the FP16 attributes and BF16 skybox; with PT_PRECISION_WIDE_BVH an
                                   opaque scene keeps only the 8-wide BVH */
    uint32_t sort_min_hits;     /* a bounce with at least this many hits sorts them by triangle bucket
                                   (1024 triangles each, BVH order) before shading; 0 = 65536,
                                   0xffffffff = never */
    uint32_t traversal_threads; /* threads per block of the extend and shadow kernels: 64, 128 or 256
                                   (the register budget per thread stays the same); 0 = 128 */
    uint32_t shade_threads;     /* threads per block of the shading kernel: 128, 256, 512 or 1024
                                   (64 registers per thread); 0 = 1024 */
} pt_engine_config;

int pte_create(const pt_engine_config* config, pt_engine** out);
void pte_destroy(pt_engine* engine);
const char* pte_last_error(const pt_engine* engine);

/* Upload a scene (a full upload as ptw_take_updates produces it: scene,
 * skybox, scene/skybox uniforms and the scene alias table; the camera is per
 * job).  A scene with identical content returns the id of the cached copy.
 * Fails with PT_ERR_OOM when the HBM budget cannot hold it. */
int pte_scene_add(pt_engine* engine, const pt_world_updates* full_upload, uint64_t* scene_id);
/* the caller no longer needs the scene; it stays cached until evicted */
int pte_scene_release(pt_engine* engine, uint64_t scene_id);

typedef struct pt_job_desc {
    uint64_t scene_id;
    pt_camera camera;        /* GpuCamera of this job (world.rs:2159-2173) */
    uint32_t width, height;  /* image size; the job covers the whole image */
    uint32_t samples;        /* samples per pixel this job adds */
    uint32_t max_bounces;    /* 0..16 */
    uint64_t continue_job;   /* 0: new accumulation; else the id of a job whose
                                accumulation (same scene, size, depth) receives
                                the samples; it starts once that job is done */
} pt_job_desc;

/* Queue a job.  Fails with PT_ERR_OOM if its buffers exceed the HBM budget. */
int pte_submit(pt_engine* engine, const pt_job_desc* job, uint64_t* job_id);

/* Launch waves while work is queued (at most two in flight) and collect
 * finished jobs, waiting at most timeout_ms for one to finish; writes up to
 * `capacity` finished job ids to `done`. */
int pte_poll(pt_engine* engine, uint32_t timeout_ms, uint64_t* done, uint32_t capacity, uint32_t* count);
/* run until no work is queued or in flight (PT_ERR_TIMEOUT after timeout_ms; 0 = no limit) */
int pte_wait_idle(pt_engine* engine, uint32_t timeout_ms);

#define PT_JOB_QUEUED 0
#define PT_JOB_RUNNING 1
#define PT_JOB_DONE 2
int pte_job_status(pt_engine* engine, uint64_t job_id, int* status, uint32_t* samples_done);
/* PT_TILE_IMAGE, PT_TILE_ACCUMULATION or (Kahan engines) PT_TILE_COMPENSATION of a
 * finished job: width * height * 4 floats */
int pte_job_read(pt_engine* engine, uint64_t job_id, int which, float* host_rgba);
/* free the job's buffers (a job continued by another keeps them until that one is released) */
int pte_job_release(pt_engine* engine, uint64_t job_id);

typedef struct pt_engine_stats {
    uint64_t waves;
    uint64_t items;
    uint64_t paths;
    uint64_t jobs_submitted;
    uint64_t jobs_done;
    uint64_t scenes_cached;
    uint64_t scene_hits;         /* pte_scene_add calls served from the cache */
    uint64_t scenes_evicted;
    uint64_t hbm_used;
    uint64_t hbm_budget;
    double gpu_ms;               /* device time of all finished waves (CUDA events) */
    uint32_t wave_paths, tile_size, steps_per_refill, use_graphs, precision, sort_min_hits;
    uint32_t traversal_threads, shade_threads;
} pt_engine_stats;
int pte_stats(pt_engine* engine, pt_engine_stats* stats);

/* Autotuner: renders the given jobs once per candidate configuration
 * (wave_paths x tile_size x steps_per_refill x sort on/off, then, with the
 * best of those, the block shapes traversal_threads x shade_threads) and
 * keeps the one with the highest paths per second of device time; writes it
 * to *chosen.  The jobs' results are discarded. */
int pte_autotune(pt_engine* engine, const pt_job_desc* jobs, uint32_t count, pt_engine_config* chosen);

#ifdef __cplusplus
}
#endif

#endif /* PT_BATCH_H */
