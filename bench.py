#!/usr/bin/env python3
"""Benchmark of the GB300 path-trace pass: Mrays/s on the large procedural scene.

Workload (one step): the whole 1920x1080 image of the ~2.1M-triangle
procedural scene (1024x512-quad heightfield, 2000 boxes, 200 icospheres,
64 emissive triangles, 1024x512 sky), 64 samples per pixel, max_bounces 8,
traced through pt_trace in calls of at most 16 samples exactly as the
reference's headless loop does (one tile covering the image).  A ray is every
extend or shadow traversal.  The scene as the kernels read it (BVH child
pairs 75 MB + triangles padded to 64 bytes 134 MB + attributes 235 MB) is
larger than the 129 MB L2, so no L2 flush is needed
between steps.

Contract: python bench.py [--gpus N --steps K --warmup W] prints one JSON line.
`--impl reference` times the CPU restatement of the reference's trace pass
(oracle/, the reference itself cannot run here) on host cores instead.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path[:0] = [str(ROOT), str(ROOT / "path-tracer_gb300")]

import numpy as np  # noqa: E402

WIDTH, HEIGHT, SPP, MAX_BOUNCES = 1920, 1080, 64, 8
# the large procedural scene is the bench line; the 36-triangle Cornell room
# (256x256, 16 spp) is the small plain-method case, measured with --workload cornell
WORKLOADS = {
    "procedural": {"image": (1920, 1080), "spp": 64,
                   "text": "procedural scene (1024x512-quad heightfield + 2000 boxes + 200 icospheres s4 + 64 "
                           "emissive triangles, 1024x512 sky)",
                   "l2": "inputs larger than L2 (scene buffers ~440 MB vs 129 MB L2), no flush"},
    "procedural_4m": {"image": (1920, 1080), "spp": 64,
                      "text": "procedural scene of the serving mix (1024x1024-quad heightfield + 4000 boxes + 360 "
                              "icospheres s4 + 64 emissive triangles, 512x256 sky)",
                      "l2": "inputs larger than L2 (scene buffers ~1.1 GB vs 129 MB L2), no flush"},
    "cornell": {"image": (256, 256), "spp": 16,
                "text": "Cornell room (36 triangles: 5 wall quads, two rotated boxes, 0.25x0.25 emissive ceiling quad; "
                        "black sky)",
                "l2": "scene (~4 KB) resident in L1/L2 by nature; no flush (the case is bound by arithmetic, "
                      "not memory)"},
}
WORKLOAD = "procedural"
METRIC = "Mrays/s"
KERNEL_NAMES = {"wavefront": 0, "plain": 1}
# include/pt_precision.h: FP32 (the reference's buffers), 8-wide quantised BVH only, FP16 attributes /
# BF16 skybox + Kahan sums on the binary BVH, or the full compressed form (all three)
PRECISIONS = {"fp32": 0, "wide": 1, "half": 6, "compressed": 7}
# DRAM bytes (read + write) per launch of the dominant kernel on this workload
# (1920x1080, 64 spp, FP32 form), measured by a single-pass ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of the first 16-spp group's
# 9 extend launches
TRAFFIC_PER_LAUNCH: dict = {("wavefront", "extend", "fp32"): 583.1e6}
# warp instructions per path per launch of each kernel class (smsp__inst_executed.sum of the 9 launches
# of each class of one 960x540 16-spp image of this scene, over 9 launches x 8,294,400 paths; the
# per-path work of a launch does not depend on the image size); with the launch's paths and its
# CUDA-event time they give the fraction of the SMs' issue slots the kernel fills
WARP_INST_PER_PATH: dict = {("wavefront", "fp32"): {"extend": 95.04, "shade": 43.44, "shadow": 32.12},
                             ("wavefront", "compressed"): {"extend": 121.68, "shade": 44.08, "shadow": 43.92}}
SMS, SCHEDULERS_PER_SM = 152, 4


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--kernel", choices=list(KERNEL_NAMES), default="wavefront")
    p.add_argument("--precision", choices=list(PRECISIONS), default="fp32")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--workload", choices=list(WORKLOADS), default="procedural",
                   help="procedural: the large scene of the bench line; procedural_4m: the 4M-triangle scene of "
                        "the serving mix; cornell: the 36-triangle room")
    p.add_argument("--spp", type=int, default=None, help="samples per pixel of one step (default: the workload's)")
    p.add_argument("--profile-run", action="store_true",
                   help="only the timed steps (no counting pass, e2e or CPU baseline): for ncu captures")
    p.add_argument("--no-latency", action="store_true",
                   help="skip the request-latency measurement (batched engine vs the plain path)")
    p.add_argument("--no-mix", action="store_true",
                   help="skip the batching / serving measurement on the mixed request stream")
    p.add_argument("--no-fp64", action="store_true",
                   help="skip the image error against the FP64 reference render")
    p.add_argument("--mix-seconds", type=float, default=10.0, help="seconds of arrivals of the serving stream")
    p.add_argument("--dump-world", default=None, help=argparse.SUPPRESS)  # child process of --impl reference
    p.add_argument("--image", type=int, nargs=2, metavar=("W", "H"), default=None,
                   help="image size (default 1920 1080); smaller sizes are for ncu captures, not bench lines")
    args = p.parse_args()
    global WIDTH, HEIGHT, SPP, WORKLOAD
    WORKLOAD = args.workload
    WIDTH, HEIGHT = args.image or WORKLOADS[WORKLOAD]["image"]
    SPP = args.spp = args.spp or WORKLOADS[WORKLOAD]["spp"]
    return args


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def max_over_ranks(x: float, pg, device: str) -> float:
    """The largest value of `x` over the replicas (a job's time is its slowest replica's);
    `pg` is torch.distributed when more than one replica runs, else None."""
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_step: float, steps: int, world_size: int, seconds: float) -> float:
    """Whole-job throughput: every replica processes `units_per_step` per step (weak scaling)."""
    return units_per_step * steps * world_size / seconds


def workload_config(world, precision: str, replicas: int) -> dict:
    """The workload of a bench line; both arms print the same dict (the implementation that ran is the
    line's top-level "kernel")."""
    return {
        "workload": f"{WORKLOADS[WORKLOAD]['text']}, {WIDTH}x{HEIGHT}, {SPP} spp, max_bounces 8, one image per step",
        "triangles": int(world.triangle_count()),
        "bvh_nodes": int(world.node_count()),
        "image": [WIDTH, HEIGHT],
        "spp": SPP,
        "max_bounces": MAX_BOUNCES,
        "l2": WORKLOADS[WORKLOAD]["l2"],
        "seed": {"procedural": 1, "procedural_4m": 7}.get(WORKLOAD, 0),
        "precision": precision,
        "parallelism": f"replicas x{replicas}",
    }


def build_world():
    import pathtracer as pt
    if WORKLOAD == "procedural":
        world = pt.World.procedural()
    elif WORKLOAD == "procedural_4m":
        from pathtracer.serving import build_scene
        world = build_scene("4M")
    else:
        world = pt.World.cornell_box()
    world.set_aspect_ratio(WIDTH / HEIGHT)
    return world, world.take_updates()


def algorithmic_bytes(t: dict, emissive: int, paths: int) -> dict:
    """Bytes the work must read or write at least once (roofline numerator), per kernel class:
    every traversal 32 (root) + 64 per interior node (both children) + 36 per
    triangle test; every hit 112 attribute + 224 material + 36 hit triangle;
    every triangle-light sample 16 * (2 + ceil(log2 E)) alias entries; every
    sky sample 2 * 12; every escaped ray 64 (bilinear sky); every path 48
    (accumulation read + write, storage texture write)."""
    alias = 16 * (2 + math.ceil(math.log2(max(emissive, 1))))
    extend = (32 * t["extend_rays"] + 64 * (t["interior_visits"] - t["shadow_interior_visits"])
              + 36 * (t["triangle_tests"] - t["shadow_triangle_tests"]))
    shadow = 32 * t["shadow_rays"] + 64 * t["shadow_interior_visits"] + 36 * t["shadow_triangle_tests"]
    shade = 372 * t["hits"] + alias * t["light_samples"] + 24 * t["sky_light_samples"] + 64 * t["sky_misses"]
    accumulate = 48 * paths
    total = extend + shadow + shade + accumulate
    return {"extend": extend, "shadow": shadow, "shade": shade, "accumulate": accumulate, "raygen": 0, "sort": 0,
            "plain": total, "total": total}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [line.split(",") for line in Path(self.file.name).read_text().splitlines() if line.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        os.unlink(self.file.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def latency_report(updates, precision: int, rate: float = 20.0, seconds: float = 3.0) -> dict:
    """p50/p99/p999 request latency (arrival -> result ready) of 512x512, 16-spp, max_bounces-8
    requests on this scene arriving as a seeded Poisson stream: through the batched engine
    (continuous batching, the requested precision form) and through the plain path (one
    request at a time, one pt_trace call of 16 samples, the plain kernel, the host waiting; its
    queueing is replayed from the measured service times)."""
    import pathtracer as pt
    from pathtracer import abi
    from pathtracer.engine import Engine
    from pathtracer.serving import percentiles, request_stream
    size, spp, depth = 512, 16, 8
    reqs = request_stream(rate, seconds, ["bench"], seed=3, progressive_fraction=0.0, fixed=(size, size, spp, depth))
    cam = abi.Camera.from_buffer_copy(updates.camera.contents)
    eng = Engine(precision=precision)
    sid = eng.add_scene(updates)
    warm = eng.submit(sid, cam, size, size, spp, depth)  # graph capture, layouts
    eng.wait_idle(timeout_ms=0)
    eng.poll(timeout_ms=0)
    eng.release(warm)
    lat, arrival_of, i = [], {}, 0
    t0 = time.perf_counter()
    while i < len(reqs) or arrival_of:
        now = time.perf_counter() - t0
        while i < len(reqs) and reqs[i].arrival <= now:
            arrival_of[eng.submit(sid, cam, size, size, spp, depth)] = reqs[i].arrival
            i += 1
        for jid in eng.poll(timeout_ms=1):
            if jid in arrival_of:  # (the warm-up job is reported here too)
                lat.append((time.perf_counter() - t0 - arrival_of.pop(jid)) * 1e3)
                eng.release(jid)
    eng.close()
    tr = pt.PathTracer(updates, (size, size))
    tr.set_kernel(abi.PT_KERNEL_PLAIN)
    tr.set_max_bounces(depth)
    tr.set_tile((size, size), (0, 0), (size, size))
    tr.trace(spp)
    tr.synchronize()
    free_at, plat = 0.0, []
    for r in reqs:
        u = abi.WorldUpdates()
        u.camera = C.pointer(cam)
        u.reset_accumulation = 1
        s0 = time.perf_counter()
        tr.apply_updates(u)
        tr.set_tile((size, size), (0, 0), (size, size))
        tr.trace(spp)
        tr.synchronize()
        service = time.perf_counter() - s0
        start = max(r.arrival, free_at)
        free_at = start + service
        plat.append((free_at - r.arrival) * 1e3)
    tr.close()
    return {"workload": f"{size}x{size}, {spp} spp, max_bounces {depth}, Poisson {rate:g} req/s for {seconds:g} s "
                        f"on this scene (seed 3)",
            "engine_ms": percentiles(lat), "plain_ms": percentiles(plat)}


MIX_SCENES = ["10k", "100k", "1M", "4M"]


def mixed_stream_report(seconds: float = 10.0, rate: float = 50.0, jobs: int = 256) -> dict:
    """The batching and serving workloads on one GPU, against the plain one-job-per-launch path.

    Scenes: procedural, about 10k / 100k / 1M / 4M triangles (pathtracer/serving.py SCENE_SIZES).
    * batching: `jobs` requests of the mix (sides log-uniform 64-1024, aspect 1:1-16:9, spp in
      {1,4,16,64}, max_bounces 4-12, random camera poses) rendered back to back: samples/s through
      the plain kernel (one pt_trace of <= 16 samples per call, the host waiting on each call:
      the reference's dispatch shape, FP32), the wavefront kernels one job per call (FP32), and the
      batched engine in the form and with the settings its autotuner run chose
      (pathtracer/engine_tuned.json: FP16 attributes / BF16 skybox + Kahan sums on the binary BVH),
      and the batched engine in the full compressed-node form (the same settings with the 8-wide
      BVH of 8-bit outward-rounded child boxes as well).
    * serving: Poisson arrivals at `rate` req/s for `seconds` s, 10 % progressive refinements, a
      fifth of the requests 512x512 x 16 spp x max_bounces 8; latency from arrival to result
      through the serving loop (continuous batching), overall and for the 512x512x16 requests
      inside the mix, on a second engine with the same settings but 4M-path waves
      (Engine.SERVING_WAVE_PATHS: the latency setting); the plain path's latencies for the same
      stream are replayed from its measured per-request service times."""
    from pathtracer import abi
    from pathtracer.engine import Engine
    from pathtracer.serving import (Server, build_scene, closed_loop, percentiles, replay_latencies,
                                    request_stream)
    t0 = time.perf_counter()
    worlds = {n: build_scene(n) for n in MIX_SCENES}
    build_s = time.perf_counter() - t0
    eng = Engine.tuned(hbm_budget_bytes=100 << 30)
    server = Server(eng, worlds)
    serve_eng = Engine.tuned(hbm_budget_bytes=100 << 30, wave_paths=Engine.SERVING_WAVE_PATHS)
    serve_server = Server(serve_eng, worlds, full=server.full)
    comp_eng = Engine.tuned(hbm_budget_bytes=100 << 30, precision=abi.PT_PRECISION_COMPRESSED)
    comp_server = Server(comp_eng, worlds, full=server.full)
    reqs = request_stream(1000.0, jobs / 1000.0 * 2.0 + 1.0, MIX_SCENES, seed=4, progressive_fraction=0.0)[:jobs]
    for e, s in ((eng, server), (serve_eng, serve_server), (comp_eng, comp_server)):
        warm = [e.submit(s.scene_ids[r.scene], s.camera(r.scene, r), r.width, r.height, r.samples,
                         r.max_bounces) for r in reqs[:8]]  # graph capture, layouts
        e.wait_idle(timeout_ms=0)
        e.poll(timeout_ms=0)  # take the warm-up jobs' completion reports
        for j in warm:
            e.release(j)
    batch = {mode: closed_loop(server, reqs, mode) for mode in ("engine", "wavefront", "plain")}
    batch["engine_compressed"] = closed_loop(comp_server, reqs, "engine")
    comp_eng.close()
    samples = batch["plain"]["samples"]
    stream = request_stream(rate, seconds, MIX_SCENES, seed=5, progressive_fraction=0.1, fixed=(512, 512, 16, 8),
                            fixed_share=0.2)
    g0 = serve_eng.stats()["gpu_ms"]
    res = serve_server.run(stream)
    busy = (serve_eng.stats()["gpu_ms"] - g0) / 1e3 / res.wall_s
    serve_eng.close()
    # the plain path on the same stream (refinements as fresh renders of their samples)
    plain_all = closed_loop(server, stream, "plain")
    plain_lat = replay_latencies(stream, plain_all["service_s"])
    plain_fixed = [lat for r, lat in zip(stream, plain_lat) if (r.width, r.height, r.samples) == (512, 512, 16)]
    eng.close()
    rate_of = {m: batch[m]["samples_per_s"] for m in batch}
    return {
        "workload": f"{jobs} jobs of the mix on procedural scenes of "
                    f"{', '.join(str(w.triangle_count()) for w in worlds.values())} triangles "
                    f"({samples} samples); serving: Poisson {rate:g} req/s for {seconds:g} s, 10% progressive, "
                    f"20% 512x512x16 spp depth 8",
        "engine": eng_config_of(Engine.tuned_config()),
        "serving_engine": eng_config_of(dict(Engine.tuned_config(), wave_paths=Engine.SERVING_WAVE_PATHS)),
        "compressed_engine": eng_config_of(dict(Engine.tuned_config(), precision=abi.PT_PRECISION_COMPRESSED)),
        "batching_samples_per_s": rate_of,
        "engine_over_plain": rate_of["engine"] / rate_of["plain"],
        "engine_compressed_over_plain": rate_of["engine_compressed"] / rate_of["plain"],
        "wavefront_over_plain": rate_of["wavefront"] / rate_of["plain"],
        "serving": {"requests": len(stream), "completed": res.completed, "rejected": res.rejected,
                    "latency_ms": percentiles(res.latencies_ms),
                    "latency_512x512x16_ms": percentiles(res.latencies_512_16_ms),
                    "samples_per_s": res.paths / res.wall_s, "gpu_busy": busy,
                    "plain_latency_ms": percentiles(plain_lat),
                    "plain_latency_512x512x16_ms": percentiles(plain_fixed)},
        "scene_build_s": build_s,
    }


def eng_config_of(cfg: dict) -> dict:
    keep = ("wave_paths", "tile_size", "steps_per_refill", "sort_min_hits", "traversal_threads", "shade_threads",
            "precision")
    return {k: cfg[k] for k in keep if k in cfg}


def pinned_updates(updates):
    """A full WorldUpdates whose buffers live in pinned host memory (for the end-to-end timing)."""
    import torch

    from pathtracer import abi
    keep = []

    def pin(ptr, nbytes):
        t = torch.empty(max(nbytes, 1), dtype=torch.uint8, pin_memory=True)
        if nbytes:
            C.memmove(t.data_ptr(), ptr, nbytes)
        keep.append(t)
        return t.data_ptr(), nbytes

    s = updates.scene.contents
    k = updates.skybox.contents
    scene = abi.SceneUpload.from_buffer_copy(s)
    h2d = 0
    for field, ctype, count in (("geometries", abi.TriangleGeometry, s.triangle_count),
                                ("attributes", abi.TriangleAttribute, s.triangle_count),
                                ("materials", abi.Material, s.material_count),
                                ("bvh_nodes", abi.BvhNode, s.node_count)):
        p, n = pin(getattr(s, field), C.sizeof(ctype) * count)
        setattr(scene, field, C.cast(p, C.POINTER(ctype)))
        h2d += n
    sky = abi.SkyboxUpload.from_buffer_copy(k)
    p, n = pin(k.rgba, 16 * k.uniforms.width * k.uniforms.height)
    sky.rgba = C.cast(p, C.POINTER(C.c_float))
    h2d += n
    if k.alias_count:
        p, n = pin(k.alias_table, 12 * k.alias_count)
        sky.alias_table = C.cast(p, C.POINTER(abi.SkyboxAliasEntry))
        h2d += n
    u = abi.WorldUpdates.from_buffer_copy(updates)
    u.scene = C.pointer(scene)
    u.skybox = C.pointer(sky)
    h2d += 16 * updates.scene_alias_count + 64 + 16 + 16
    keep.extend([scene, sky])
    return u, keep, h2d


def oracle_sample(world, seconds: float, threads: int = 0):
    """Time the oracle's FP32 restatement on a strided pixel subset of the same workload,
    sized to take about `seconds`; returns (Mrays/s, threads, description).  `world` is a full
    WorldUpdates or an oracle.OracleWorld."""
    import oracle
    ow = world if isinstance(world, oracle.OracleWorld) else oracle.world_from_updates(world)
    threads = threads or oracle.max_threads()

    def run(stride_px: int, spp: int):
        ys, xs = np.mgrid[0:HEIGHT:stride_px, 0:WIDTH:stride_px]
        px = np.stack([xs.ravel(), ys.ravel()], axis=1).astype(np.uint32)
        t0 = time.perf_counter()
        _, rec = oracle.trace_paths(ow, (WIDTH, HEIGHT), MAX_BOUNCES, px, 1, spp, threads=threads, records=True)
        dt = time.perf_counter() - t0
        rays = int(rec["extend_rays"].sum() + rec["shadow_rays"].sum())
        return rays, dt, px.shape[0]

    rays, dt, n_cal = run(max(1, int(math.sqrt(WIDTH * HEIGHT / 4096))), 4)  # calibration on ~4096 pixels
    rate = rays / max(dt, 1e-6)
    want_rays = rate * seconds
    rays_per_px = rays / max(1, n_cal * 4) * SPP
    n_px = max(64, int(want_rays / max(rays_per_px, 1.0)))
    stride = max(1, math.ceil(math.sqrt(WIDTH * HEIGHT / n_px)))  # never above the time budget
    rays, dt, npx = run(stride, SPP)
    desc = f"every {stride}th pixel in x and y ({npx} pixels) x {SPP} spp of the {WIDTH}x{HEIGHT} image, {threads} threads"
    return rays / dt / 1e6, threads, desc, dt


# the buffers of a full world upload, in the order dump_world writes them
UPLOAD_PARTS = ("geometries", "attributes", "materials", "bvh_nodes", "srgb", "linear", "sky", "sky_alias",
                "scene_alias", "camera", "scene_uniforms", "skybox_uniforms")


def dump_world(path: str) -> None:
    """Build the workload's world with the library and write its full upload to `path` (.npz).
    Runs in a child process of the reference arm, so that process never maps the library."""
    world, u = build_world()
    s, k = u.scene.contents, u.skybox.contents

    def raw(ptr, n):
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(n,)).copy() if n else np.zeros(0, np.uint8)

    layer = 8192 * 8192 * 4
    parts = {
        "geometries": raw(s.geometries, 36 * s.triangle_count),
        "attributes": raw(s.attributes, 112 * s.triangle_count),
        "materials": raw(s.materials, 224 * s.material_count),
        "bvh_nodes": raw(s.bvh_nodes, 32 * s.node_count),
        "srgb": raw(s.srgb_texture_atlases, layer * s.srgb_atlas_count),
        "linear": raw(s.linear_texture_atlases, layer * s.linear_atlas_count),
        "sky": raw(k.rgba, 16 * k.uniforms.width * k.uniforms.height),
        "sky_alias": raw(k.alias_table, 12 * k.alias_count),
        "scene_alias": raw(u.scene_alias_table, 16 * u.scene_alias_count),
        "camera": np.frombuffer(bytes(u.camera.contents), np.uint8).copy(),
        "scene_uniforms": np.frombuffer(bytes(u.scene_uniforms.contents), np.uint8).copy(),
        "skybox_uniforms": np.frombuffer(bytes(u.skybox_uniforms.contents), np.uint8).copy(),
        "counts": np.array([s.triangle_count, s.material_count, s.node_count, s.srgb_atlas_count,
                            s.linear_atlas_count, k.alias_count, u.scene_alias_count], np.uint64),
    }
    np.savez(path, **parts)


def oracle_world_from_dump(path: str):
    """(OracleWorld, arrays it points into, counts) from a dump_world file; no library involved."""
    import oracle
    from pathtracer import abi
    d = np.load(path)
    keep = {name: np.ascontiguousarray(d[name]) for name in UPLOAD_PARTS}
    tri, mats, nodes, srgb, linear, sky_alias, scene_alias = (int(x) for x in d["counts"])
    w = oracle.OracleWorld()
    w.geometries, w.attributes, w.triangle_count = keep["geometries"].ctypes.data, keep["attributes"].ctypes.data, tri
    w.materials, w.material_count = keep["materials"].ctypes.data, mats
    w.bvh_nodes, w.node_count = keep["bvh_nodes"].ctypes.data, nodes
    w.srgb_atlases, w.srgb_atlas_count = (keep["srgb"].ctypes.data if srgb else None), srgb
    w.linear_atlases, w.linear_atlas_count = (keep["linear"].ctypes.data if linear else None), linear
    w.camera = abi.Camera.from_buffer_copy(keep["camera"].tobytes())
    w.skybox_rgba = keep["sky"].ctypes.data
    w.skybox = abi.SkyboxUniforms.from_buffer_copy(keep["skybox_uniforms"].tobytes())
    w.skybox_aliases, w.skybox_alias_count = (keep["sky_alias"].ctypes.data if sky_alias else None), sky_alias
    w.scene = abi.SceneUniforms.from_buffer_copy(keep["scene_uniforms"].tobytes())
    w.scene_aliases, w.scene_alias_count = (keep["scene_alias"].ctypes.data if scene_alias else None), scene_alias
    return w, keep, {"triangles": tri, "bvh_nodes": nodes}


def gpu_library_mapped() -> bool:
    """Whether this process has the GPU library (libpt.so) mapped."""
    try:
        return "libpt.so" in Path("/proc/self/maps").read_text()
    except OSError:
        return False


class _Counts:
    """triangle_count() / node_count() of a dumped world, for workload_config."""

    def __init__(self, counts):
        self.c = counts

    def triangle_count(self):
        return self.c["triangles"]

    def node_count(self):
        return self.c["bvh_nodes"]


def run_reference(args):
    rank, _, world_size = dist_env()
    if rank != 0:
        return
    # the scene is built in a child process and handed over as its upload bytes: this process loads
    # only the oracle (the reference's CPU restatement), never the GPU library
    with tempfile.TemporaryDirectory() as tmp:
        path = str(Path(tmp) / "world.npz")
        cmd = [sys.executable, str(Path(__file__).resolve()), "--dump-world", path, "--workload", WORKLOAD,
               "--image", str(WIDTH), str(HEIGHT)]
        subprocess.run(cmd, check=True)
        ow, keep, counts = oracle_world_from_dump(path)
    world = _Counts(counts)
    import oracle
    threads = oracle.max_threads()
    per_step = max(2.0, min(args.cpu_seconds, 20.0))
    values = []
    for i in range(args.warmup + args.steps):
        v, threads, desc, dt = oracle_sample(ow, per_step if i >= args.warmup else 1.0)
        if i >= args.warmup:
            values.append((v, dt))
    value = float(np.mean([v for v, _ in values]))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean([d for _, d in values]) * 1e3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (scene built from a seed)",
        "config": workload_config(world, "fp32", args.gpus), "kernel": "cpu",
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's own trace pass (Rust + WGSL via wgpu) cannot run on this box; this is the "
                "oracle's C++ restatement of src/render/trace.slang, OpenMP over paths; the scene is built in a "
                "child process and passed as its upload bytes",
        "maps_gpu_library": gpu_library_mapped(),
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import pathtracer as pt
    from pathtracer import abi

    rank, local_rank, world_size = dist_env()
    torch.cuda.set_device(local_rank)
    pg = None
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist

    world, updates = build_world()
    emissive = updates.scene_uniforms.contents.emissive_triangles_count
    tracer = pt.PathTracer(updates, (WIDTH, HEIGHT), device=local_rank)
    tracer.set_kernel(KERNEL_NAMES[args.kernel])
    tracer.set_precision(PRECISIONS[args.precision])
    tracer.set_max_bounces(MAX_BOUNCES)

    spp = args.spp

    def step():
        tracer.set_tile((WIDTH, HEIGHT), (0, 0), (WIDTH, HEIGHT))
        remaining = spp
        while remaining > 0:
            remaining -= tracer.trace(remaining)

    if args.profile_run:
        for _ in range(args.steps):
            step()
        tracer.synchronize()
        tracer.close()
        print(json.dumps({"profile_run": True, "kernel": args.kernel, "spp": spp, "steps": args.steps}))
        return

    # counting pass over the identical (deterministic) workload
    tracer.set_tile((WIDTH, HEIGHT), (0, 0), (WIDTH, HEIGHT))
    totals, remaining = None, spp
    while remaining > 0:
        n, totals = tracer.trace_counted(remaining, totals)
        remaining -= n
    rays_per_step = totals["extend_rays"] + totals["shadow_rays"]
    paths_per_step = WIDTH * HEIGHT * spp
    bytes_per_step = algorithmic_bytes(totals, emissive, paths_per_step)

    for _ in range(max(args.warmup, 0)):
        step()
    tracer.synchronize()

    stream = torch.cuda.ExternalStream(tracer.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    tracer.synchronize()
    launches0 = tracer.launch_count()
    with ClockSampler(local_rank) as clocks:
        start.record(stream)
        for _ in range(args.steps):
            step()
        stop.record(stream)
        tracer.synchronize()
        torch.cuda.synchronize()
    elapsed_ms = start.elapsed_time(stop)
    launches = tracer.launch_count() - launches0
    # per-kernel times from a separate instrumented pass: with profiling on, the
    # library runs the stages one after another (no overlap of consecutive groups
    # or of a bounce's shadow stage), so each launch's CUDA-event time is its own
    prof_steps = min(args.steps, 3)
    tracer.reset_kernel_times()
    tracer.set_profiling(True)
    for _ in range(prof_steps):
        step()
    tracer.synchronize()
    times = tracer.kernel_times()
    tracer.set_profiling(False)
    for k in times.launches:  # per image
        times.launches[k] = times.launches[k] * args.steps // prof_steps
        times.milliseconds[k] = times.milliseconds[k] * args.steps / prof_steps
    elapsed_ms = max_over_ranks(elapsed_ms, pg, "cuda")
    if pg:
        pg.barrier()
    value = job_rate(rays_per_step, args.steps, world_size, elapsed_ms / 1e3) / 1e6

    # dominant kernel and its roofline
    cls = max(times.milliseconds, key=lambda k: times.milliseconds[k])
    cls_launches = max(1, times.launches[cls])
    avg_launch_s = times.milliseconds[cls] / cls_launches / 1e3
    launches_per_step = cls_launches / args.steps
    bytes_per_launch = bytes_per_step[cls] / launches_per_step
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = bytes_per_launch / avg_launch_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": TRAFFIC_PER_LAUNCH.get((args.kernel, cls, args.precision))
                if WORKLOAD == "procedural" and WIDTH * HEIGHT * spp == 1920 * 1080 * 64 else None, "kernel": cls,
                "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_s * 1e3,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs), of measured" if peaks else "fallback 6.8 TB/s",
                "launch_timing": f"CUDA events around each launch on its stream, {prof_steps} instrumented steps "
                                 "after the timed ones, stages serialised (no overlap between groups)"}

    # image error of the step's image (its accumulation holds samples 1..spp)
    # against the FP64 reference render of the same paths on the GPU
    rmse = None
    if rank == 0 and not args.no_fp64:
        acc = tracer.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64) / spp
        t64 = time.perf_counter()
        ref = tracer.render_fp64(1, spp) / spp
        rmse = {"value": float(np.sqrt(np.mean((acc - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))),
                "definition": "sqrt(mean((img - fp64)^2)) / sqrt(mean(fp64^2)) over the whole image, per-pixel means",
                "image": [WIDTH, HEIGHT], "spp": spp, "precision": args.precision,
                "fp64_render_s": time.perf_counter() - t64}

    # issue-slot bound of the traversal and shading kernels: warp instructions per launch over the
    # issue slots of its duration at the sampled SM clock
    issue = None
    inst = WARP_INST_PER_PATH.get((args.kernel, args.precision))
    clock_summary = clocks.summary()
    if inst and WORKLOAD == "procedural" and WIDTH * HEIGHT == 1920 * 1080 and clock_summary.get("sm_mhz"):
        paths_per_launch = WIDTH * HEIGHT * min(spp, abi.PT_MAX_SAMPLES_PER_TRACE)
        hz = clock_summary["sm_mhz"] * 1e6
        issue = {"unit": "fraction of issue slots", "sm_mhz": clock_summary["sm_mhz"], "kernels": {}}
        for k, per_path in inst.items():
            n = max(1, times.launches[k])
            avg_s = times.milliseconds[k] / n / 1e3
            issue["kernels"][k] = {"warp_inst_per_launch": per_path * paths_per_launch, "avg_launch_ms": avg_s * 1e3,
                                   "frac": per_path * paths_per_launch / (SMS * SCHEDULERS_PER_SM * hz * avg_s)}

    # end to end through the C ABI: world upload from pinned host memory, the
    # render, and the RGBA8 result read back, every step
    pinned, keep, h2d = pinned_updates(updates)
    tracer.apply_updates(pinned)
    step()
    tracer.display_tile()
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, args.e2e_steps)
    for _ in range(e2e_steps):
        tracer.apply_updates(pinned)
        step()
        tracer.display_tile()
    e2e_s = max_over_ranks(time.perf_counter() - t0, pg, "cuda")
    e2e_value = job_rate(rays_per_step, e2e_steps, world_size, e2e_s) / 1e6

    latency = None
    if rank == 0 and world_size == 1 and not args.no_latency:
        latency = latency_report(updates, PRECISIONS[args.precision])

    mix = None
    if rank == 0 and world_size == 1 and not args.no_mix and WORKLOAD == "procedural":
        mix = mixed_stream_report(seconds=args.mix_seconds)

    cpu = None
    if rank == 0 and world_size == 1 and not args.no_cpu_baseline:
        v, threads, desc, _ = oracle_sample(updates, args.cpu_seconds)
        cpu = {"value": v, "unit": METRIC, "cores": threads, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (scene built from a seed)",
            "config": workload_config(world, args.precision, world_size), "kernel": args.kernel,
            "rays_per_step": rays_per_step, "samples_per_s": job_rate(paths_per_step, args.steps, world_size,
                                                                     elapsed_ms / 1e3),
            # whole-pass algorithmic bytes per ray and the Mrays/s they would allow at the HBM peak
            "bytes_per_ray": bytes_per_step["total"] / rays_per_step,
            "hbm_roofline_mrays": peak * 1e9 / (bytes_per_step["total"] / rays_per_step) / 1e6,
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": WIDTH * HEIGHT * 4},
            "issue_bound": issue,
            "gpu_launches": launches, "clocks": clock_summary, "latency": latency,
            "rmse_vs_fp64": rmse, "mixed_stream": mix,
            "kernel_ms": {k: v for k, v in times.milliseconds.items() if times.launches[k]},
        }
        print(json.dumps(line), flush=True)
    tracer.close()
    del keep
    if pg:
        pg.destroy_process_group()


def main():
    args = parse_args()
    if args.dump_world:
        dump_world(args.dump_world)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
