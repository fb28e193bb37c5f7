"""Serving loop over the batched engine: requests arrive as a Poisson stream,
are admitted into the engine as they arrive (continuous batching: they join
the next wave while earlier requests are still on the GPU), and the latency
from arrival to completion is recorded per request.

Request mix (the batching / serving workloads): image side log-uniform in
[64, 1024] with aspect 1:1 to 16:9, samples in {1, 4, 16, 64}, max_bounces in
[4, 12], scene drawn from procedural scenes of about 10k, 100k, 1M (and
optionally 4M) triangles with random camera poses; a fraction of requests
are progressive refinements that add samples to the resident accumulation of
an earlier request.  Requests the engine refuses (HBM budget) are counted as
rejected.

    python -m pathtracer.serving --rate 50 --duration 10
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np

import pathtracer as pt
from pathtracer import abi
from pathtracer.engine import Engine

# procedural scene parameters for about 10k, 100k, 1M and 4M triangles
SCENE_SIZES = {
    "10k": dict(grid_x=48, grid_z=48, boxes=200, spheres=2, sphere_subdivision=3, emissive_triangles=16),
    "100k": dict(grid_x=160, grid_z=160, boxes=1000, spheres=30, sphere_subdivision=3, emissive_triangles=32),
    "1M": dict(grid_x=512, grid_z=512, boxes=2000, spheres=90, sphere_subdivision=4, emissive_triangles=64),
    "4M": dict(grid_x=1024, grid_z=1024, boxes=4000, spheres=360, sphere_subdivision=4, emissive_triangles=64),
}


def build_scene(size: str, seed: int = 7) -> pt.World:
    return pt.World.procedural(seed=seed, skybox_width=512, skybox_height=256, **SCENE_SIZES[size])


@dataclass
class Request:
    arrival: float
    scene: str
    width: int
    height: int
    samples: int
    max_bounces: int
    yaw: float
    pitch: float
    progressive: bool = False


@dataclass
class ServeResult:
    latencies_ms: list = field(default_factory=list)
    latencies_512_16_ms: list = field(default_factory=list)
    completed: int = 0
    rejected: int = 0
    paths: int = 0
    wall_s: float = 0.0


def request_stream(rate: float, duration: float, scenes: list[str], seed: int = 1,
                   progressive_fraction: float = 0.1, fixed: tuple | None = None,
                   fixed_share: float = 1.0) -> list[Request]:
    """Poisson arrivals of the request mix; with `fixed` = (W, H, SPP, DEPTH), that share of the requests
    (all by default) takes this shape instead and is never a progressive refinement."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        side = math.exp(rng.uniform(math.log(64), math.log(1024)))
        aspect = rng.uniform(1.0, 16.0 / 9.0)
        w, h = max(8, int(side * math.sqrt(aspect))), max(8, int(side / math.sqrt(aspect)))
        spp = int(rng.choice([1, 4, 16, 64]))
        depth = int(rng.integers(4, 13))
        progressive = bool(rng.random() < progressive_fraction)
        if fixed is not None and (fixed_share >= 1.0 or rng.random() < fixed_share):
            w, h, spp, depth = fixed
            progressive = False
        out.append(Request(t, scenes[int(rng.integers(len(scenes)))], w, h, spp, depth,
                           float(rng.uniform(-0.6, 0.6)), float(rng.uniform(-0.5, -0.2)), progressive=progressive))


class Server:
    """Admission + continuous batching on one engine; scenes cached by content hash."""

    def __init__(self, engine: Engine, worlds: dict[str, pt.World], full: dict | None = None):
        """full: the worlds' full updates, when another server took them already (they stay valid
        only until the next take_updates of a world, i.e. until the first camera() call)."""
        self.engine = engine
        self.worlds = worlds
        self.full = full if full is not None else {name: w.take_updates() for name, w in worlds.items()}
        self.scene_ids = {name: engine.add_scene(u) for name, u in self.full.items()}
        self._last = {name: abi.Camera.from_buffer_copy(u.camera.contents) for name, u in self.full.items()}

    def camera(self, name: str, req: Request) -> abi.Camera:
        w = self.worlds[name]
        w.set_aspect_ratio(req.width / req.height)
        w.edit_camera(yaw=req.yaw, pitch=req.pitch)
        u = w.take_updates()
        if u.camera:
            self._last[name] = abi.Camera.from_buffer_copy(u.camera.contents)
        return abi.Camera.from_buffer_copy(self._last[name])

    def run(self, requests: list[Request], max_outstanding_paths: int = 2_000_000_000,
            keep_finished: int = 256, on_done=None) -> ServeResult:
        """Serve the stream.  The `keep_finished` most recently finished jobs stay resident (their
        accumulations can be refined by later progressive requests, which keep the refined job's
        camera); older ones are released.  on_done(job_id, request, camera, total_samples), if
        given, is called when a job finishes, while its result is still resident."""
        eng, res = self.engine, ServeResult()
        arrival_of, is_512_16, paths_of = {}, {}, {}
        camera_of, samples_of = {}, {}  # resident jobs: camera and samples in the accumulation
        finished: dict[tuple, list[int]] = {}  # (scene, w, h, depth) -> finished job ids to refine
        kept: OrderedDict[int, tuple] = OrderedDict()  # the same jobs, oldest first
        outstanding, i = 0, 0
        t0 = time.perf_counter()
        while i < len(requests) or arrival_of:
            now = time.perf_counter() - t0
            while i < len(requests) and requests[i].arrival <= now:
                r = requests[i]
                i += 1
                key = (r.scene, r.width, r.height, r.max_bounces)
                cont = 0
                if r.progressive and finished.get(key):
                    cont = finished[key].pop()
                    del kept[cont]
                paths = r.width * r.height * r.samples
                if outstanding + paths > max_outstanding_paths:
                    res.rejected += 1
                    continue
                cam = camera_of[cont] if cont else self.camera(r.scene, r)
                try:
                    jid = eng.submit(self.scene_ids[r.scene], cam, r.width, r.height, r.samples,
                                     r.max_bounces, continue_job=cont)
                except pt.PathTracerError:
                    res.rejected += 1
                    continue
                camera_of[jid] = cam
                samples_of[jid] = r.samples + (samples_of[cont] if cont else 0)
                arrival_of[jid] = (r.arrival, key, cont, r)
                is_512_16[jid] = (r.width, r.height, r.samples) == (512, 512, 16)
                paths_of[jid] = paths
                outstanding += paths
            for jid in eng.poll(timeout_ms=1):
                if jid not in arrival_of:  # a job submitted outside this stream (e.g. a warm-up)
                    continue
                done_at = time.perf_counter() - t0
                arrival, key, cont, req = arrival_of.pop(jid)
                if on_done is not None:
                    on_done(jid, req, camera_of[jid], samples_of[jid])
                lat = (done_at - arrival) * 1e3
                res.latencies_ms.append(lat)
                if is_512_16.pop(jid):
                    res.latencies_512_16_ms.append(lat)
                res.completed += 1
                p = paths_of.pop(jid)
                res.paths += p
                outstanding -= p
                if cont:
                    eng.release(cont)
                    camera_of.pop(cont, None)
                    samples_of.pop(cont, None)
                finished.setdefault(key, []).append(jid)
                kept[jid] = key
                while len(kept) > keep_finished:
                    old_jid, old_key = kept.popitem(last=False)
                    finished[old_key].remove(old_jid)
                    eng.release(old_jid)
                    camera_of.pop(old_jid, None)
                    samples_of.pop(old_jid, None)
        res.wall_s = time.perf_counter() - t0
        for ids in finished.values():
            for jid in ids:
                eng.release(jid)
        return res


def closed_loop(server: Server, requests: list[Request], mode: str) -> dict:
    """Render every request back to back (arrival times ignored) and return samples per second.

    mode "plain": one job at a time through pt_trace with the plain kernel
    (one thread per pixel, one launch per sample, at most 16 samples per call,
    the host waiting for each call) - the reference's dispatch organisation;
    "wavefront": one job at a time through pt_trace with the wavefront kernels;
    "engine": all jobs submitted to the batched engine at once.
    One PathTracer per scene is reused across requests (camera update + set_tile)."""
    total = sum(r.width * r.height * r.samples for r in requests)
    if mode == "engine":
        eng = server.engine
        t0 = time.perf_counter()
        ids = [eng.submit(server.scene_ids[r.scene], server.camera(r.scene, r), r.width, r.height, r.samples,
                          r.max_bounces) for r in requests]
        eng.wait_idle(timeout_ms=0)
        dt = time.perf_counter() - t0
        for j in ids:
            eng.release(j)
        return {"mode": mode, "samples": total, "seconds": dt, "samples_per_s": total / dt}
    kernel = abi.PT_KERNEL_PLAIN if mode == "plain" else abi.PT_KERNEL_WAVEFRONT
    tracers = {}
    for name, full in server.full.items():
        tracers[name] = pt.PathTracer(full, (64, 64))
        tracers[name].set_kernel(kernel)
    service = []
    t0 = time.perf_counter()
    for r in requests:
        s0 = time.perf_counter()
        tr = tracers[r.scene]
        cam = server.camera(r.scene, r)
        u = abi.WorldUpdates()
        u.camera = C.pointer(cam)
        u.reset_accumulation = 1
        tr.apply_updates(u)
        tr.set_max_bounces(r.max_bounces)
        tr.set_tile((r.width, r.height), (0, 0), (r.width, r.height))
        left = r.samples
        while left > 0:
            left -= tr.trace(left)
            tr.synchronize()
        service.append(time.perf_counter() - s0)
    dt = time.perf_counter() - t0
    for tr in tracers.values():
        tr.close()
    return {"mode": mode, "samples": total, "seconds": dt, "samples_per_s": total / dt, "service_s": service}


def replay_latencies(requests: list[Request], service_s: list[float]) -> list[float]:
    """Arrival-to-completion latency (ms) of each request on a server that handles one request at a time,
    in arrival order, each taking its measured service time."""
    free_at, out = 0.0, []
    for r, s in zip(requests, service_s):
        start = max(r.arrival, free_at)
        free_at = start + s
        out.append((free_at - r.arrival) * 1e3)
    return out


def percentiles(xs: list) -> dict:
    if not xs:
        return {"p50": None, "p99": None, "p999": None, "n": 0}
    a = np.asarray(xs)
    return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99)),
            "p999": float(np.percentile(a, 99.9)), "n": int(a.size)}


def main(argv=None) -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--rate", type=float, default=50.0, help="mean requests per second")
    p.add_argument("--duration", type=float, default=10.0, help="seconds of arrivals")
    p.add_argument("--scenes", default="10k,100k,1M")
    p.add_argument("--fixed", default="", help="W,H,SPP,DEPTH: every request this shape (e.g. 512,512,16,8)")
    p.add_argument("--fixed-share", type=float, default=1.0,
                   help="with --fixed: the share of the requests of that shape (the others follow the mix)")
    p.add_argument("--tuned", action="store_true",
                   help="the engine settings of pathtracer/engine_tuned.json (their precision form replaces "
                        "--precision)")
    p.add_argument("--wave-paths", type=int, default=0, help="paths per wave (0: the engine's or the tuned value)")
    p.add_argument("--warmup", type=int, default=8,
                   help="requests of another seed rendered before the stream (graph capture, buffer layouts)")
    p.add_argument("--progressive", type=float, default=0.1)
    p.add_argument("--budget-gb", type=float, default=150.0)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--precision", choices=["fp32", "wide", "half", "compressed"], default="fp32",
                   help="engine form: the reference's FP32 buffers, the 8-wide BVH, FP16 attributes / BF16 skybox "
                        "+ Kahan sums on the binary BVH, or the compressed form (all three)")
    p.add_argument("--autotune", action="store_true",
                   help="with --compare: let the engine's autotuner pick wave size, tile size, refill steps, the "
                        "hit-sort threshold and the kernels' block shapes on 16 of the requests first")
    p.add_argument("--save-tuned", action="store_true",
                   help="with --compare --autotune: store the chosen settings in pathtracer/engine_tuned.json")
    p.add_argument("--compare", type=int, default=0,
                   help="instead of serving: render this many requests of the mix back to back with the plain "
                        "kernel, the wavefront kernel (one job per call) and the batched engine")
    args = p.parse_args(argv)
    names = args.scenes.split(",")
    t = time.perf_counter()
    worlds = {n: build_scene(n) for n in names}
    build_s = time.perf_counter() - t
    forms = {"fp32": abi.PT_PRECISION_FP32, "wide": abi.PT_PRECISION_WIDE_BVH,
             "half": abi.PT_PRECISION_HALF_ATTRIBUTES | abi.PT_PRECISION_KAHAN,
             "compressed": abi.PT_PRECISION_COMPRESSED}
    precision = forms[args.precision]
    budget = int(args.budget_gb * (1 << 30))
    if args.tuned:
        over = {"wave_paths": args.wave_paths} if args.wave_paths else {}
        eng = Engine.tuned(hbm_budget_bytes=budget, **over)
        args.precision = {v: k for k, v in forms.items()}.get(Engine.tuned_config()["precision"], args.precision)
    else:
        eng = Engine(hbm_budget_bytes=budget, precision=precision, wave_paths=args.wave_paths)
    server = Server(eng, worlds)
    fixed = tuple(int(x) for x in args.fixed.split(",")) if args.fixed else None
    if args.compare:
        reqs = request_stream(1000.0, args.compare / 1000.0 * 2.0 + 1.0, names, args.seed, 0.0, fixed)[:args.compare]
        out = {"requests": len(reqs), "engine_precision": args.precision,
               "triangles": {n: worlds[n].triangle_count() for n in names}}
        if args.autotune:
            sample = [abi.JobDesc(server.scene_ids[r.scene], server.camera(r.scene, r), r.width, r.height, r.samples,
                                  r.max_bounces, 0) for r in reqs[:16]]
            t = time.perf_counter()
            out["autotuned"] = eng.autotune(sample)
            out["autotune_s"] = time.perf_counter() - t
            if args.save_tuned:
                from pathlib import Path
                cmd = ("python -m pathtracer.serving --compare " + str(args.compare) + " --scenes " + args.scenes +
                       " --precision " + args.precision + " --autotune --save-tuned")
                (Path(__file__).resolve().parent / "engine_tuned.json").write_text(json.dumps(
                    {"config": out["autotuned"], "command": cmd, "seed": args.seed}, indent=1) + "\n")
        for mode in ("engine", "wavefront", "plain"):
            out[mode] = {k: v for k, v in closed_loop(server, reqs, mode).items() if k != "service_s"}
        out["engine_over_plain"] = out["engine"]["samples_per_s"] / out["plain"]["samples_per_s"]
        out["wavefront_over_plain"] = out["wavefront"]["samples_per_s"] / out["plain"]["samples_per_s"]
        print(json.dumps(out))
        eng.close()
        return
    if args.warmup > 0:
        warm = request_stream(1000.0, args.warmup / 1000.0 * 2.0 + 1.0, names, args.seed + 1000, 0.0)[:args.warmup]
        ids = [eng.submit(server.scene_ids[r.scene], server.camera(r.scene, r), r.width, r.height, r.samples,
                          r.max_bounces) for r in warm]
        eng.wait_idle(timeout_ms=0)
        eng.poll(timeout_ms=0)
        for j in ids:
            eng.release(j)
    reqs = request_stream(args.rate, args.duration, names, args.seed, args.progressive, fixed,
                          fixed_share=args.fixed_share)
    res = server.run(reqs)
    st = eng.stats()
    print(json.dumps({
        "rate_req_s": args.rate, "duration_s": args.duration, "requests": len(reqs), "completed": res.completed,
        "rejected": res.rejected, "latency_ms": percentiles(res.latencies_ms),
        "latency_512x512x16_ms": percentiles(res.latencies_512_16_ms),
        "samples_per_s": res.paths / res.wall_s, "wall_s": res.wall_s, "gpu_ms": st["gpu_ms"],
        "waves": st["waves"], "scene_build_s": build_s, "engine_precision": args.precision,
        "wave_paths": st["wave_paths"],
        "triangles": {n: worlds[n].triangle_count() for n in names},
    }))
    eng.close()


if __name__ == "__main__":
    main()
