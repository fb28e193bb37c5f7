"""Measure the precision form on its workload: the Cornell room with
procedural 1024^2 textures on four of its eight meshes, 256x256, 1024 spp,
max_bounces 8.

For the FP32 form and the compressed form (8-wide quantised BVH, FP16
attributes / BF16 skybox, Kahan sums) it reports samples/s and Mrays/s
(CUDA events around the whole image), the relative RMSE of a crop against the
FP64 oracle render with the same RNG streams, and the hit-id agreement of the
wide traversal with the binary one on random rays.

    python -m pathtracer.precision_check [--spp 1024] [--crop 64]
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT)]

import pathtracer as pt  # noqa: E402
from pathtracer import abi  # noqa: E402

SIZE = 256


def render(updates, prec: int, spp: int, rays_per_sample: float | None = None):
    import torch
    tr = pt.PathTracer(updates, (SIZE, SIZE))
    tr.set_precision(prec)
    tr.set_max_bounces(8)
    tr.set_tile((SIZE, SIZE), (0, 0), (SIZE, SIZE))
    tr.trace(4)  # warm-up: builds the derived layouts
    tr.synchronize()
    tr.set_tile((SIZE, SIZE), (0, 0), (SIZE, SIZE))
    stream = torch.cuda.ExternalStream(tr.stream())
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    done = 0
    while done < spp:
        done += tr.trace(spp - done)
    stop.record(stream)
    stop.synchronize()
    ms = start.elapsed_time(stop)
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64) / spp
    tr.close()
    return acc, ms


def main(argv=None) -> None:
    import oracle
    p = argparse.ArgumentParser()
    p.add_argument("--spp", type=int, default=1024)
    p.add_argument("--crop", type=int, default=64, help="side of the centre crop compared with the FP64 oracle")
    p.add_argument("--seed", type=int, default=1)
    args = p.parse_args(argv)
    w = pt.World.cornell_box_textured(args.seed)
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    # rays per image from the counting variant (FP32 paths)
    tr = pt.PathTracer(u, (SIZE, SIZE))
    tr.set_max_bounces(8)
    tr.set_tile((SIZE, SIZE), (0, 0), (SIZE, SIZE))
    totals, left = None, 16
    while left > 0:
        n, totals = tr.trace_counted(left, totals)
        left -= n
    tr.close()
    rays_per_spp = (totals["extend_rays"] + totals["shadow_rays"]) / 16.0
    out = {"workload": f"textured Cornell room, {SIZE}x{SIZE}, {args.spp} spp, max_bounces 8",
           "triangles": w.triangle_count(), "rays_per_sample_pass": rays_per_spp}
    images = {}
    for name, prec in (("fp32", abi.PT_PRECISION_FP32), ("compressed", abi.PT_PRECISION_COMPRESSED)):
        img, ms = render(u, prec, args.spp)
        images[name] = img
        out[name] = {"ms": ms, "samples_per_s": SIZE * SIZE * args.spp / (ms / 1e3),
                     "mrays_per_s": rays_per_spp * args.spp / (ms / 1e3) / 1e6}
    # FP64 oracle on the centre crop
    c0 = (SIZE - args.crop) // 2
    xs, ys = np.meshgrid(np.arange(c0, c0 + args.crop), np.arange(c0, c0 + args.crop))
    px = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.uint32)
    t = time.perf_counter()
    rad64, _ = oracle.trace_paths(oracle.world_from_updates(u), (SIZE, SIZE), 8, px, 1, args.spp, precision=64)
    ref = rad64.mean(axis=0).reshape(args.crop, args.crop, 3)
    out["fp64_oracle_seconds"] = time.perf_counter() - t
    for name, img in images.items():
        crop = img[c0:c0 + args.crop, c0:c0 + args.crop]
        out[name]["rel_rmse_vs_fp64"] = float(np.sqrt(np.mean((crop - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))
    # hit ids: wide vs binary traversal on random rays through the room
    rng = np.random.default_rng(5)
    o = rng.uniform(0.02, 0.98, (200000, 3)).astype(np.float32)
    d = rng.normal(size=(200000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tr = pt.PathTracer(u, (8, 8))
    hit, t_bin, _ = tr.debug_intersect(o, d, records=False)
    tr.set_precision(abi.PT_PRECISION_WIDE_BVH)
    whit, t_wide, _ = tr.debug_intersect(o, d, records=False)
    tr.close()
    out["hit_ids"] = {"rays": int(hit.size), "differ": int(np.count_nonzero(whit != hit)),
                      "t_bits_differ": int(np.count_nonzero(t_wide.view(np.uint32) != t_bin.view(np.uint32)))}
    out["speedup_compressed_over_fp32"] = out["compressed"]["samples_per_s"] / out["fp32"]["samples_per_s"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
