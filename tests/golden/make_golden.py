"""Regenerate the golden fixtures of tests/golden/ (committed; run by hand).

The reference (Rust + Slang/WGSL) cannot run in this container and ships no
golden vectors for the trace path, so these fixtures come from the pure-Python
restatement in oracle/world_ref.py, which is written independently of the C++
builder and oracle they pin:
  rng.json          rand() bit sequences and compute_main seeds
  bvh.json          binned SAH BVHs (world.rs:1430-1591) of the Cornell box
                    triangles and of a seeded random triangle soup
  alias.json        Vose alias tables (world.rs:542-575)
Usage: python tests/golden/make_golden.py
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path[:0] = [str(ROOT), str(ROOT / "path-tracer_gb300")]

from oracle import world_ref  # noqa: E402

OUT = Path(__file__).resolve().parent


def random_soup(seed: int, n: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-10, 10, (n, 1, 3))
    offsets = rng.normal(0, 0.5, (n, 3, 3))
    return (centers + offsets).reshape(n, 9).astype(np.float32)


def cornell_triangles() -> np.ndarray:
    """The 36 triangles of the Cornell box in the order they are added (before the BVH reorder)."""
    import pathtracer as pt
    w = pt.World.cornell_box()
    g = w.geometries()
    order = w.bvh_order()
    out = np.empty_like(g)
    out[order] = g
    return out


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    rng = {"sequences": [], "seeds": []}
    for state in (1, 0xA511E9B3, 0xDEADBEEF, 0x7FFFFFFF):
        vals, _ = world_ref.pcg_rand(state, 64)
        rng["sequences"].append({"state": state, "bits": [int(b) for b in vals.view(np.uint32)]})
    for px, py, n in [(0, 0, 1), (17, 3, 2), (255, 255, 16), (1919, 1079, 64), (1000, 500, 33)]:
        rng["seeds"].append({"pixel_n": [px, py, n], "seed": world_ref.seed(px, py, n)})
    (OUT / "rng.json").write_text(json.dumps(rng, indent=1))

    bvh = {}
    corn = cornell_triangles()
    nodes, order = world_ref.build_bvh(corn)
    bvh["cornell"] = {"triangles": [int(b) for b in corn.view(np.uint32).ravel()],
                      "nodes": world_ref.nodes_as_u32(nodes).tolist(), "order": order.tolist()}
    for seed, n in [(7, 300), (11, 2000)]:
        soup = random_soup(seed, n)
        nodes, order = world_ref.build_bvh(soup)
        nu = world_ref.nodes_as_u32(nodes)
        bvh[f"soup_{seed}_{n}"] = {"seed": seed, "count": n, "node_count": len(nodes),
                                   "nodes_sha256": digest(nu), "order_sha256": digest(order)}
    (OUT / "bvh.json").write_text(json.dumps(bvh))

    alias = []
    r = np.random.default_rng(3)
    for weights in ([1.0, 2.0, 3.0, 4.0], [0.0, 5.0, 0.0, 1e-9, 3.0], list(r.exponential(size=40)),
                    [1.0] * 7):
        e = world_ref.alias_table(weights)
        alias.append({"weights": [float(x) for x in weights],
                      "entries": [[float(t), int(a), float(p)] for t, a, p in e]})
    (OUT / "alias.json").write_text(json.dumps(alias, indent=1))


if __name__ == "__main__":
    main()
