"""Pure-Python restatement of the reference's world-builder math - TEST INFRASTRUCTURE ONLY.

Written independently of path-tracer_gb300/csrc/world.cpp so the tests can
check the C++ builder node for node.  Float32 arithmetic is emulated exactly:
every operation rounds once to binary32 (numpy float32 scalars), and the
Rust `mul_add` calls are evaluated as exact rationals rounded once.

  subdivide            world.rs:1430-1591 (root world.rs:1339-1345)
  alias_table          world.rs:542-575
  light probabilities  world.rs:484-498
Small inputs only (pure Python loops).
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np

f32 = np.float32
INF = f32(np.inf)


def _round_f32(x: Fraction) -> np.float32:
    """Round an exact rational to the nearest binary32 (ties to even)."""
    c = f32(float(x))
    best = None
    for cand in (np.nextafter(c, f32(-np.inf)), c, np.nextafter(c, f32(np.inf))):
        if not np.isfinite(cand):
            continue
        err = abs(Fraction(float(cand)) - x)
        key = (err, int(np.array(cand, dtype=np.float32).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return best[1]


def fma32(a, b, c) -> np.float32:
    a, b, c = f32(a), f32(b), f32(c)
    if not (np.isfinite(a) and np.isfinite(b) and np.isfinite(c)):
        with np.errstate(all="ignore"):
            return f32(np.float64(a) * np.float64(b) + np.float64(c))
    return _round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def _min(a, b):
    return b if np.isnan(a) else (a if np.isnan(b) else (a if a < b else b))


def _max(a, b):
    return b if np.isnan(a) else (a if np.isnan(b) else (a if a > b else b))


class _Box:
    __slots__ = ("lo", "hi")

    def __init__(self):
        self.lo = [INF, INF, INF]
        self.hi = [-INF, -INF, -INF]

    def grow(self, lo, hi):
        self.lo = [_min(self.lo[k], lo[k]) for k in range(3)]
        self.hi = [_max(self.hi[k], hi[k]) for k in range(3)]

    def half_area(self):
        with np.errstate(all="ignore"):
            e = [f32(self.hi[k] - self.lo[k]) for k in range(3)]
            return fma32(e[2], e[0], fma32(e[0], e[1], f32(e[1] * e[2])))


def build_bvh(tris: np.ndarray):
    """tris: (n, 9) float32.  Returns (nodes list of (min3, left_first, max3, tri_count), order)."""
    t = np.asarray(tris, dtype=np.float32).reshape(-1, 9)
    items = []
    for i in range(t.shape[0]):
        v = [t[i, 0:3], t[i, 3:6], t[i, 6:9]]
        lo = [_min(_min(v[0][k], v[1][k]), v[2][k]) for k in range(3)]
        hi = [_max(_max(v[0][k], v[1][k]), v[2][k]) for k in range(3)]
        cen = [f32(f32(f32(v[0][k] + v[1][k]) + v[2][k]) / f32(3.0)) for k in range(3)]
        items.append((lo, hi, cen, i))
    nodes = [[None, 0, None, 0]]

    def bounds(a, b):
        box = _Box()
        for it in items[a:b]:
            box.grow(it[0], it[1])
        return box

    root = bounds(0, len(items))
    nodes[0][0], nodes[0][2] = root.lo, root.hi

    def bin_of(x):
        if not x > 0:
            return 0
        return min(int(x), 7)

    def subdivide(ni, start, end):
        count = end - start
        if count <= 2:
            nodes[ni][1], nodes[ni][3] = start, count
            return
        clo = [INF, INF, INF]
        chi = [-INF, -INF, -INF]
        for it in items[start:end]:
            clo = [_min(clo[k], it[2][k]) for k in range(3)]
            chi = [_max(chi[k], it[2][k]) for k in range(3)]
        best_axis, best_split, best_cost = 0, 0, f32(np.finfo(np.float32).max)
        for axis in range(3):
            lo, hi = clo[axis], chi[axis]
            if lo == hi:
                continue
            boxes = [_Box() for _ in range(8)]
            counts = [0] * 8
            scale = f32(f32(8.0) / f32(hi - lo))
            for it in items[start:end]:
                b = bin_of(f32(f32(it[2][axis] - lo) * scale))
                counts[b] += 1
                boxes[b].grow(it[0], it[1])
            la, lc, ra, rc = [None] * 7, [0] * 7, [None] * 7, [0] * 7
            acc, s = _Box(), 0
            for i in range(7):
                s += counts[i]
                acc.grow(boxes[i].lo, boxes[i].hi)
                lc[i], la[i] = s, acc.half_area()
            acc, s = _Box(), 0
            for i in range(7, 0, -1):
                s += counts[i]
                acc.grow(boxes[i].lo, boxes[i].hi)
                rc[i - 1], ra[i - 1] = s, acc.half_area()
            for i in range(7):
                with np.errstate(all="ignore"):
                    cost = fma32(f32(lc[i]), la[i], f32(f32(rc[i]) * ra[i]))
                if cost < best_cost:
                    best_cost, best_axis, best_split = cost, axis, i
        lo_n, hi_n = nodes[ni][0], nodes[ni][2]
        e = [f32(hi_n[k] - lo_n[k]) for k in range(3)]
        leaf_cost = f32(f32(count) * fma32(e[2], e[0], fma32(e[0], e[1], f32(e[1] * e[2]))))
        if best_cost >= leaf_cost:
            nodes[ni][1], nodes[ni][3] = start, count
            return
        lo, hi = clo[best_axis], chi[best_axis]
        scale = f32(f32(8.0) / f32(hi - lo))

        def get_bin(j):
            return bin_of(f32(f32(items[j][2][best_axis] - lo) * scale))

        left, right = start, end - 1
        while True:
            while left <= right and get_bin(left) <= best_split:
                left += 1
            while right > left and get_bin(right) > best_split:
                right -= 1
            if left >= right:
                break
            items[left], items[right] = items[right], items[left]
            left += 1
            right -= 1
        split = left
        lc_i = len(nodes)
        nodes.append([None, 0, None, 0])
        nodes.append([None, 0, None, 0])
        lb, rb = bounds(start, split), bounds(split, end)
        nodes[lc_i][0], nodes[lc_i][2] = lb.lo, lb.hi
        nodes[lc_i + 1][0], nodes[lc_i + 1][2] = rb.lo, rb.hi
        nodes[ni][1], nodes[ni][3] = lc_i, 0
        subdivide(lc_i, start, split)
        subdivide(lc_i + 1, split, end)

    subdivide(0, 0, len(items))
    order = np.array([it[3] for it in items], dtype=np.uint32)
    return nodes, order


def nodes_as_u32(nodes) -> np.ndarray:
    out = np.zeros((len(nodes), 8), dtype=np.uint32)
    for i, (lo, lf, hi, tc) in enumerate(nodes):
        out[i, 0:3] = np.array(lo, dtype=np.float32).view(np.uint32)
        out[i, 3] = lf
        out[i, 4:7] = np.array(hi, dtype=np.float32).view(np.uint32)
        out[i, 7] = tc
    return out


def alias_table(weights):
    """Vose alias entries (threshold f32, alias u32, selection probability f32)."""
    w = [float(x) for x in weights]
    total = 0.0
    for x in w:
        total += x
    if not total > 0.0:
        return []
    n = len(w)
    entries = [[f32(1.0), i, f32(x / total)] for i, x in enumerate(w)]
    scaled = [x / total * float(n) for x in w]
    small = [i for i in range(n) if scaled[i] < 1.0]
    large = [i for i in range(n) if not scaled[i] < 1.0]
    while small and large:
        low, high = small.pop(), large.pop()
        entries[low][0] = f32(min(max(scaled[low], 0.0), 1.0))
        entries[low][1] = high
        scaled[high] = (scaled[high] + scaled[low]) - 1.0
        (small if scaled[high] < 1.0 else large).append(high)
    return entries


def light_probabilities(geometry_flux: float, emissive_count: int, sky_flux: float):
    g = f32(geometry_flux) if emissive_count > 0 else f32(0.0)
    s = f32(sky_flux)
    scale = _max(g, s)
    if scale > 0:
        gg, ss = f32(g / scale), f32(s / scale)
        return f32(gg / f32(gg + ss)), f32(ss / f32(gg + ss))
    return f32(0.0), f32(0.0)


def pcg_rand(state: int, count: int):
    """rand() of trace.slang:195-202 on Python integers -> (floats, final state)."""
    out = []
    s = state & 0xFFFFFFFF
    for _ in range(count):
        s = (s * 747796405 + 2891336453) & 0xFFFFFFFF
        word = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
        bits = 0x3F800000 | (((word >> 22) ^ word) >> 9)
        out.append(np.array([bits], dtype=np.uint32).view(np.float32)[0] - f32(1.0))
    return np.array(out, dtype=np.float32), s


def seed(px: int, py: int, n: int) -> int:
    s = ((px * 0x9E3779B9) ^ (py * 0x85EBCA6B) ^ (n * 0x27D4EB2D) ^ 0xA511E9B3) & 0xFFFFFFFF
    return s | 1
