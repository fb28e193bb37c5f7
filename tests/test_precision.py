"""Precision form, host side (include/pt_precision.h): the 8-wide BVH collapsed
from the reference's binary tree must contain every binary child box after
decoding (so no ray the binary traversal follows is culled), reach every
binary leaf exactly once, and quantise tightly; the FP16 attribute records
must round to nearest even like numpy's float16 conversion."""
import numpy as np
import pytest

import pathtracer as pt


def decode(origin, q, ebyte):
    """origin + q * 2^(e - 127) in float32: the product is exact, the sum rounds once (as in the kernel)."""
    s = np.ldexp(np.float32(1.0), ebyte.astype(np.int32) - 127).astype(np.float32)
    return (np.float32(origin) + q.astype(np.float32) * s).astype(np.float32)


def subtree_ranges(nodes: np.ndarray) -> dict:
    """(first triangle, count) of every binary subtree -> its node (children follow their parent)."""
    first = np.zeros(nodes.shape[0], np.int64)
    count = np.zeros(nodes.shape[0], np.int64)
    for k in range(nodes.shape[0] - 1, -1, -1):
        lf, tc = int(nodes[k, 3]), int(nodes[k, 7])
        if tc:
            first[k], count[k] = lf, tc
        else:
            first[k], count[k] = min(first[lf], first[lf + 1]), count[lf] + count[lf + 1]
    out = {}
    for k in range(nodes.shape[0]):  # the topmost node of a range wins
        out.setdefault((int(first[k]), int(count[k])), k)
    return out


def check_wide(nodes: np.ndarray, tri_count: int, merge: int = 0):
    wide, depth = pt.build_wide_bvh(nodes, merge)
    assert 1 <= depth <= 64
    assert 0 < wide.size <= nodes.shape[0]
    bmin = nodes[:, 0:3].view(np.float32)
    bmax = nodes[:, 4:7].view(np.float32)
    count = nodes[:, 7]
    node_of_range = subtree_ranges(nodes)
    seen_children = np.zeros(wide.size, dtype=np.int64)
    ranges = []
    for wi, w in enumerate(wide):
        n = int(w["child_count"])
        assert 1 <= n <= 8
        for i in range(n):
            c, tc = int(w["child"][i]), int(w["tri_count"][i])
            if tc:
                b = node_of_range[(c, tc)]
                assert count[b] > 0 or tc <= merge  # a binary leaf, or a merged small subtree
                ranges.append((c, tc))
            else:
                assert wi < c < wide.size  # children after parents: acyclic
                seen_children[c] += 1
                b = int(wide[c]["source_node"])
                assert count[b] == 0
            for a in range(3):
                lo = decode(w["origin"][a], np.array([w["lo"][a][i]]), np.array([w["exponent"][a]]))[0]
                hi = decode(w["origin"][a], np.array([w["hi"][a][i]]), np.array([w["exponent"][a]]))[0]
                assert lo <= bmin[b, a] and hi >= bmax[b, a], (wi, i, a)
                # tight: one quantum less would no longer contain the box
                ql, qh = int(w["lo"][a][i]), int(w["hi"][a][i])
                if ql < 255:
                    assert decode(w["origin"][a], np.array([ql + 1]), np.array([w["exponent"][a]]))[0] > bmin[b, a]
                if qh > 0:
                    assert decode(w["origin"][a], np.array([qh - 1]), np.array([w["exponent"][a]]))[0] < bmax[b, a]
    assert seen_children[0] == 0 and np.all(seen_children[1:] == 1)  # a tree
    ranges.sort()
    pos = 0
    for first, n in ranges:  # the leaves tile [0, triangles) exactly once
        assert first == pos
        pos += n
    assert pos == tri_count
    return wide


def test_wide_bvh_cornell():
    w = pt.World.cornell_box()
    wide = check_wide(w.bvh_nodes(), w.triangle_count())
    assert wide.size >= 1


def test_wide_bvh_procedural():
    w = pt.World.procedural(grid_x=48, grid_z=24, boxes=40, spheres=4, sphere_subdivision=2, emissive_triangles=8,
                            skybox_width=16, skybox_height=8)
    nodes = w.bvh_nodes()
    wide = check_wide(nodes, w.triangle_count())
    # the collapse opens up to 8 children: far fewer wide nodes than binary interior nodes
    assert wide["child_count"][0] == 8
    assert wide.size < 0.5 * np.count_nonzero(nodes[:, 7] == 0)


def test_wide_bvh_random_soups():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 17, 500):
        c = rng.uniform(-100, 100, (n, 1, 3))
        tris = (c + rng.normal(0, 1.5, (n, 3, 3))).astype(np.float32).reshape(n, 9)
        nodes, _ = pt.build_bvh(tris)
        check_wide(nodes, n)


@pytest.mark.parametrize("merge", [2, 4, 8])
def test_wide_bvh_merged_leaves(merge):
    w = pt.World.procedural(grid_x=48, grid_z=24, boxes=40, spheres=4, sphere_subdivision=2, emissive_triangles=8,
                            skybox_width=16, skybox_height=8)
    nodes = w.bvh_nodes()
    plain = check_wide(nodes, w.triangle_count())
    merged = check_wide(nodes, w.triangle_count(), merge)
    # binary leaves already hold up to 2 triangles, so merging pays from 4 on
    assert merged.size < plain.size if merge >= 4 else merged.size == plain.size
    assert merged["tri_count"].max() <= max(merge, int(nodes[:, 7].max()))


def test_wide_bvh_rejects_bad_trees():
    nodes = pt.World.cornell_box().bvh_nodes().copy()
    bad = nodes.copy()
    bad[0, 3] = nodes.shape[0] + 5  # root children out of range
    with pytest.raises(pt.PathTracerError):
        pt.build_wide_bvh(bad)
    cyc = nodes.copy()
    interior = np.nonzero(cyc[1:, 7] == 0)[0]
    if interior.size:
        i = int(interior[0]) + 1
        cyc[i, 3] = 1  # points back up towards the root: not a tree
        with pytest.raises(pt.PathTracerError):
            pt.build_wide_bvh(cyc)


def test_half_attributes_round_to_nearest_even():
    rng = np.random.default_rng(5)
    n = 4096
    vals = rng.normal(0, 1, (n, 27)).astype(np.float32)
    special = np.array([65504.0, 65519.996, 65520.0, 1e6, 2.0 ** -24, 2.0 ** -25, 1.5 * 2.0 ** -25, 2.0 ** -14,
                        2.0 ** -14 * (1 - 2.0 ** -11), -0.0, 1.0 + 2.0 ** -11, 1.0 + 3 * 2.0 ** -11, 1e-8,
                        -65520.0, 3.0e-5], dtype=np.float32)
    vals.reshape(-1)[: special.size] = special
    vals[:, 18:27:4] = np.where(rng.random((n, 3)) < 0.5, -1.0, 1.0)  # tangent handedness (w)
    mat = rng.integers(0, 1000, n, dtype=np.uint32)
    buf = np.zeros((n, 28), dtype=np.uint32)
    buf[:, 0] = mat
    buf[:, 1:] = vals.view(np.uint32)
    attrs = buf.copy()
    half = pt.half_attributes(attrs.view(np.dtype((np.void, 112))).reshape(n))
    h16 = half.view(np.uint16).reshape(n, 32)
    f = vals

    def exp16(a):
        with np.errstate(over="ignore"):
            return np.asarray(a, dtype=np.float32).astype(np.float16).view(np.uint16)
    # normals n0..n2: xyz then 0
    for k in range(3):
        np.testing.assert_array_equal(h16[:, 4 * k:4 * k + 3], exp16(f[:, 3 * k:3 * k + 3]))
        assert np.all(h16[:, 4 * k + 3] == 0)
    # uvs at float offsets 9..14 -> halves 24..29; tangents at 15..26 -> halves 12..23
    np.testing.assert_array_equal(h16[:, 24:30], exp16(f[:, 9:15]))
    np.testing.assert_array_equal(h16[:, 12:24], exp16(f[:, 15:27]))
    np.testing.assert_array_equal(half.view(np.uint32).reshape(n, 16)[:, 15], mat)


def fma32(a, b, c):
    """float32 fma: the exact product and sum rounded once (through float64; the rare double
    rounding is far inside the slack checked below)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def reference_accept(lo, hi, rcp, nod, hit_t):
    """The binary traversal's slab test (trace.slang:597-609) in float32."""
    t0 = fma32(lo, rcp, nod)
    t1 = fma32(hi, rcp, nod)
    with np.errstate(invalid="ignore"):
        near = np.fmax(np.fmax(np.fmin(t0[..., 0], t1[..., 0]), np.fmin(t0[..., 1], t1[..., 1])),
                       np.fmin(t0[..., 2], t1[..., 2]))
        far = np.fmin(np.fmin(np.fmax(t0[..., 0], t1[..., 0]), np.fmax(t0[..., 1], t1[..., 1])),
                      np.fmax(t0[..., 2], t1[..., 2]))
    return (near <= far) & (far > 0) & (near < hit_t)


def wide_accept(origin, ebyte, qlo, qhi, rcp, nod, hit_t):
    """The 8-wide kernel's test: t = fma(1 + q 2^-15, 2^(e+15) rcp, B - a15 -/+ eps) per bound."""
    a15 = (np.ldexp(np.float32(1), ebyte.astype(np.int32) - 127 + 15).astype(np.float32) * rcp).astype(np.float32)
    b = fma32(origin, rcp, nod)
    c0 = (b - a15).astype(np.float32)
    eps = ((np.abs(b) + np.abs(a15) + np.abs(nod)).astype(np.float32) * np.float32(2.0 ** -19)).astype(np.float32)
    neg = rcp < 0
    qn = np.where(neg, qhi, qlo).astype(np.float32)
    qf = np.where(neg, qlo, qhi).astype(np.float32)
    vn = (1 + qn * np.float32(2.0 ** -15)).astype(np.float32)
    vf = (1 + qf * np.float32(2.0 ** -15)).astype(np.float32)
    tn = fma32(vn, a15, (c0 - eps).astype(np.float32))
    tf = fma32(vf, a15, (c0 + eps).astype(np.float32))
    near = np.max(tn, axis=-1)
    far = np.min(tf, axis=-1)
    return (near <= far) & (far > 0) & (near < hit_t)


def test_wide_box_test_accepts_whatever_the_binary_test_accepts():
    """For every child of every wide node and many rays (random, and aimed at box corners and
    edges, where rounding decides), the kernel's slab test on the quantised box accepts every
    ray the reference's slab test accepts on the binary node the child stands for."""
    w = pt.World.procedural(grid_x=48, grid_z=24, boxes=40, spheres=4, sphere_subdivision=2, emissive_triangles=8,
                            skybox_width=16, skybox_height=8)
    nodes = w.bvh_nodes()
    wide, _ = pt.build_wide_bvh(nodes)
    node_of_range = subtree_ranges(nodes)
    rows = []  # (wide node, child slot, binary node)
    for wi, wn in enumerate(wide):
        for i in range(int(wn["child_count"])):
            c, tc = int(wn["child"][i]), int(wn["tri_count"][i])
            rows.append((wi, i, node_of_range[(c, tc)] if tc else int(wide[c]["source_node"])))
    rows = np.array(rows)
    bmin = nodes[rows[:, 2], 0:3].view(np.float32)
    bmax = nodes[rows[:, 2], 4:7].view(np.float32)
    origin = wide["origin"][rows[:, 0]].astype(np.float32)
    ebyte = wide["exponent"][rows[:, 0]]
    qlo = wide["lo"][rows[:, 0], :, rows[:, 1]]
    qhi = wide["hi"][rows[:, 0], :, rows[:, 1]]
    rng = np.random.default_rng(17)
    lo_all, hi_all = bmin.min(axis=0), bmax.max(axis=0)
    misses = 0
    for trial in range(24):
        n = rows.shape[0]
        o = rng.uniform(lo_all - 5, hi_all + 5, (n, 3)).astype(np.float32)
        if trial % 3 == 0:
            d = rng.normal(size=(n, 3))
        else:  # towards a corner (trial 1 mod 3) or an edge midpoint of the binary box
            pick = rng.integers(0, 2, (n, 3)).astype(bool)
            target = np.where(pick, bmin, bmax).astype(np.float64)
            if trial % 3 == 2:
                k = rng.integers(0, 3, n)
                target[np.arange(n), k] = 0.5 * (bmin[np.arange(n), k] + bmax[np.arange(n), k])
            d = target - o
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        with np.errstate(divide="ignore"):
            rcp = (np.float32(1) / d).astype(np.float32)
        nod = (-o * rcp).astype(np.float32)
        hit_t = np.where(rng.random(n) < 0.5, np.float32(np.inf), rng.uniform(0.1, 60, n)).astype(np.float32)
        ref = reference_accept(bmin, bmax, rcp, nod, hit_t)
        wid = wide_accept(origin, ebyte, qlo, qhi, rcp, nod, hit_t)
        misses += int(np.count_nonzero(ref & ~wid))
    assert misses == 0


def test_wide_children_placed_for_octant_order():
    """Eight clusters at the corners of a cube: the root wide node holds one cluster per slot, and slot s
    holds the cluster lying furthest back along octant s's direction (minus on the axes of s's set bits),
    so a ray with direction signs o that visits slots i ^ o, i = 0..7, meets the nearest cluster first."""
    rng = np.random.default_rng(5)
    tris = []
    for corner in range(8):
        c = np.array([(1 if corner & (1 << a) else -1) * 10.0 for a in range(3)])
        tris.append(c + rng.normal(0, 0.5, (6, 3, 3)))
    tris = np.concatenate(tris).astype(np.float32).reshape(-1, 9)
    nodes, _ = pt.build_bvh(tris)
    wide = check_wide(nodes, tris.shape[0])
    root = wide[0]
    assert int(root["child_count"]) == 8
    for s in range(8):
        center = [float(decode(root["origin"][a], root["lo"][a][s:s + 1], root["exponent"][a:a + 1])[0] +
                        decode(root["origin"][a], root["hi"][a][s:s + 1], root["exponent"][a:a + 1])[0]) / 2
                  for a in range(3)]
        for a in range(3):
            # D(s)[a] = -1 when bit a of s is set, so the slot's cluster sits at +10 there, else at -10
            assert (center[a] > 0) == bool(s & (1 << a)), (s, a, center)
