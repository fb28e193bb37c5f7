"""Precision form on the GPU (include/pt_precision.h).

* 8-wide quantised BVH: every ray's closest hit (triangle and t bits) equals
  the binary traversal's, and a render with only the wide BVH selected is
  bit-identical to the FP32 render (same hits, so the same paths).
* Kahan accumulation: the accumulation and compensation buffers equal a
  float32 Kahan sum of the per-sample radiance, in sample order.
* The full compressed form (wide BVH + FP16 attributes / BF16 skybox + Kahan)
  stays within 1 % relative RMSE of the FP64 oracle render.
"""
import numpy as np
import pytest

import oracle
import pathtracer as pt
from pathtracer import abi

pytestmark = pytest.mark.gpu


def pixels_of(origin, size, image):
    xs = np.arange(origin[0], min(origin[0] + size[0], image[0]))
    ys = np.arange(origin[1], min(origin[1] + size[1], image[1]))
    return np.array([[x, y] for y in ys for x in xs], np.uint32)


def rays(lo, hi, n, seed, axis_parallel: bool):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    if axis_parallel:
        d[: n // 2, 0] = 0.0
        d[n // 2:, 1:] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


@pytest.fixture(scope="module")
def scenes():
    out = {}
    w = pt.World.cornell_box()
    w.set_aspect_ratio(1.0)
    out["cornell"] = (w, w.take_updates(), (-0.2, 1.2))
    w = pt.World.procedural(grid_x=256, grid_z=128, boxes=400, spheres=40, sphere_subdivision=3,
                            emissive_triangles=32, skybox_width=256, skybox_height=128)
    w.set_aspect_ratio(1.0)
    out["terrain"] = (w, w.take_updates(), (np.array([-30, 0, -15]), np.array([30, 12, 15])))
    return out


@pytest.mark.parametrize("name", ["cornell", "terrain"])
def test_wide_hits_equal_binary(scenes, name):
    _, u, (lo, hi) = scenes[name]
    tr = pt.PathTracer(u, (8, 8))
    o, d = rays(lo, hi, 100000, 11, axis_parallel=False)
    hit, t, _ = tr.debug_intersect(o, d)
    tr.set_precision(abi.PT_PRECISION_WIDE_BVH)
    whit, wt, _ = tr.debug_intersect(o, d, records=False)
    diff = whit != hit
    tie = diff & (wt == t) & (hit >= 0) & (whit >= 0)
    nearer = diff & ((hit < 0) | (wt < t)) & (whit >= 0)
    print(f"{name}: {int(diff.sum())} of {hit.size} closest hits differ (exact-t ties {int(tie.sum())}, "
          f"wide nearer {int(nearer.sum())}); hit fraction {(hit >= 0).mean():.2f}")
    assert int(diff.sum()) == 0
    np.testing.assert_array_equal(wt.view(np.uint32), t.view(np.uint32))
    assert (hit >= 0).mean() > 0.3
    tr.close()


@pytest.mark.parametrize("name", ["cornell", "terrain"])
def test_wide_axis_parallel_rays_never_farther(scenes, name):
    """A zero direction component makes the reference's slab test compute 0 * inf; the wide test
    treats that axis as unconstrained, so it tests a superset of triangles: the same hit or a
    nearer one the binary box test culled, never a farther one."""
    _, u, (lo, hi) = scenes[name]
    tr = pt.PathTracer(u, (8, 8))
    o, d = rays(lo, hi, 40000, 12, axis_parallel=True)
    hit, t, _ = tr.debug_intersect(o, d)
    tr.set_precision(abi.PT_PRECISION_WIDE_BVH)
    whit, wt, _ = tr.debug_intersect(o, d, records=False)
    same = whit == hit
    print(f"{name}: axis-parallel rays, {int((~same).sum())} of {hit.size} hits differ "
          f"(binary missed {int(((hit < 0) & (whit >= 0)).sum())})")
    assert np.all(wt[hit >= 0] <= t[hit >= 0])
    assert np.all((whit >= 0)[hit >= 0])
    tr.close()


@pytest.mark.parametrize("name", ["cornell", "terrain"])
def test_wide_render_bit_identical(scenes, name):
    _, u, _ = scenes[name]
    out = []
    for prec in (abi.PT_PRECISION_FP32, abi.PT_PRECISION_WIDE_BVH):
        tr = pt.PathTracer(u, (96, 80))
        tr.set_precision(prec)
        tr.set_max_bounces(8)
        tr.set_tile((256, 256), (80, 90), (96, 80))
        tr.trace(6)
        assert tr.precision_active() == prec
        out.append(tr.read_tile(abi.PT_TILE_ACCUMULATION))
        tr.close()
    np.testing.assert_array_equal(out[0].view(np.uint32), out[1].view(np.uint32))
    assert out[0][..., :3].max() > 0


def kahan(rad):
    """float32 Kahan sums over axis 0 (samples in order); returns (sum, compensation)."""
    s = np.zeros(rad.shape[1:], np.float32)
    c = np.zeros(rad.shape[1:], np.float32)
    for x in rad.astype(np.float32):
        y = (x - c).astype(np.float32)
        t = (s + y).astype(np.float32)
        c = ((t - s).astype(np.float32) - y).astype(np.float32)
        s = t
    return s, c


def test_kahan_accumulation_exact(scenes):
    _, u, _ = scenes["cornell"]
    tr = pt.PathTracer(u, (48, 40))
    tr.set_precision(abi.PT_PRECISION_KAHAN)
    tr.set_max_bounces(8)
    tr.set_tile((128, 128), (30, 40), (48, 40))
    recs = [tr.trace_recorded(16), tr.trace_recorded(11)]  # the second call continues the sums
    assert tr.sample_count() == 27
    rad = np.concatenate([r["radiance"].reshape(-1, 40, 48, 3) for r in recs])
    want_sum, want_comp = kahan(rad)
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3]
    comp = tr.read_tile(abi.PT_TILE_COMPENSATION)[..., :3]
    np.testing.assert_array_equal(acc.view(np.uint32), want_sum.view(np.uint32))
    np.testing.assert_array_equal(comp.view(np.uint32), want_comp.view(np.uint32))
    plain = np.zeros((40, 48, 3), np.float32)
    for x in rad:
        plain = (plain + x).astype(np.float32)
    exact = rad.astype(np.float64).sum(axis=0)
    assert np.abs(acc - exact).sum() <= np.abs(plain - exact).sum()
    tr.close()


def test_compressed_rmse_vs_fp64():
    """Precision workload (textured Cornell room), all three compressions, vs the FP64 oracle."""
    w = pt.World.cornell_box_textured(1)
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    ow = oracle.world_from_updates(u)
    size, origin, image, spp = (48, 48), (100, 60), (256, 256), 128
    px = pixels_of(origin, size, image)
    rad64, _ = oracle.trace_paths(ow, image, 8, px, 1, spp, precision=64)
    ref = rad64.mean(axis=0).reshape(size[1], size[0], 3)
    errs = {}
    half = abi.PT_PRECISION_HALF_ATTRIBUTES | abi.PT_PRECISION_KAHAN
    for prec in (abi.PT_PRECISION_FP32, half, abi.PT_PRECISION_COMPRESSED):
        tr = pt.PathTracer(u, size)
        tr.set_precision(prec)
        tr.set_max_bounces(8)
        tr.set_tile(image, origin, size)
        done = 0
        while done < spp:
            done += tr.trace(spp - done)
        assert tr.precision_active() == prec
        acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64) / spp
        errs[prec] = np.sqrt(np.mean((acc - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
        tr.close()
    print(f"relative RMSE vs FP64 oracle at {spp} spp: FP32 {errs[0]:.3e}, FP16 attributes {errs[half]:.3e}, "
          f"compressed {errs[7]:.3e}")
    assert errs[abi.PT_PRECISION_FP32] < 1e-3
    assert errs[half] < 1e-2
    assert errs[abi.PT_PRECISION_COMPRESSED] < 1e-2


def test_precision_state_rules(scenes):
    _, u, _ = scenes["cornell"]
    tr = pt.PathTracer(u, (8, 8))
    with pytest.raises(pt.PathTracerError) as e:
        tr.set_precision(8)
    assert e.value.code == abi.PT_ERR_INVALID_ARG
    tr.set_kernel(abi.PT_KERNEL_PLAIN)
    with pytest.raises(pt.PathTracerError) as e:
        tr.set_precision(abi.PT_PRECISION_WIDE_BVH)
    assert e.value.code == abi.PT_ERR_STATE
    tr.set_kernel(abi.PT_KERNEL_WAVEFRONT)
    tr.set_precision(abi.PT_PRECISION_COMPRESSED)
    with pytest.raises(pt.PathTracerError) as e:
        tr.set_kernel(abi.PT_KERNEL_PLAIN)
    assert e.value.code == abi.PT_ERR_STATE
    tr.set_tile((8, 8), (0, 0), (8, 8))
    tr.trace(1)
    assert tr.precision_active() == abi.PT_PRECISION_COMPRESSED
    tr.close()


def test_non_opaque_world_keeps_binary_traversal():
    """Non-opaque materials draw random numbers in traversal order, so the wide BVH is not used."""
    w = pt.World.procedural(grid_x=64, grid_z=32, boxes=60, spheres=6, sphere_subdivision=2, emissive_triangles=8,
                            skybox_width=64, skybox_height=32, non_opaque=1)
    assert any(m.alpha_mode == abi.PT_ALPHA_MODE_BLEND for m in w.materials())
    w.set_aspect_ratio(1.0)
    tr = pt.PathTracer(w.take_updates(), (16, 16))
    tr.set_precision(abi.PT_PRECISION_COMPRESSED)
    tr.set_tile((64, 64), (20, 30), (16, 16))
    tr.trace(2)
    assert tr.precision_active() == abi.PT_PRECISION_COMPRESSED & ~abi.PT_PRECISION_WIDE_BVH
    assert np.isfinite(tr.read_tile(abi.PT_TILE_ACCUMULATION)).all()
    tr.close()
