"""CUDA kernels vs the CPU oracle, through the C ABI.

Per path: node-visit order (FNV-1a hash), closest-hit triangle per bounce,
every counter and the radiance bits must be identical; the accumulation
buffer and storage texture must match the oracle's FP32 running sums bit for
bit, both from the recording kernels and from the kernels the library runs
otherwise; RMSE against the FP64 oracle render is reported and bounded.
"""
import numpy as np
import pytest

import oracle
import pathtracer as pt
from pathtracer import abi
from worlds import material_zoo_world, non_opaque_world

pytestmark = pytest.mark.gpu

KERNELS = [abi.PT_KERNEL_PLAIN, abi.PT_KERNEL_WAVEFRONT]


def pixels_of(origin, size, image):
    xs = np.arange(origin[0], min(origin[0] + size[0], image[0]))
    ys = np.arange(origin[1], min(origin[1] + size[1], image[1]))
    return np.array([[x, y] for y in ys for x in xs], np.uint32)


def assert_records_equal(gpu, ref):
    assert gpu.shape == ref.shape
    for field in ("visit_hash", "hit", "extend_rays", "shadow_rays", "interior_visits", "leaf_visits",
                  "triangle_tests", "shadow_interior_visits", "shadow_leaf_visits", "shadow_triangle_tests",
                  "rand_draws", "hits", "sky_misses", "light_samples", "sky_light_samples"):
        bad = np.nonzero(np.any((gpu[field] != ref[field]).reshape(gpu.shape[0], -1), axis=1))[0]
        assert bad.size == 0, f"{field} differs in {bad.size} paths, first {bad[:5]}"
    np.testing.assert_array_equal(gpu["radiance"].view(np.uint32), ref["radiance"].view(np.uint32))


def assert_fast_accumulation(tr, image, origin, size, spp, ref):
    """The kernels that run outside the tests (no per-path records) give the oracle's accumulation
    bits for the same paths: the tile is traced again from its first sample with pt_trace."""
    tr.set_tile(image, origin, size)
    done = 0
    while done < spp:
        done += tr.trace(spp - done)
    vis = (min(size[0], image[0] - origin[0]), min(size[1], image[1] - origin[1]))
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[:vis[1], :vis[0], :3].reshape(-1, 3)
    want = oracle.accumulate(ref["radiance"].reshape(spp, -1, 3))[-1]
    np.testing.assert_array_equal(acc.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("kernel", KERNELS)
def test_cornell_full_image_bit_exact(cornell, kernel):
    """Config 1: 256x256, 16 spp, max_bounces 8, every path of every sample."""
    _, updates, ow = cornell
    tr = pt.PathTracer(updates, (256, 256))
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    tr.set_tile((256, 256), (0, 0), (256, 256))
    gpu = tr.trace_recorded(16)
    assert tr.sample_count() == 16
    px = pixels_of((0, 0), (256, 256), (256, 256))
    rad, ref = oracle.trace_paths(ow, (256, 256), 8, px, 1, 16, records=True)
    assert_records_equal(gpu, ref)
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)
    want = oracle.accumulate(rad)[-1].reshape(256, 256, 3)
    np.testing.assert_array_equal(acc[..., :3].view(np.uint32), want.view(np.uint32))
    assert (acc[..., 3] == 1.0).all()
    img = tr.read_tile(abi.PT_TILE_IMAGE)
    want_img = (np.float32(abi.EXPOSURE) * want) / np.float32(16)
    np.testing.assert_array_equal(img[..., :3].view(np.uint32), want_img.astype(np.float32).view(np.uint32))
    # light actually reaches the camera through every bounce type
    assert ref["hits"].sum() > 0 and ref["light_samples"].sum() > 0 and ref["radiance"].max() > 0
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_cornell_fp64_rmse(cornell, kernel):
    """Relative RMSE of the FP32 GPU render against the FP64 oracle render (same RNG streams)."""
    _, updates, ow = cornell
    tr = pt.PathTracer(updates, (128, 128))
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    tr.set_tile((256, 256), (64, 64), (128, 128))
    tr.trace(16)
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64) / 16
    px = pixels_of((64, 64), (128, 128), (256, 256))
    rad64, _ = oracle.trace_paths(ow, (256, 256), 8, px, 1, 16, precision=64)
    ref = rad64.mean(axis=0).reshape(128, 128, 3)
    rel_rmse = np.sqrt(np.mean((acc - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    print(f"config 1 relative RMSE vs FP64 oracle (16 spp, 128x128 crop): {rel_rmse:.3e}")
    assert rel_rmse < 1e-3
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_tiles_edges_and_seed_independence(cornell, kernel):
    """Ragged edge tiles, tile-local accumulation and per-pixel seeds that do not depend on the tiling."""
    _, updates, ow = cornell
    image = (100, 70)
    results = {}
    for tile in (32, 64, 100):
        tr = pt.PathTracer(updates, (tile, tile))
        tr.set_kernel(kernel)
        tr.set_max_bounces(4)
        full = np.zeros((image[1], image[0], 3), np.float32)
        for y in range(0, image[1], tile):
            for x in range(0, image[0], tile):
                tr.set_tile(image, (x, y), (tile, tile))
                assert tr.trace(3) == 3
                vis = (min(tile, image[0] - x), min(tile, image[1] - y))
                acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)
                full[y:y + vis[1], x:x + vis[0]] = acc[:vis[1], :vis[0], :3]
        results[tile] = full
        tr.close()
    np.testing.assert_array_equal(results[32], results[64])
    np.testing.assert_array_equal(results[32], results[100])
    px = pixels_of((0, 0), image, image)
    rad, _ = oracle.trace_paths(ow, image, 4, px, 1, 3)
    want = oracle.accumulate(rad)[-1].reshape(image[1], image[0], 3)
    np.testing.assert_array_equal(results[32].view(np.uint32), want.view(np.uint32))


def random_rays(lo, hi, n, seed):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d[: n // 8, 0] = 0.0          # axis-parallel components: infinite reciprocals
    d[n // 8: n // 4, 1:] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def test_intersect_random_rays_cornell(cornell):
    _, updates, ow = cornell
    tr = pt.PathTracer(updates, (8, 8))
    o, d = random_rays(-0.2, 1.2, 20000, 1)
    hit, t, rec = tr.debug_intersect(o, d)
    rhit, rt, rrec = oracle.intersect(ow, o, d)
    np.testing.assert_array_equal(hit, rhit)
    np.testing.assert_array_equal(t.view(np.uint32), rt.view(np.uint32))
    np.testing.assert_array_equal(rec["visit_hash"], rrec["visit_hash"])
    np.testing.assert_array_equal(rec["triangle_tests"], rrec["triangle_tests"])
    assert (hit >= 0).mean() > 0.3
    tr.close()


@pytest.fixture(scope="module")
def large_world():
    """Config 2 scene (about 2.1M triangles) with its full upload and oracle view."""
    w = pt.World.procedural()
    w.set_aspect_ratio(1920 / 1080)
    u = w.take_updates()
    return w, u, oracle.world_from_updates(u)


def test_large_scene_intersect(large_world):
    w, u, ow = large_world
    tr = pt.PathTracer(u, (8, 8))
    o, d = random_rays(np.array([-30, 0, -15]), np.array([30, 12, 15]), 50000, 2)
    hit, t, rec = tr.debug_intersect(o, d)
    rhit, rt, rrec = oracle.intersect(ow, o, d)
    np.testing.assert_array_equal(hit, rhit)
    np.testing.assert_array_equal(t.view(np.uint32), rt.view(np.uint32))
    np.testing.assert_array_equal(rec["visit_hash"], rrec["visit_hash"])
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_large_scene_tile_bit_exact(large_world, kernel):
    """Config 2 scene, 1920x1080 image, a 64x64 tile, 4 spp, max_bounces 8: every path bit-exact."""
    w, u, ow = large_world
    assert w.triangle_count() > 2_000_000
    tr = pt.PathTracer(u, (64, 64))
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    light = sky = 0
    for origin in ((900, 500), (1880, 1050)):
        tr.set_tile((1920, 1080), origin, (64, 64))
        gpu = tr.trace_recorded(4).reshape(4, 64, 64)
        vis = (min(64, 1920 - origin[0]), min(64, 1080 - origin[1]))
        gpu = gpu[:, :vis[1], :vis[0]].reshape(-1)
        px = pixels_of(origin, (64, 64), (1920, 1080))
        _, ref = oracle.trace_paths(ow, (1920, 1080), 8, px, 1, 4, records=True)
        assert_records_equal(gpu, ref)
        assert_fast_accumulation(tr, (1920, 1080), origin, (64, 64), 4, ref)
        light += int(ref["light_samples"].sum())
        sky += int(ref["sky_light_samples"].sum())
    assert light > 0 and sky > 0  # both light categories exercised
    tr.close()


def test_counted_totals_match_records(cornell):
    _, updates, _ = cornell
    tr = pt.PathTracer(updates, (64, 64))
    tr.set_max_bounces(8)
    tr.set_tile((256, 256), (10, 20), (64, 64))
    _, totals = tr.trace_counted(3)
    tr.set_tile((256, 256), (10, 20), (64, 64))
    recs = tr.trace_recorded(3)
    for k in abi.COUNT_FIELDS:
        assert totals[k] == int(recs[k].sum()), k
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_textured_cornell_tile_bit_exact(kernel):
    """The precision workload's scene in FP32: procedural 1024^2 sRGB textures on four of eight meshes."""
    w = pt.World.cornell_box_textured(1)
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    ow = oracle.world_from_updates(u)
    tr = pt.PathTracer(u, (64, 64))
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    tr.set_tile((256, 256), (96, 128), (64, 64))
    gpu = tr.trace_recorded(4)
    px = pixels_of((96, 128), (64, 64), (256, 256))
    _, ref = oracle.trace_paths(ow, (256, 256), 8, px, 1, 4, records=True)
    assert_records_equal(gpu, ref)
    assert_fast_accumulation(tr, (256, 256), (96, 128), (64, 64), 4, ref)
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_gltf_textured_bit_exact(tmp_path, kernel):
    """A glTF scene whose material has PNG base-colour and metallic-roughness textures and a JPEG normal
    map, packed into the atlases by the import, under a sky: identical paths in kernels and oracle."""
    from test_gltf import write_gltf
    from test_texture_io import QUANT, _test_image, encode_jpeg, write_png
    rng = np.random.default_rng(4)
    base = write_png(rng.integers(0, 256, size=(64, 64, 3)), 2, 8)
    mr = write_png(rng.integers(0, 65536, size=(16, 16, 4)), 6, 16)
    normal, _ = encode_jpeg(_test_image(32, 32, 2), [(1, 1), (1, 1), (1, 1)], QUANT)
    mat = {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicRoughnessTexture": {"index": 1},
                                    "metallicFactor": 0.5},
           "normalTexture": {"index": 2, "scale": 0.8}}
    s2 = np.sqrt(0.5)
    nodes = [{"mesh": 0}, {"mesh": 0, "rotation": [s2, 0, 0, s2]}, {"mesh": 0, "rotation": [0, -s2, 0, s2]}]
    path = write_gltf(tmp_path, nodes, [0, 1, 2], [mat], True, images=[(base, "view"), (mr, "view"), (normal, "view")])
    w = pt.World.from_gltf(path)
    w.set_aspect_ratio(1.0)
    y, x = np.mgrid[0:32, 0:64]
    sky = np.stack([0.5 + 0.5 * np.sin(x / 10.0), 0.6 + 0.3 * np.cos(y / 6.0), np.full((32, 64), 0.9),
                    np.ones((32, 64))], axis=-1).astype(np.float32)
    w.set_skybox_rgba(sky)
    u = w.take_updates()
    assert u.scene.contents.srgb_atlas_count == 1 and u.scene.contents.linear_atlas_count == 1
    ow = oracle.world_from_updates(u)
    tr = pt.PathTracer(u, (64, 64))
    tr.set_kernel(kernel)
    tr.set_max_bounces(4)
    tr.set_tile((128, 128), (32, 32), (64, 64))
    gpu = tr.trace_recorded(2)
    _, ref = oracle.trace_paths(ow, (128, 128), 4, pixels_of((32, 32), (64, 64), (128, 128)), 1, 2, records=True)
    assert_records_equal(gpu, ref)
    assert_fast_accumulation(tr, (128, 128), (32, 32), (64, 64), 2, ref)
    assert (gpu["hits"] > 0).mean() > 0.5  # the camera sees the textured quads
    tr.close()
    w.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_large_scene_fp64_rmse(large_world, kernel):
    """Config 2: relative RMSE of a 48x48 crop at 64 spp against the FP64 oracle render (same RNG streams)."""
    w, u, ow = large_world
    origin, size, spp = (900, 500), (48, 48), 64
    tr = pt.PathTracer(u, size)
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    tr.set_tile((1920, 1080), origin, size)
    done = 0
    while done < spp:
        done += tr.trace(spp - done)
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64) / spp
    px = pixels_of(origin, size, (1920, 1080))
    rad64, _ = oracle.trace_paths(ow, (1920, 1080), 8, px, 1, spp, precision=64)
    ref = rad64.mean(axis=0).reshape(size[1], size[0], 3)
    rel_rmse = np.sqrt(np.mean((acc - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    print(f"config 2 relative RMSE vs FP64 oracle ({spp} spp, 48x48 crop, kernel {kernel}): {rel_rmse:.3e}")
    assert rel_rmse < 1e-2
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_non_opaque_tile_bit_exact(kernel):
    """BLEND and MASK materials: per-path visit order, hits, random-number draws (including those drawn
    inside the extend and shadow traversals) and radiance identical to the oracle."""
    w = non_opaque_world()
    u = w.take_updates()
    ow = oracle.world_from_updates(u)
    tr = pt.PathTracer(u, (48, 48))
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    draws = 0
    for origin in ((40, 60), (100, 100)):
        tr.set_tile((128, 128), origin, (48, 48))
        gpu = tr.trace_recorded(4).reshape(4, 48, 48)
        vis = (min(48, 128 - origin[0]), min(48, 128 - origin[1]))
        gpu = gpu[:, :vis[1], :vis[0]].reshape(-1)
        px = pixels_of(origin, (48, 48), (128, 128))
        _, ref = oracle.trace_paths(ow, (128, 128), 8, px, 1, 4, records=True)
        assert_records_equal(gpu, ref)
        assert_fast_accumulation(tr, (128, 128), origin, (48, 48), 4, ref)
        draws += int(ref["rand_draws"].sum())
    assert draws > 0
    # the paths' hits include surfaces of both non-opaque kinds
    mats = w.materials()
    mat_of_tri = np.frombuffer(w.attributes_raw().tobytes(), np.uint32).reshape(w.triangle_count(), -1)[:, 0]
    hits = ref["hit"][ref["hit"] >= 0]
    modes = {int(mats[int(mat_of_tri[t])].alpha_mode) for t in hits}
    assert {abi.PT_ALPHA_MODE_BLEND, abi.PT_ALPHA_MODE_MASK} <= modes
    tr.close()


@pytest.mark.parametrize("kernel", KERNELS)
def test_material_zoo_bit_exact(kernel):
    """Anisotropic GGX, a tinted coat at IOR 2.4 over a half-weight base, a half metal, a texture in every
    material slot (base colour, metallic-roughness, normal map, emission, specular colour and weight) and a
    textured half-weight emitter: every path identical to the oracle; with the 8-wide BVH of the precision
    form the accumulation is the oracle's too."""
    w = material_zoo_world()
    u = w.take_updates()
    ow = oracle.world_from_updates(u)
    image, origin, size = (128, 64), (16, 22), (96, 24)
    tr = pt.PathTracer(u, size)
    tr.set_kernel(kernel)
    tr.set_max_bounces(8)
    tr.set_tile(image, origin, size)
    gpu = tr.trace_recorded(4)
    px = pixels_of(origin, size, image)
    _, ref = oracle.trace_paths(ow, image, 8, px, 1, 4, records=True)
    assert_records_equal(gpu, ref)
    mat_of_tri = np.frombuffer(w.attributes_raw().tobytes(), np.uint32).reshape(w.triangle_count(), -1)[:, 0]
    first = ref["hit"][:, 0]
    assert set(range(5)) <= set(mat_of_tri[first[first >= 0]].tolist())  # every zoo sphere is seen
    assert_fast_accumulation(tr, image, origin, size, 4, ref)
    if kernel == abi.PT_KERNEL_WAVEFRONT:
        want = oracle.accumulate(ref["radiance"].reshape(4, -1, 3))[-1]
        tr.set_precision(abi.PT_PRECISION_WIDE_BVH)
        tr.set_tile(image, origin, size)
        tr.trace(4)
        assert tr.precision_active() == abi.PT_PRECISION_WIDE_BVH
        acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].reshape(-1, 3)
        np.testing.assert_array_equal(acc.view(np.uint32), want.view(np.uint32))
    tr.close()
