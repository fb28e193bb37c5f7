"""Image error of every configuration against the FP64 reference render on
the GPU (pt_render_fp64).

The FP64 render runs the whole path in double arithmetic from the same FP32
world buffers and the shader's own f32 random numbers (trace.slang:195-202,
736-737), so `render / fp64 - 1` measures the FP32 arithmetic error of the
image, not Monte Carlo noise.  It is first pinned to the CPU oracle's FP64
mode (oracle/trace_oracle.cpp, libm transcendentals) on crops of five
scenes; then whole images are compared:

  C1  Cornell room, 256x256, 16 spp, plain and wavefront kernels
  C2  procedural scene (2.1M triangles), 1920x1080, 64 spp, FP32 and compressed
  C3  textured Cornell room, 256x256, 1024 spp, FP32 and compressed
  C4  a sample of the batching mix through the engine (compressed form)
  C5  a served request stream with progressive refinements (compressed form)

Relative RMSE = sqrt(mean((a - b)^2)) / sqrt(mean(b^2)) over all pixels and
channels of the per-pixel means (trace.slang:1299-1308 accumulates per pixel).
Each bound sits just above the value measured on a GB300 (printed with -s):
the renders are deterministic, so a change in the FP32 arithmetic shows.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import pathtracer as pt
from pathtracer import abi
from pathtracer.engine import Engine
from pathtracer.serving import Request, Server, build_scene, request_stream
from worlds import material_zoo_world, non_opaque_world

pytestmark = pytest.mark.gpu

RESULTS = {}


def rel_rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def pixels_of(origin, size, image):
    xs = np.arange(origin[0], min(origin[0] + size[0], image[0]))
    ys = np.arange(origin[1], min(origin[1] + size[1], image[1]))
    return np.array([[x, y] for y in ys for x in xs], np.uint32)


def report(name, value, bound):
    RESULTS[name] = value
    print(f"\n  relative RMSE vs FP64, {name}: {value:.3e} (bound {bound:.1e})")
    assert value < bound, (name, value)


def render(updates, image, spp, bounces=8, kernel=abi.PT_KERNEL_WAVEFRONT, precision=abi.PT_PRECISION_FP32,
           tile=None, origin=(0, 0)):
    """FP32 (or compressed) accumulation of one tile, and the FP64 sums of the same paths."""
    tile = tile or image
    tr = pt.PathTracer(updates, tile)
    tr.set_kernel(kernel)
    tr.set_precision(precision)
    tr.set_max_bounces(bounces)
    tr.set_tile(image, origin, tile)
    while tr.sample_count() < spp:
        tr.trace(spp - tr.sample_count())
    assert tr.precision_active() == precision
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64)
    return tr, acc


# ------------------------------------------------ the FP64 render is the oracle's FP64 render

def crop_scenes():
    c = pt.World.cornell_box()
    c.set_aspect_ratio(1.0)
    t = pt.World.cornell_box_textured(1)
    t.set_aspect_ratio(1.0)
    p = pt.World.procedural(grid_x=256, grid_z=128, boxes=400, spheres=40, sphere_subdivision=3,
                            emissive_triangles=32, skybox_width=256, skybox_height=128)
    p.set_aspect_ratio(16 / 9)
    return {"cornell": (c, (256, 256), (100, 90), 4), "cornell_textured": (t, (256, 256), (100, 60), 4),
            "material_zoo": (material_zoo_world(), (128, 128), (40, 40), 2),
            "non_opaque": (non_opaque_world(), (128, 128), (40, 40), 2),
            "procedural": (p, (640, 360), (300, 170), 2)}


@pytest.mark.parametrize("name", ["cornell", "cornell_textured", "material_zoo", "non_opaque", "procedural"])
def test_gpu_fp64_render_equals_oracle_fp64(name):
    """Both FP64 renders take the same decisions; they differ only in the last bits of the
    transcendentals (CUDA's double functions against libm): measured <= 6e-16 relative RMSE."""
    world, image, origin, spp = crop_scenes()[name]
    u = world.take_updates()
    size = (32, 32)
    tr = pt.PathTracer(u, size)
    tr.set_max_bounces(8)
    tr.set_tile(image, origin, size)
    gpu = tr.render_fp64(1, spp)
    assert tr.sample_count() == 0  # the FP64 render leaves the accumulation alone
    tr.close()
    rad64, _ = oracle.trace_paths(oracle.world_from_updates(u), image, 8, pixels_of(origin, size, image), 1, spp,
                                  precision=64)
    cpu = rad64.sum(axis=0).reshape(size[1], size[0], 3)
    assert cpu.max() > 0
    assert rel_rmse(gpu, cpu) < 1e-12
    np.testing.assert_allclose(gpu, cpu, rtol=1e-9, atol=1e-12)


def test_fp64_render_arguments():
    w = pt.World.cornell_box()
    tr = pt.PathTracer(w.take_updates(), (8, 8))
    for first, count in ((0, 1), (1, 0), (0xFFFFFFFF, 2)):
        with pytest.raises(pt.PathTracerError) as e:
            tr.render_fp64(first, count)
        assert e.value.code == abi.PT_ERR_INVALID_ARG
    # an edge tile: pixels outside the image stay zero
    tr.set_tile((20, 20), (16, 16), (8, 8))
    out = tr.render_fp64(3, 1)
    assert out[4:, :].max() == 0 and out[:, 4:].max() == 0 and out[:4, :4].max() > 0
    tr.close()


# ------------------------------------------------------------------ whole images, every config

@pytest.mark.parametrize("kernel", [abi.PT_KERNEL_PLAIN, abi.PT_KERNEL_WAVEFRONT])
def test_c1_full_image(kernel):
    w = pt.World.cornell_box()
    w.set_aspect_ratio(1.0)
    tr, acc = render(w.take_updates(), (256, 256), 16, kernel=kernel)
    ref = tr.render_fp64(1, 16)
    tr.close()
    report(f"C1 256x256x16 {'plain' if kernel else 'wavefront'}", rel_rmse(acc / 16, ref / 16), 3.8e-5)


@pytest.fixture(scope="module")
def c2():
    w = pt.World.procedural()
    w.set_aspect_ratio(1920 / 1080)
    u = w.take_updates()
    tr, acc = render(u, (1920, 1080), 64)
    ref = tr.render_fp64(1, 64)
    tr.close()
    return w, u, acc, ref


def test_c2_full_image_fp32(c2):
    _, _, acc, ref = c2
    report("C2 1920x1080x64 FP32", rel_rmse(acc / 64, ref / 64), 1.2e-3)


def test_c2_full_image_compressed(c2):
    _, u, _, ref = c2
    tr, acc = render(u, (1920, 1080), 64, precision=abi.PT_PRECISION_COMPRESSED)
    tr.close()
    report("C2 1920x1080x64 compressed", rel_rmse(acc / 64, ref / 64), 6.5e-3)


@pytest.fixture(scope="module")
def c3():
    w = pt.World.cornell_box_textured(1)
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    tr, acc = render(u, (256, 256), 1024)
    ref = tr.render_fp64(1, 1024)
    tr.close()
    return w, u, acc, ref


def test_c3_full_image_fp32(c3):
    _, _, acc, ref = c3
    report("C3 256x256x1024 FP32", rel_rmse(acc / 1024, ref / 1024), 1.1e-5)


def test_c3_full_image_compressed(c3):
    """The precision contract: the compressed form within 1 % relative RMSE of FP64 at 1024 spp."""
    _, u, _, ref = c3
    tr, acc = render(u, (256, 256), 1024, precision=abi.PT_PRECISION_COMPRESSED)
    comp = tr.read_tile(abi.PT_TILE_COMPENSATION)
    tr.close()
    assert np.abs(comp).max() > 0  # Kahan sums in use
    assert rel_rmse(acc / 1024, ref / 1024) <= 1e-2
    report("C3 256x256x1024 compressed", rel_rmse(acc / 1024, ref / 1024), 1.0e-4)


@pytest.fixture(scope="module")
def mix_scenes():
    return {n: build_scene(n) for n in ("10k", "100k", "1M")}


def fp64_of_job(full, camera, width, height, samples, bounces):
    u = abi.WorldUpdates.from_buffer_copy(full)
    u.camera = C.pointer(camera)
    tr = pt.PathTracer(u, (width, height))
    tr.set_max_bounces(bounces)
    tr.set_tile((width, height), (0, 0), (width, height))
    ref = tr.render_fp64(1, samples)
    tr.close()
    return ref


@pytest.fixture(scope="module")
def c4_jobs(mix_scenes):
    """16 jobs of the batching mix (sides log-uniform 64-1024, aspect 1:1-16:9, spp {1,4,16,64}, depth
    4-12, random camera poses) of at most 2^22 paths each, on the 10k / 100k / 1M-triangle scenes,
    with the FP64 render of each."""
    eng = Engine(wave_paths=1 << 21, tile_size=32)
    server = Server(eng, mix_scenes)
    reqs = [r for r in request_stream(1000.0, 1.0, list(mix_scenes), seed=5, progressive_fraction=0.0)
            if r.width * r.height * r.samples <= 1 << 22][:16]
    cams = [server.camera(r.scene, r) for r in reqs]
    refs = [fp64_of_job(server.full[r.scene], cam, r.width, r.height, r.samples, r.max_bounces) / r.samples
            for r, cam in zip(reqs, cams)]
    eng.close()
    return server.full, reqs, cams, refs


@pytest.mark.parametrize("precision,bound", [(abi.PT_PRECISION_FP32, 1.3e-2), (abi.PT_PRECISION_COMPRESSED, 1.9e-2)])
def test_c4_batched_jobs(c4_jobs, precision, bound):
    """The jobs traced together in the engine's waves.  Most of them have 1-16 spp, so the error is
    that of single paths whose FP32 rounding flips a decision (a Russian-roulette draw, a lobe
    choice, a grazing hit), which averages away only with more samples (C3 at 1024 spp)."""
    full, reqs, cams, refs = c4_jobs
    eng = Engine(wave_paths=1 << 21, tile_size=32, precision=precision)
    ids = {name: eng.add_scene(u) for name, u in full.items()}
    jobs = [eng.submit(ids[r.scene], cam, r.width, r.height, r.samples, r.max_bounces) for r, cam in zip(reqs, cams)]
    eng.wait_idle(timeout_ms=0)
    num = den = 0.0
    worst = 0.0
    for r, jid, ref in zip(reqs, jobs, refs):
        acc = eng.read(jid, r.width, r.height, abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64) / r.samples
        num += float(np.sum((acc - ref) ** 2))
        den += float(np.sum(ref ** 2))
        worst = max(worst, rel_rmse(acc, ref))
    eng.close()
    form = "compressed" if precision else "FP32"
    print(f"\n  C4 {form} worst single job: {worst:.3e}")
    report(f"C4 16 batched jobs {form} (all pixels)", float(np.sqrt(num / den)), bound)


def test_c5_served_requests():
    """A Poisson stream of the serving mix (20 requests, a third of them progressive refinements of a
    resident accumulation) through the serving loop in the compressed form; every served result is
    compared with the FP64 render of all its samples."""
    eng = Engine(wave_paths=1 << 20, tile_size=32, precision=abi.PT_PRECISION_COMPRESSED)
    server = Server(eng, {"100k": build_scene("100k")})
    rng = np.random.default_rng(21)
    reqs, t = [], 0.0
    for _ in range(20):
        t += rng.exponential(1.0 / 200.0)
        w, h = [(256, 144), (192, 192)][int(rng.integers(2))]
        reqs.append(Request(t, "100k", w, h, int(rng.choice([4, 16])), 8, float(rng.uniform(-0.6, 0.6)),
                            float(rng.uniform(-0.5, -0.2)), progressive=bool(rng.random() < 0.35)))
    got = []

    def on_done(jid, req, cam, total):
        got.append((req, abi.Camera.from_buffer_copy(cam), total,
                    eng.read(jid, req.width, req.height, abi.PT_TILE_ACCUMULATION)[..., :3].astype(np.float64)))

    res = server.run(reqs, on_done=on_done)
    assert res.completed == len(reqs) and any(total > req.samples for req, _, total, _ in got)
    num = den = 0.0
    for req, cam, total, acc in got:
        ref = fp64_of_job(server.full["100k"], cam, req.width, req.height, total, req.max_bounces)
        num += float(np.sum((acc / total - ref / total) ** 2))
        den += float(np.sum((ref / total) ** 2))
    eng.close()
    report("C5 20 served requests incl. refinements (all pixels)", float(np.sqrt(num / den)), 9e-3)
