"""Batched engine (include/pt_batch.h): jobs of different scenes, sizes,
sample counts and depths traced in shared waves must give exactly the bits
each job gets alone (through the engine, and through pt_trace)."""
import ctypes as C

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi
from pathtracer.engine import Engine
from worlds import non_opaque_world

pytestmark = pytest.mark.gpu


class SceneSet:
    """Worlds kept alive with their full uploads and a camera per aspect ratio."""

    def __init__(self):
        self.worlds = {
            "cornell": pt.World.cornell_box(),
            "terrain": pt.World.procedural(grid_x=96, grid_z=48, boxes=60, spheres=6, sphere_subdivision=2,
                                           emissive_triangles=12, skybox_width=128, skybox_height=64),
        }
        self.full = {name: w.take_updates() for name, w in self.worlds.items()}
        self.last = {name: abi.Camera.from_buffer_copy(u.camera.contents) for name, u in self.full.items()}

    def camera(self, name, width, height, yaw=0.0):
        """GpuCamera for this aspect ratio and yaw (camera edits only: the full uploads stay valid)."""
        w = self.worlds[name]
        w.set_aspect_ratio(width / height)
        w.edit_camera(yaw=yaw)
        u = w.take_updates()
        if u.camera:
            self.last[name] = abi.Camera.from_buffer_copy(u.camera.contents)
        return abi.Camera.from_buffer_copy(self.last[name])

    def updates_with_camera(self, name, camera):
        u = abi.WorldUpdates.from_buffer_copy(self.full[name])
        u.camera = C.pointer(camera)
        return u


@pytest.fixture(scope="module")
def scenes():
    return SceneSet()


def render_alone(scenes, name, camera, width, height, spp, bounces):
    tr = pt.PathTracer(scenes.updates_with_camera(name, camera), (width, height))
    tr.set_max_bounces(bounces)
    tr.set_tile((width, height), (0, 0), (width, height))
    done = 0
    while done < spp:
        done += tr.trace(spp - done)
    out = tr.read_tile(abi.PT_TILE_ACCUMULATION), tr.read_tile(abi.PT_TILE_IMAGE)
    tr.close()
    return out


JOBS = [("cornell", 96, 64, 4, 8, 0.0), ("terrain", 80, 80, 2, 5, 0.3), ("cornell", 33, 47, 3, 12, -0.2),
        ("terrain", 150, 40, 1, 4, 0.0), ("terrain", 64, 64, 6, 8, 1.0)]


def test_mixed_jobs_equal_alone(scenes):
    eng = Engine(wave_paths=1 << 15, tile_size=16)
    ids = {name: eng.add_scene(scenes.full[name]) for name in scenes.full}
    cams = [scenes.camera(n, w, h, yaw) for n, w, h, _, _, yaw in JOBS]
    jobs = [eng.submit(ids[n], cam, w, h, spp, b) for (n, w, h, spp, b, _), cam in zip(JOBS, cams)]
    eng.wait_idle(timeout_ms=300000)
    st = eng.stats()
    assert st["waves"] > 1 and st["jobs_done"] == len(JOBS)  # several waves, items from several jobs
    for (n, w, h, spp, b, _), cam, jid in zip(JOBS, cams, jobs):
        status, done = eng.status(jid)
        assert status == abi.PT_JOB_DONE and done == spp
        acc = eng.read(jid, w, h, abi.PT_TILE_ACCUMULATION)
        img = eng.read(jid, w, h, abi.PT_TILE_IMAGE)
        want_acc, want_img = render_alone(scenes, n, cam, w, h, spp, b)
        np.testing.assert_array_equal(acc.view(np.uint32), want_acc.view(np.uint32))
        np.testing.assert_array_equal(img.view(np.uint32), want_img.view(np.uint32))
    # the same jobs one at a time through the engine give the same bits
    for (n, w, h, spp, b, _), cam, jid in zip(JOBS[:2], cams, jobs):
        solo = eng.submit(ids[n], cam, w, h, spp, b)
        eng.wait_idle(timeout_ms=300000)
        np.testing.assert_array_equal(eng.read(solo, w, h, abi.PT_TILE_ACCUMULATION),
                                      eng.read(jid, w, h, abi.PT_TILE_ACCUMULATION))
    eng.close()



def test_non_opaque_jobs_equal_alone(scenes):
    """Jobs on a scene with BLEND and MASK materials (random numbers drawn inside traversal, so the engine
    runs them in its non-opaque waves) beside opaque Cornell jobs: each equals its pt_trace render alone."""
    w = non_opaque_world()
    full = w.take_updates()
    cam = abi.Camera.from_buffer_copy(full.camera.contents)
    eng = Engine(wave_paths=1 << 15, tile_size=16)
    nid = eng.add_scene(full)
    cid = eng.add_scene(scenes.full["cornell"])
    ccam = scenes.camera("cornell", 64, 48)
    spec = [(nid, cam, 96, 96, 3, 8), (cid, ccam, 64, 48, 2, 6), (nid, cam, 40, 40, 5, 12)]
    jobs = [eng.submit(sid, c, wd, ht, spp, b) for sid, c, wd, ht, spp, b in spec]
    eng.wait_idle(timeout_ms=300000)
    for (sid, c, wd, ht, spp, b), jid in zip(spec, jobs):
        assert eng.status(jid) == (abi.PT_JOB_DONE, spp)
        if sid == cid:
            want_acc, want_img = render_alone(scenes, "cornell", c, wd, ht, spp, b)
        else:
            u = abi.WorldUpdates.from_buffer_copy(full)
            u.camera = C.pointer(c)
            tr = pt.PathTracer(u, (wd, ht))
            tr.set_max_bounces(b)
            tr.set_tile((wd, ht), (0, 0), (wd, ht))
            while tr.sample_count() < spp:
                tr.trace(spp - tr.sample_count())
            want_acc, want_img = tr.read_tile(abi.PT_TILE_ACCUMULATION), tr.read_tile(abi.PT_TILE_IMAGE)
            tr.close()
        np.testing.assert_array_equal(eng.read(jid, wd, ht, abi.PT_TILE_ACCUMULATION).view(np.uint32),
                                      want_acc.view(np.uint32))
        np.testing.assert_array_equal(eng.read(jid, wd, ht, abi.PT_TILE_IMAGE).view(np.uint32),
                                      want_img.view(np.uint32))
    eng.close()



@pytest.mark.parametrize("shapes", [(64, 256), (256, 128), (128, 512)])
def test_block_shapes_keep_bits(scenes, shapes):
    """Other threads-per-block choices for the traversal and shading kernels give the same bits."""
    eng = Engine(wave_paths=1 << 15, tile_size=16, traversal_threads=shapes[0], shade_threads=shapes[1])
    assert (eng.stats()["traversal_threads"], eng.stats()["shade_threads"]) == shapes
    ids = {name: eng.add_scene(scenes.full[name]) for name in scenes.full}
    spec = JOBS[:3]
    cams = [scenes.camera(n, w, h, yaw) for n, w, h, _, _, yaw in spec]
    jobs = [eng.submit(ids[n], cam, w, h, spp, b) for (n, w, h, spp, b, _), cam in zip(spec, cams)]
    eng.wait_idle(timeout_ms=300000)
    for (n, w, h, spp, b, _), cam, jid in zip(spec, cams, jobs):
        want_acc, _ = render_alone(scenes, n, cam, w, h, spp, b)
        np.testing.assert_array_equal(eng.read(jid, w, h, abi.PT_TILE_ACCUMULATION).view(np.uint32),
                                      want_acc.view(np.uint32))
    eng.close()
    with pytest.raises(pt.PathTracerError):
        Engine(traversal_threads=96)


def test_progressive_refinement(scenes):
    eng = Engine(wave_paths=1 << 16, tile_size=32)
    sid = eng.add_scene(scenes.full["terrain"])
    cam = scenes.camera("terrain", 72, 48)
    first = eng.submit(sid, cam, 72, 48, 2, 8)
    second = eng.submit(sid, cam, 72, 48, 3, 8, continue_job=first)  # waits for the first pass
    eng.wait_idle(timeout_ms=300000)
    assert eng.status(second) == (abi.PT_JOB_DONE, 5)
    want_acc, want_img = render_alone(scenes, "terrain", cam, 72, 48, 5, 8)
    np.testing.assert_array_equal(eng.read(second, 72, 48, abi.PT_TILE_ACCUMULATION).view(np.uint32),
                                  want_acc.view(np.uint32))
    np.testing.assert_array_equal(eng.read(second, 72, 48, abi.PT_TILE_IMAGE).view(np.uint32),
                                  want_img.view(np.uint32))
    eng.release(first)
    eng.release(second)
    eng.close()


def test_hit_sorting_keeps_every_job_bit_exact(scenes):
    """Sorting each bounce's hits before shading only reorders the work: same bits as unsorted."""
    outs = []
    for sort in (1, 0xFFFFFFFF):  # sort from one hit on, and never
        eng = Engine(wave_paths=1 << 15, tile_size=16, sort_min_hits=sort)
        ids = {name: eng.add_scene(scenes.full[name]) for name in scenes.full}
        cams = [scenes.camera(n, w, h, yaw) for n, w, h, _, _, yaw in JOBS]
        jobs = [eng.submit(ids[n], cam, w, h, spp, b) for (n, w, h, spp, b, _), cam in zip(JOBS, cams)]
        eng.wait_idle(timeout_ms=300000)
        assert eng.stats()["sort_min_hits"] == sort
        outs.append([eng.read(j, w, h, abi.PT_TILE_ACCUMULATION) for (_, w, h, _, _, _), j in zip(JOBS, jobs)])
        eng.close()
    for a, b in zip(*outs):
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


def test_graph_replay_matches_plain_launches(scenes):
    outs = []
    for graphs in (True, False):
        eng = Engine(wave_paths=1 << 14, tile_size=16, use_graphs=graphs)
        sid = eng.add_scene(scenes.full["cornell"])
        cam = scenes.camera("cornell", 40, 40)
        j = eng.submit(sid, cam, 40, 40, 4, 6)
        eng.wait_idle(timeout_ms=300000)
        outs.append(eng.read(j, 40, 40, abi.PT_TILE_ACCUMULATION))
        assert eng.stats()["use_graphs"] == int(graphs)
        eng.close()
    np.testing.assert_array_equal(outs[0], outs[1])


def test_scene_cache_budget_and_eviction(scenes):
    eng = Engine(wave_paths=1 << 13, tile_size=16, hbm_budget_bytes=1 << 30)
    a = eng.add_scene(scenes.full["cornell"])
    assert eng.add_scene(scenes.full["cornell"]) == a  # identical content: cache hit
    st = eng.stats()
    assert st["scene_hits"] == 1 and st["scenes_cached"] == 1
    eng.release_scene(a)
    eng.release_scene(a)
    b = eng.add_scene(scenes.full["terrain"])
    assert b != a and eng.stats()["scenes_cached"] == 2
    eng.close()
    # a budget too small for the scene is refused, not oversubscribed
    small = Engine(wave_paths=1 << 12, tile_size=16, hbm_budget_bytes=(1 << 12) * 200 + (40 << 20))
    with pytest.raises(pt.PathTracerError) as e:
        small.add_scene(scenes.full["terrain"])
        small.add_scene(pt.World.procedural(grid_x=256, grid_z=256, boxes=0, spheres=0, emissive_triangles=4,
                                            skybox_width=64, skybox_height=32).take_updates())
    assert e.value.code == abi.PT_ERR_OOM
    small.close()


def test_scene_identity_is_content(scenes):
    """The cache keys scenes by their bytes, not their host pointers: a copy of a scene is a hit, and one
    changed texel of the sky (the last float of the last buffer hashed before the uniforms) is a new scene."""
    eng = Engine(wave_paths=1 << 13, tile_size=16)
    full = scenes.full["terrain"]
    a = eng.add_scene(full)
    k = full.skybox.contents
    n = 4 * k.uniforms.width * k.uniforms.height
    sky = np.ctypeslib.as_array(k.rgba, shape=(n,)).copy()
    u = abi.WorldUpdates.from_buffer_copy(full)
    up = abi.SkyboxUpload.from_buffer_copy(k)
    up.rgba = sky.ctypes.data_as(C.POINTER(C.c_float))
    u.skybox = C.pointer(up)
    assert eng.add_scene(u) == a  # same bytes at another address
    sky[n - 2] = np.nextafter(sky[n - 2], np.float32(np.inf))
    b = eng.add_scene(u)
    assert b != a
    st = eng.stats()
    assert st["scene_hits"] == 1 and st["scenes_cached"] == 2
    eng.close()


def test_poll_reports_each_job_once(scenes):
    eng = Engine(wave_paths=1 << 14, tile_size=16)
    sid = eng.add_scene(scenes.full["cornell"])
    cam = scenes.camera("cornell", 32, 32)
    ids = {eng.submit(sid, cam, 32, 32, 1 + k % 3, 4) for k in range(20)}
    seen = []
    for _ in range(10000):
        seen += eng.poll(timeout_ms=50)
        if len(seen) == len(ids):
            break
    assert sorted(seen) == sorted(ids)
    assert eng.poll(timeout_ms=0) == []
    eng.close()


def test_autotune_picks_a_candidate(scenes):
    eng = Engine(wave_paths=1 << 20, tile_size=32)
    sid = eng.add_scene(scenes.full["cornell"])
    cam = scenes.camera("cornell", 128, 128)
    cfg = eng.autotune([abi.JobDesc(sid, cam, 128, 128, 2, 4, 0), abi.JobDesc(sid, cam, 64, 64, 4, 4, 0)])
    assert cfg["wave_paths"] in (1 << 20, 1 << 21, 1 << 22, 1 << 23)
    assert cfg["tile_size"] in (16, 32, 64) and cfg["steps_per_refill"] in (16, 32)
    assert cfg["sort_min_hits"] in (65536, 0xFFFFFFFF)
    assert cfg["traversal_threads"] in (64, 128, 256) and cfg["shade_threads"] in (128, 256, 512, 1024)
    st = eng.stats()
    assert (st["traversal_threads"], st["shade_threads"]) == (cfg["traversal_threads"], cfg["shade_threads"])
    j = eng.submit(sid, cam, 64, 64, 2, 4)
    eng.wait_idle(timeout_ms=300000)
    assert eng.status(j)[0] == abi.PT_JOB_DONE
    eng.close()


@pytest.mark.parametrize("form", [abi.PT_PRECISION_COMPRESSED,
                                  abi.PT_PRECISION_HALF_ATTRIBUTES | abi.PT_PRECISION_KAHAN])
def test_compressed_engine_equals_alone(scenes, form):
    """The precision forms in the engine (8-wide BVH, FP16 attributes, BF16 sky, Kahan; or all but the
    8-wide BVH) give each job the bits pt_trace gives it alone in the same form."""
    eng = Engine(wave_paths=1 << 15, tile_size=16, precision=form)
    ids = {name: eng.add_scene(scenes.full[name]) for name in scenes.full}
    cams = [scenes.camera(n, w, h, yaw) for n, w, h, _, _, yaw in JOBS[:3]]
    jobs = [eng.submit(ids[n], cam, w, h, spp, b) for (n, w, h, spp, b, _), cam in zip(JOBS[:3], cams)]
    eng.wait_idle(timeout_ms=300000)
    for (n, w, h, spp, b, _), cam, jid in zip(JOBS[:3], cams, jobs):
        tr = pt.PathTracer(scenes.updates_with_camera(n, cam), (w, h))
        tr.set_precision(form)
        tr.set_max_bounces(b)
        tr.set_tile((w, h), (0, 0), (w, h))
        done = 0
        while done < spp:
            done += tr.trace(spp - done)
        for which in (abi.PT_TILE_ACCUMULATION, abi.PT_TILE_IMAGE, abi.PT_TILE_COMPENSATION):
            np.testing.assert_array_equal(eng.read(jid, w, h, which).view(np.uint32),
                                          tr.read_tile(which).view(np.uint32))
        tr.close()
    eng.close()
