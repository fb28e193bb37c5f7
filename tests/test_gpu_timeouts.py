"""Bounded host waits (pt_synchronize, pte_wait_idle).

The reference waits for the GPU without bound (device.poll with
wait_indefinitely, headless.rs:249,373).  Here both waits take a limit: they
give up with PT_ERR_TIMEOUT while work is still queued, leave the context or
engine usable, and the work then completes with the bits an unwaited render
gets.  The limit runs out on real queued work (a render of tens of
milliseconds against a 1 ms limit); nothing on the GPU is made to hang.
"""
import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi
from pathtracer.engine import Engine

pytestmark = pytest.mark.gpu

SIZE = 1024


@pytest.fixture(scope="module")
def terrain():
    w = pt.World.procedural(grid_x=256, grid_z=128, boxes=400, spheres=40, sphere_subdivision=3,
                            emissive_triangles=32, skybox_width=256, skybox_height=128)
    w.set_aspect_ratio(1.0)
    return w, w.take_updates()


def render(updates, spp, wait_first_ms=None):
    tr = pt.PathTracer(updates, (SIZE, SIZE))
    tr.set_max_bounces(8)
    tr.set_tile((SIZE, SIZE), (0, 0), (SIZE, SIZE))
    assert tr.trace(spp) == spp  # queued on the context's stream; the call does not wait
    timed_out = False
    if wait_first_ms is not None:
        try:
            tr.synchronize(timeout_ms=wait_first_ms)
        except pt.PathTracerError as e:
            assert e.code == abi.PT_ERR_TIMEOUT and "did not finish" in e.message
            timed_out = True
    tr.synchronize()  # no limit
    acc = tr.read_tile(abi.PT_TILE_ACCUMULATION)
    assert tr.sample_count() == spp
    tr.close()
    return acc, timed_out


def test_synchronize_times_out_and_the_render_completes(terrain):
    _, u = terrain
    acc, timed_out = render(u, 16, wait_first_ms=1)
    assert timed_out  # 16.8 M paths on 600k triangles take far longer than 1 ms
    want, _ = render(u, 16)
    np.testing.assert_array_equal(acc.view(np.uint32), want.view(np.uint32))


def test_engine_wait_idle_times_out_and_the_job_completes(terrain):
    w, u = terrain
    cam = abi.Camera.from_buffer_copy(u.camera.contents)
    eng = Engine(wave_paths=1 << 20, tile_size=32)
    sid = eng.add_scene(u)
    jid = eng.submit(sid, cam, SIZE, SIZE, 64, 8)
    with pytest.raises(pt.PathTracerError) as e:
        eng.wait_idle(timeout_ms=1)
    assert e.value.code == abi.PT_ERR_TIMEOUT
    status, _ = eng.status(jid)
    assert status != abi.PT_JOB_DONE
    eng.wait_idle(timeout_ms=0)  # no limit
    status, done = eng.status(jid)
    assert status == abi.PT_JOB_DONE and done == 64
    acc = eng.read(jid, SIZE, SIZE, abi.PT_TILE_ACCUMULATION)
    eng.close()
    # the same job through pt_trace alone: the engine's bits equal it
    tr = pt.PathTracer(u, (SIZE, SIZE))
    tr.set_max_bounces(8)
    tr.set_tile((SIZE, SIZE), (0, 0), (SIZE, SIZE))
    done = 0
    while done < 64:
        done += tr.trace(64 - done)
    want = tr.read_tile(abi.PT_TILE_ACCUMULATION)
    tr.close()
    np.testing.assert_array_equal(acc.view(np.uint32), want.view(np.uint32))
