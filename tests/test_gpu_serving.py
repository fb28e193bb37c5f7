"""The serving loop on the GPU (pathtracer/serving.py): requests arrive as a
Poisson stream while earlier ones are on the device, join the engine's waves
(compressed form), and some refine a resident accumulation.  Every served
result must carry the bits that a pt_trace render of the same request gives
alone in the same form - the refinements the bits of one render of all their
samples."""
import ctypes as C

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi
from pathtracer.engine import Engine
from pathtracer.serving import Request, Server, build_scene

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone():
    worlds = {"10k": build_scene("10k")}
    eng = Engine(wave_paths=1 << 18, tile_size=16, precision=abi.PT_PRECISION_COMPRESSED)
    server = Server(eng, worlds)
    rng = np.random.default_rng(11)
    sizes, reqs, t = [(96, 64), (64, 48)], [], 0.0
    for _ in range(40):
        t += rng.exponential(1.0 / 400.0)
        w, h = sizes[int(rng.integers(2))]
        reqs.append(Request(t, "10k", w, h, int(rng.choice([1, 4, 16])), int(rng.choice([4, 8])),
                            float(rng.uniform(-0.6, 0.6)), float(rng.uniform(-0.5, -0.2)),
                            progressive=bool(rng.random() < 0.3)))
    got = {}

    def on_done(jid, req, cam, total):
        got[jid] = (req, abi.Camera.from_buffer_copy(cam), total,
                    eng.read(jid, req.width, req.height, abi.PT_TILE_ACCUMULATION),
                    eng.read(jid, req.width, req.height, abi.PT_TILE_COMPENSATION))

    res = server.run(reqs, on_done=on_done)
    assert res.completed == len(reqs) == len(got) and res.rejected == 0
    assert any(total > req.samples for req, _, total, _, _ in got.values())  # refinements happened
    assert eng.stats()["waves"] > 1
    full = server.full["10k"]
    for jid, (req, cam, total, acc, comp) in got.items():
        u = abi.WorldUpdates.from_buffer_copy(full)
        u.camera = C.pointer(cam)
        tr = pt.PathTracer(u, (req.width, req.height))
        tr.set_precision(abi.PT_PRECISION_COMPRESSED)
        tr.set_max_bounces(req.max_bounces)
        tr.set_tile((req.width, req.height), (0, 0), (req.width, req.height))
        while tr.sample_count() < total:
            tr.trace(total - tr.sample_count())
        np.testing.assert_array_equal(acc.view(np.uint32), tr.read_tile(abi.PT_TILE_ACCUMULATION).view(np.uint32))
        np.testing.assert_array_equal(comp.view(np.uint32), tr.read_tile(abi.PT_TILE_COMPENSATION).view(np.uint32))
        tr.close()
    eng.close()
