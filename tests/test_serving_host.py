"""Host logic of the serving loop (pathtracer/serving.py) against a fake
engine on the CPU: every admitted request completes once, admission stops at
the outstanding-path cap, progressive requests continue a resident
accumulation of the same (scene, size, depth), and no more than
`keep_finished` finished jobs stay resident."""
import numpy as np

import pathtracer as pt
from pathtracer.serving import Request, Server, request_stream


class FakeEngine:
    """Jobs finish on the second poll after their submission; records what is resident."""

    def __init__(self):
        self.next = 1
        self.pending = []  # (job, polls seen)
        self.resident = set()
        self.max_resident = 0
        self.continued = []  # (job, continue_job)
        self.released = []

    def add_scene(self, updates):
        return 7

    def submit(self, scene_id, camera, width, height, samples, max_bounces, continue_job=0):
        assert scene_id == 7 and width > 0 and height > 0 and samples > 0
        if continue_job:
            assert continue_job in self.resident
            self.continued.append((self.next, continue_job))
        jid = self.next
        self.next += 1
        self.pending.append([jid, 0])
        self.resident.add(jid)
        self.max_resident = max(self.max_resident, len(self.resident))
        return jid

    def poll(self, timeout_ms=0):
        done = []
        for p in self.pending:
            p[1] += 1
            if p[1] >= 2:
                done.append(p[0])
        self.pending = [p for p in self.pending if p[1] < 2]
        return done

    def release(self, jid):
        assert jid in self.resident and all(p[0] != jid for p in self.pending)
        self.resident.discard(jid)
        self.released.append(jid)


def _server():
    w = pt.World.cornell_box()
    return Server(FakeEngine(), {"room": w})


def test_every_request_completes_and_residency_is_capped():
    server = _server()
    reqs = request_stream(rate=5000.0, duration=0.2, scenes=["room"], seed=3, progressive_fraction=0.3)
    # make keys collide so that progressive requests find finished jobs to continue
    for r in reqs:
        r.width, r.height, r.max_bounces = 64, 48, 4
    res = server.run(reqs, keep_finished=8)
    eng = server.engine
    assert res.completed == len(reqs) and res.rejected == 0
    assert eng.continued, "no progressive request continued a resident job"
    assert not eng.resident  # everything released at the end
    # resident: the jobs in flight plus at most 8 kept for refinement
    assert eng.max_resident <= 8 + len(reqs)
    assert len(set(eng.released)) == len(eng.released) == eng.next - 1


def test_keep_finished_bounds_resident_jobs():
    server = _server()
    reqs = [Request(0.0, "room", 32 + k, 32, 1, 4, 0.0, -0.3) for k in range(200)]  # all distinct keys
    res = server.run(reqs, keep_finished=16)
    assert res.completed == 200
    eng = server.engine
    # every request arrives at once: at most 200 in flight, and finished ones beyond 16 are released
    assert eng.max_resident <= 200
    assert not eng.resident


def test_outstanding_path_cap_rejects():
    server = _server()
    reqs = [Request(0.0, "room", 100, 100, 16, 4, 0.0, -0.3) for _ in range(10)]
    res = server.run(reqs, max_outstanding_paths=3 * 100 * 100 * 16)
    assert res.completed == 3 and res.rejected == 7
    assert np.all(np.array(res.latencies_ms) >= 0)


def test_refinements_keep_the_camera_and_count_samples():
    """A progressive request adds samples to the refined job's view: same camera, samples summed."""
    s = _server()
    cams = {}
    orig = s.engine.submit

    def submit(scene_id, camera, width, height, samples, max_bounces, continue_job=0):
        jid = orig(scene_id, camera, width, height, samples, max_bounces, continue_job)
        cams[jid] = bytes(camera)
        return jid

    s.engine.submit = submit
    seen = {}
    reqs = [Request(0.0, "room", 32, 32, 4, 6, 0.1, -0.3),
            Request(0.0, "room", 32, 32, 2, 6, -0.4, -0.2, progressive=True),
            Request(0.0, "room", 32, 32, 3, 6, 0.5, -0.4, progressive=True)]
    # the refinements arrive after the first job has finished
    reqs[1].arrival, reqs[2].arrival = 0.05, 0.1
    s.run(reqs, on_done=lambda jid, req, cam, total: seen.__setitem__(jid, (bytes(cam), total)))
    assert [c for _, c in s.engine.continued] == [1, 2]
    assert seen[1][1] == 4 and seen[2][1] == 6 and seen[3][1] == 9
    assert cams[1] == cams[2] == cams[3] == seen[3][0]
