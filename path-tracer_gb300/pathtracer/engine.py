"""Python wrapper of the batched render engine (include/pt_batch.h)."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from . import PathTracerError, abi
from .abi import load


TUNED = Path(__file__).resolve().parent / "engine_tuned.json"


class Engine:
    """Many render jobs of uneven size, samples, depth and scene traced together on one GPU."""

    @staticmethod
    def tuned_config() -> dict:
        """The engine settings pte_autotune chose on the batching mix, in the FP16-attribute form
        (FP16 attributes / BF16 skybox + Kahan sums on the binary BVH: 640 Msamples/s there against
        575 for the full compressed form with the 8-wide BVH); engine_tuned.json, written by
        `python -m pathtracer.serving --compare 256 --scenes 10k,100k,1M,4M --precision half
        --autotune --save-tuned`."""
        return json.loads(TUNED.read_text())["config"]

    # Wave size for latency-bound serving.  A wave holds the paths the engine traces per launch
    # sequence; a request arriving while one is in flight waits for it.  On the serving stream of
    # the mixed workload (Poisson 50 req/s, a fifth of them 512x512 x 16 spp = 4.2M paths) the
    # 512x512 requests' p99 latency was 54 / 45 ms with 8M-path waves (the batching optimum),
    # 37 / 35 ms with 4M-path waves and 56 / 49 ms with 2M-path waves (two arrival seeds; more
    # waves per request cost more than the shorter wait saves); the GPU is about 45 % busy there,
    # so the smaller waves cost no throughput.
    SERVING_WAVE_PATHS = 4 << 20

    @classmethod
    def tuned(cls, device: int = 0, hbm_budget_bytes: int = 0, **overrides) -> "Engine":
        """An engine with the autotuned settings; keyword arguments replace single settings
        (e.g. wave_paths=Engine.SERVING_WAVE_PATHS for a latency-bound server)."""
        cfg = dict(cls.tuned_config(), **overrides)
        return cls(device=device, hbm_budget_bytes=hbm_budget_bytes, wave_paths=cfg["wave_paths"],
                   tile_size=cfg["tile_size"], steps_per_refill=cfg["steps_per_refill"], use_graphs=True,
                   precision=cfg["precision"], sort_min_hits=cfg["sort_min_hits"],
                   traversal_threads=cfg["traversal_threads"], shade_threads=cfg["shade_threads"])

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, wave_paths: int = 0, tile_size: int = 0,
                 steps_per_refill: int = 0, use_graphs: bool = True, precision: int = 0, sort_min_hits: int = 0,
                 traversal_threads: int = 0, shade_threads: int = 0):
        """precision: PT_PRECISION_* bits (0 = the reference's FP32 buffers, 6 = FP16 attributes / BF16
        skybox + Kahan sums, 7 = those and the 8-wide BVH: the compressed form);
        sort_min_hits: hits of a bounce are sorted by triangle bucket before shading from this many on
        (0 = the default 65536, 0xffffffff = never); traversal_threads / shade_threads: threads per block
        of the traversal kernels (64, 128 or 256; 0 = 128) and of the shading kernel (128, 256, 512 or 1024;
        0 = 1024)."""
        self._lib = load()
        cfg = abi.EngineConfig(device, hbm_budget_bytes, wave_paths, tile_size, steps_per_refill, int(use_graphs),
                               precision, sort_min_hits, traversal_threads, shade_threads)
        h = C.c_void_p()
        rc = self._lib.pte_create(C.byref(cfg), C.byref(h))
        if rc != abi.PT_OK:
            raise PathTracerError(rc, "pte_create failed (see stderr)")
        self._h = h

    def _check(self, rc: int) -> None:
        if rc != abi.PT_OK:
            raise PathTracerError(rc, self._lib.pte_last_error(self._h).decode(errors="replace"))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pte_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, full_updates: abi.WorldUpdates) -> int:
        sid = C.c_uint64()
        self._check(self._lib.pte_scene_add(self._h, C.byref(full_updates), C.byref(sid)))
        return sid.value

    def release_scene(self, scene_id: int) -> None:
        self._check(self._lib.pte_scene_release(self._h, scene_id))

    def submit(self, scene_id: int, camera: abi.Camera, width: int, height: int, samples: int, max_bounces: int,
               continue_job: int = 0) -> int:
        d = abi.JobDesc(scene_id, camera, width, height, samples, max_bounces, continue_job)
        jid = C.c_uint64()
        self._check(self._lib.pte_submit(self._h, C.byref(d), C.byref(jid)))
        return jid.value

    def poll(self, timeout_ms: int = 0, capacity: int = 256) -> list[int]:
        done = (C.c_uint64 * capacity)()
        n = C.c_uint32()
        self._check(self._lib.pte_poll(self._h, timeout_ms, done, capacity, C.byref(n)))
        return list(done[:n.value])

    def wait_idle(self, timeout_ms: int = 0) -> None:
        self._check(self._lib.pte_wait_idle(self._h, timeout_ms))

    def status(self, job_id: int) -> tuple[int, int]:
        st = C.c_int()
        n = C.c_uint32()
        self._check(self._lib.pte_job_status(self._h, job_id, C.byref(st), C.byref(n)))
        return st.value, n.value

    def read(self, job_id: int, width: int, height: int, which: int = abi.PT_TILE_IMAGE) -> np.ndarray:
        out = np.empty((height, width, 4), dtype=np.float32)
        self._check(self._lib.pte_job_read(self._h, job_id, which, out.ctypes.data))
        return out

    def release(self, job_id: int) -> None:
        self._check(self._lib.pte_job_release(self._h, job_id))

    def stats(self) -> dict:
        s = abi.EngineStats()
        self._check(self._lib.pte_stats(self._h, C.byref(s)))
        return {name: getattr(s, name) for name, _ in abi.EngineStats._fields_}

    def autotune(self, jobs: list[abi.JobDesc]) -> dict:
        arr = (abi.JobDesc * len(jobs))(*jobs)
        cfg = abi.EngineConfig()
        self._check(self._lib.pte_autotune(self._h, arr, len(jobs), C.byref(cfg)))
        return {name: getattr(cfg, name) for name, _ in abi.EngineConfig._fields_}
