"""CPU oracle of the path-trace pass - TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs import this package, and only as the checker or the timed CPU
baseline.  The product (path-tracer_gb300/) never imports it.

Parity unpinned: see oracle/oracle.h.  The restatement follows
src/render/trace.slang line by line (citations in trace_oracle.cpp).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "path-tracer_gb300"))

from pathtracer import abi  # noqa: E402  (types of the C ABI)
from pathtracer import RECORD_DTYPE, records_to_numpy  # noqa: E402

LIB_PATH = ROOT / "oracle" / "_build" / "liboracle.so"

FMATH = {"sin": 0, "cos": 1, "acos": 2, "atan2": 3, "pow": 4, "log2": 5, "exp2": 6, "sincos_sin": 7, "sincos_cos": 8}


class OracleWorld(C.Structure):
    _fields_ = [
        ("geometries", C.c_void_p), ("attributes", C.c_void_p), ("triangle_count", C.c_uint64),
        ("materials", C.c_void_p), ("material_count", C.c_uint64),
        ("bvh_nodes", C.c_void_p), ("node_count", C.c_uint64),
        ("srgb_atlases", C.c_void_p), ("srgb_atlas_count", C.c_uint32),
        ("linear_atlases", C.c_void_p), ("linear_atlas_count", C.c_uint32),
        ("camera", abi.Camera), ("skybox_rgba", C.c_void_p), ("skybox", abi.SkyboxUniforms),
        ("skybox_aliases", C.c_void_p), ("skybox_alias_count", C.c_uint64),
        ("scene", abi.SceneUniforms), ("scene_aliases", C.c_void_p), ("scene_alias_count", C.c_uint64),
    ]


_LIB = None


def load() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            from pathtracer.build import build
            build()
        lib = C.CDLL(str(LIB_PATH))
        P = C.POINTER
        lib.oracle_trace_paths.restype = C.c_int
        lib.oracle_trace_paths.argtypes = [P(OracleWorld), P(C.c_uint32), C.c_uint32, C.c_void_p, C.c_uint64,
                                           C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
        lib.oracle_intersect.restype = C.c_int
        lib.oracle_intersect.argtypes = [P(OracleWorld), C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_rand_sequence.restype = None
        lib.oracle_rand_sequence.argtypes = [C.c_uint32, C.c_uint32, C.c_void_p]
        lib.oracle_seed.restype = C.c_uint32
        lib.oracle_seed.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
        lib.oracle_fmath.restype = None
        lib.oracle_fmath.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]
        lib.oracle_max_threads.restype = C.c_int
        lib.oracle_max_threads.argtypes = []
        lib.oracle_elementary.restype = C.c_int
        lib.oracle_elementary.argtypes = [C.c_int, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.oracle_shade_cases.restype = C.c_int
        lib.oracle_shade_cases.argtypes = [C.c_int, C.c_void_p, C.c_uint64, C.c_void_p]
        lib.oracle_sample_lights.restype = C.c_int
        lib.oracle_sample_lights.argtypes = [P(OracleWorld), C.c_int, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]
        _LIB = lib
    return _LIB


def world_from_updates(u: abi.WorldUpdates) -> OracleWorld:
    """The world as the trace pass sees it, from a full upload (pointers stay owned by the World)."""
    if not (u.scene and u.skybox and u.camera and u.scene_uniforms and u.skybox_uniforms):
        raise ValueError("oracle needs a full world upload")
    s = u.scene.contents
    k = u.skybox.contents
    w = OracleWorld()
    w.geometries = C.cast(s.geometries, C.c_void_p)
    w.attributes = C.cast(s.attributes, C.c_void_p)
    w.triangle_count = s.triangle_count
    w.materials = C.cast(s.materials, C.c_void_p)
    w.material_count = s.material_count
    w.bvh_nodes = C.cast(s.bvh_nodes, C.c_void_p)
    w.node_count = s.node_count
    w.srgb_atlases = C.cast(s.srgb_texture_atlases, C.c_void_p)
    w.srgb_atlas_count = s.srgb_atlas_count
    w.linear_atlases = C.cast(s.linear_texture_atlases, C.c_void_p)
    w.linear_atlas_count = s.linear_atlas_count
    w.camera = u.camera.contents
    w.skybox_rgba = C.cast(k.rgba, C.c_void_p)
    w.skybox = u.skybox_uniforms.contents
    w.skybox_aliases = C.cast(k.alias_table, C.c_void_p)
    w.skybox_alias_count = k.alias_count
    w.scene = u.scene_uniforms.contents
    w.scene_aliases = C.cast(u.scene_alias_table, C.c_void_p)
    w.scene_alias_count = u.scene_alias_count
    return w


def trace_paths(world: OracleWorld, image_size, max_bounces: int, pixels: np.ndarray, sample_first: int,
                sample_count: int, precision: int = 32, threads: int = 0, records: bool = False):
    """Per-sample radiance [sample][pixel][3] (float32 for precision 32, float64 for 64) and records."""
    lib = load()
    px = np.ascontiguousarray(pixels, dtype=np.uint32).reshape(-1, 2)
    n = px.shape[0]
    img = (C.c_uint32 * 2)(*image_size)
    rad64 = np.zeros((sample_count, n, 3), dtype=np.float64)
    rad32 = np.zeros((sample_count, n, 3), dtype=np.float32) if precision == 32 else None
    recs = np.zeros(sample_count * n, dtype=RECORD_DTYPE) if records else None
    rc = lib.oracle_trace_paths(C.byref(world), img, max_bounces, px.ctypes.data, n, sample_first, sample_count,
                                precision, threads, rad32.ctypes.data if rad32 is not None else None,
                                rad64.ctypes.data, recs.ctypes.data if recs is not None else None)
    if rc != 0:
        raise ValueError("oracle_trace_paths rejected its arguments")
    return (rad32 if precision == 32 else rad64), recs


def intersect(world: OracleWorld, origins, directions, t_max=None):
    lib = load()
    o = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
    d = np.ascontiguousarray(directions, dtype=np.float32).reshape(-1, 3)
    n = o.shape[0]
    tm = np.full(n, np.finfo(np.float32).max, np.float32) if t_max is None else np.ascontiguousarray(t_max, np.float32)
    hit = np.empty(n, np.int32)
    ht = np.empty(n, np.float32)
    recs = np.zeros(n, dtype=RECORD_DTYPE)
    lib.oracle_intersect(C.byref(world), n, o.ctypes.data, d.ctypes.data, tm.ctypes.data, hit.ctypes.data,
                         ht.ctypes.data, recs.ctypes.data)
    return hit, ht, recs


def rand_sequence(state: int, count: int) -> np.ndarray:
    out = np.empty(count, np.float32)
    load().oracle_rand_sequence(state, count, out.ctypes.data)
    return out


def seed(px: int, py: int, n: int) -> int:
    return load().oracle_seed(px, py, n)


def fmath(name: str, x, y=None) -> np.ndarray:
    xa = np.ascontiguousarray(x, dtype=np.float32).ravel()
    ya = np.ascontiguousarray(y if y is not None else np.zeros_like(xa), dtype=np.float32).ravel()
    out = np.empty_like(xa)
    load().oracle_fmath(FMATH[name], xa.ctypes.data, ya.ctypes.data, out.ctypes.data, xa.size)
    return out


# oracle_elementary operations (oracle.h ORACLE_OP_*): name -> (op, inputs, output components)
ELEMENTARY = {"normalize": 0, "dot": 1, "mix": 2, "reflect": 3, "fract": 4, "min": 5, "max": 6, "clamp": 7,
              "rsqrt": 8, "to_u32": 9, "srgb": 10, "slab": 11, "camera_ray": 12}
_ELEM_OUT = {"normalize": 3, "reflect": 3, "camera_ray": 3}


def elementary(name: str, a, b=None, c=None) -> np.ndarray:
    """One of the parity mode's elementary operations over n elements (vectors as n x 3)."""
    op = ELEMENTARY[name]
    aa = np.ascontiguousarray(a, dtype=np.float32)
    n = aa.shape[0]
    ba = np.ascontiguousarray(b, dtype=np.float32) if b is not None else None
    ca = np.ascontiguousarray(c, dtype=np.float32) if c is not None else None
    k = _ELEM_OUT.get(name, 1)
    out = np.zeros((n, k) if k > 1 else n, dtype=np.float32)
    rc = load().oracle_elementary(op, n, aa.ctypes.data, ba.ctypes.data if ba is not None else None,
                                  ca.ctypes.data if ca is not None else None, out.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_elementary rejected its arguments")
    return out.view(np.uint32) if name == "to_u32" else out


SHADE_CASE = np.dtype([("base_color", "<f4", 3), ("base_weight", "<f4"), ("base_metalness", "<f4"),
                       ("base_diffuse_roughness", "<f4"), ("specular_color", "<f4", 3), ("specular_weight", "<f4"),
                       ("specular_roughness", "<f4"), ("specular_anisotropy", "<f4"), ("specular_ior", "<f4"),
                       ("wo", "<f4", 3), ("wi", "<f4", 3), ("rng", "<u4")])
SHADE_RESULT = np.dtype([("e_dielectric", "<f8", 3), ("p_ggx", "<f8"), ("p_u", "<f8"), ("f", "<f8", 3),
                         ("pdf", "<f8"), ("sampled_wi", "<f8", 3), ("sampled_f", "<f8", 3), ("sampled_pdf", "<f8"),
                         ("rng_after", "<u4"), ("pad", "<u4")])
LIGHT_RESULT = np.dtype([("direction", "<f8", 3), ("distance", "<f8"), ("emission", "<f8", 3), ("pdf", "<f8"),
                         ("triangle_index", "<i4"), ("rng_after", "<u4")])
assert SHADE_CASE.itemsize == 80 and SHADE_RESULT.itemsize == 136 and LIGHT_RESULT.itemsize == 72


def shade_cases(cases: np.ndarray, precision: int = 32) -> np.ndarray:
    """Shading points (SHADE_CASE records) -> SHADE_RESULT records (oracle_shade_cases)."""
    cs = np.ascontiguousarray(cases, dtype=SHADE_CASE)
    out = np.zeros(cs.shape[0], dtype=SHADE_RESULT)
    if load().oracle_shade_cases(precision, cs.ctypes.data, cs.shape[0], out.ctypes.data) != 0:
        raise ValueError("oracle_shade_cases rejected its arguments")
    return out


def sample_lights(world: OracleWorld, origins, rng_states, precision: int = 32) -> np.ndarray:
    """sample_light from each origin with its RNG state -> LIGHT_RESULT records."""
    o = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
    r = np.ascontiguousarray(rng_states, dtype=np.uint32)
    out = np.zeros(o.shape[0], dtype=LIGHT_RESULT)
    if load().oracle_sample_lights(C.byref(world), precision, o.shape[0], o.ctypes.data, r.ctypes.data,
                                   out.ctypes.data) != 0:
        raise ValueError("oracle_sample_lights rejected its arguments")
    return out


def max_threads() -> int:
    return load().oracle_max_threads()


def accumulate(radiance: np.ndarray) -> np.ndarray:
    """Running per-pixel sums in sample order, FP32 (trace.slang:1303): [sample][pixel][3]."""
    acc = np.empty_like(radiance, dtype=np.float32)
    run = np.zeros(radiance.shape[1:], dtype=np.float32)
    for s in range(radiance.shape[0]):
        run = (run + radiance[s].astype(np.float32)).astype(np.float32)
        acc[s] = run
    return acc


__all__ = ["OracleWorld", "world_from_updates", "trace_paths", "intersect", "rand_sequence", "seed", "fmath",
           "accumulate", "max_threads", "load", "elementary", "shade_cases", "sample_lights", "SHADE_CASE"]
