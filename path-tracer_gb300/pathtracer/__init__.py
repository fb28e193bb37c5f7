"""GB300 path-trace pass behind the reference's render interface.

`World` mirrors the reference's world builder (src/render/world.rs: World::new,
edit_* , take_updates), `PathTracer` mirrors src/render/path_tracer.rs
(PathTracer::new, set_tile, set_max_bounces, apply_updates, trace,
sample_count) and `render_tiles` mirrors headless::render_tiles
(src/render/headless.rs:207-285).  All compute runs in libpt.so through the C
ABI of include/pt.h; failures raise PathTracerError carrying the C status
code and message.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi
from .abi import load


class PathTracerError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{abi.ERROR_NAMES.get(code, code)}: {message}")
        self.code = code
        self.message = message


def _as_array(ptr, ctype, count: int) -> np.ndarray:
    if count == 0:
        return np.zeros(0, dtype=np.dtype((np.void, C.sizeof(ctype))))
    buf = C.cast(ptr, C.POINTER(ctype * count)).contents
    return np.frombuffer(buf, dtype=np.dtype((np.void, C.sizeof(ctype)))).copy()


class World:
    """Host-side world: scene buffers, BVH, lights, skybox and camera."""

    def __init__(self, handle: int):
        self._lib = load()
        self._h = C.c_void_p(handle)

    # --- construction
    @classmethod
    def empty(cls) -> "World":
        lib = load()
        h = C.c_void_p()
        cls._check_static(lib, lib.ptw_create(C.byref(h)), "ptw_create")
        return cls(h.value)

    @classmethod
    def cornell_box(cls) -> "World":
        lib = load()
        h = C.c_void_p()
        cls._check_static(lib, lib.ptw_scene_cornell_box(C.byref(h)), "ptw_scene_cornell_box")
        return cls(h.value)

    @classmethod
    def from_gltf(cls, path, build: bool = True) -> "World":
        """A world holding a glTF 2.0 scene (.glb / .gltf); built (BVH, camera) unless build=False."""
        w = cls.empty()
        err = C.create_string_buffer(512)
        rc = w._lib.ptw_load_gltf(w._h, str(path).encode(), err, len(err))
        if rc != abi.PT_OK:
            w.close()
            raise PathTracerError(rc, f"glTF import of {path}: {err.value.decode(errors="replace")}")
        if build:
            w.build()
        return w

    @classmethod
    def from_gltf_bytes(cls, data: bytes, build: bool = True) -> "World":
        """A world holding a .glb (or self-contained .gltf) given as bytes, as Scene::new(bytes) takes it."""
        w = cls.empty()
        err = C.create_string_buffer(512)
        buf = C.create_string_buffer(bytes(data), len(data))
        rc = w._lib.ptw_load_gltf_bytes(w._h, buf, len(data), err, len(err))
        if rc != abi.PT_OK:
            w.close()
            raise PathTracerError(rc, f"glTF import: {err.value.decode(errors="replace")}")
        if build:
            w.build()
        return w

    @classmethod
    def cornell_box_textured(cls, seed: int = 1) -> "World":
        """The Cornell room as eight meshes, four with procedural 1024^2 textures (precision workload)."""
        lib = load()
        h = C.c_void_p()
        cls._check_static(lib, lib.ptw_scene_cornell_box_textured(seed, C.byref(h)), "ptw_scene_cornell_box_textured")
        return cls(h.value)

    @staticmethod
    def procedural_defaults() -> abi.ProceduralParams:
        p = abi.ProceduralParams()
        load().ptw_procedural_defaults(C.byref(p))
        return p

    @classmethod
    def procedural(cls, params: abi.ProceduralParams | None = None, **overrides) -> "World":
        lib = load()
        p = params if params is not None else cls.procedural_defaults()
        for k, v in overrides.items():
            setattr(p, k, v)
        h = C.c_void_p()
        cls._check_static(lib, lib.ptw_scene_procedural(C.byref(p), C.byref(h)), "ptw_scene_procedural")
        return cls(h.value)

    @staticmethod
    def _check_static(lib, rc: int, what: str) -> None:
        if rc != abi.PT_OK:
            raise PathTracerError(rc, what)

    def _check(self, rc: int) -> None:
        if rc != abi.PT_OK:
            raise PathTracerError(rc, self._lib.ptw_last_error(self._h).decode(errors="replace"))

    def close(self) -> None:
        if self._h:
            self._lib.ptw_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- editing (world.rs:613-787)
    def add_material(self, material: abi.Material) -> int:
        idx = C.c_uint32()
        self._check(self._lib.ptw_add_material(self._h, C.byref(material), C.byref(idx)))
        return idx.value

    def add_mesh(self, positions, material_index: int, normals=None, uvs=None, tangents=None, indices=None) -> None:
        keep = []

        def ptr(a, dtype, ctype):
            if a is None:
                return None
            arr = np.ascontiguousarray(a, dtype=dtype)
            keep.append(arr)
            return arr.ctypes.data_as(C.POINTER(ctype))

        pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 3)
        m = abi.Mesh()
        m.positions = ptr(pos, np.float32, C.c_float)
        m.normals = ptr(normals, np.float32, C.c_float)
        m.uvs = ptr(uvs, np.float32, C.c_float)
        m.tangents = ptr(tangents, np.float32, C.c_float)
        m.vertex_count = pos.shape[0]
        if indices is not None:
            idx = np.ascontiguousarray(indices, dtype=np.uint32).ravel()
            m.indices = ptr(idx, np.uint32, C.c_uint32)
            m.index_count = idx.size
        m.material_index = material_index
        self._check(self._lib.ptw_add_mesh(self._h, C.byref(m)))

    def build(self) -> None:
        self._check(self._lib.ptw_build(self._h))

    def set_skybox_rgba(self, rgba: np.ndarray) -> None:
        a = np.ascontiguousarray(rgba, dtype=np.float32)
        h, w = a.shape[0], a.shape[1]
        self._check(self._lib.ptw_set_skybox_rgba(self._h, a.ctypes.data, w, h))

    def set_skybox_file(self, path) -> None:
        """Skybox from a Radiance .hdr or OpenEXR .exr file (the reference's skybox assets)."""
        err = C.create_string_buffer(512)
        rc = self._lib.ptw_set_skybox_file(self._h, str(path).encode(), err, len(err))
        if rc != abi.PT_OK:
            raise PathTracerError(rc, f"skybox {path}: {err.value.decode(errors="replace")}")

    def set_skybox_bytes(self, data: bytes) -> None:
        """Skybox from an .hdr / .exr image given as bytes (World::replace_skybox)."""
        err = C.create_string_buffer(512)
        buf = C.create_string_buffer(bytes(data), len(data))
        rc = self._lib.ptw_set_skybox_bytes(self._h, buf, len(data), err, len(err))
        if rc != abi.PT_OK:
            raise PathTracerError(rc, f"skybox: {err.value.decode(errors="replace")}")

    def edit_emission_scale(self, scale: float) -> None:
        """World::edit_emission_scale: emissive materials get their initial strength times `scale`."""
        self._check(self._lib.ptw_edit_emission_scale(self._h, scale))

    def emission_scale(self) -> float:
        return self._lib.ptw_emission_scale(self._h)

    def edit_skybox_average_luminance(self, luminance: float) -> None:
        self._check(self._lib.ptw_edit_skybox_average_luminance(self._h, luminance))

    def set_aspect_ratio(self, aspect: float) -> None:
        self._check(self._lib.ptw_set_aspect_ratio(self._h, aspect))

    def edit_camera(self, position=None, yaw=None, pitch=None, fov=None) -> None:
        def f(v, n=1):
            return None if v is None else (C.c_float * n)(*([v] if n == 1 else v))
        self._check(self._lib.ptw_edit_camera(self._h, f(position, 3), f(yaw), f(pitch), f(fov)))

    def edit_material(self, index: int, material: abi.Material) -> None:
        self._check(self._lib.ptw_edit_material(self._h, index, C.byref(material)))

    def take_updates(self) -> abi.WorldUpdates:
        u = abi.WorldUpdates()
        self._check(self._lib.ptw_take_updates(self._h, C.byref(u)))
        return u

    # --- read access
    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def triangle_count(self) -> int:
        return self._lib.ptw_triangle_count(self._h)

    def node_count(self) -> int:
        return self._lib.ptw_node_count(self._h)

    def material_count(self) -> int:
        return self._lib.ptw_material_count(self._h)

    def bvh_max_depth(self) -> int:
        return self._lib.ptw_bvh_max_depth(self._h)

    def geometries(self) -> np.ndarray:
        n = self.triangle_count()
        return _as_array(self._lib.ptw_geometries(self._h), abi.TriangleGeometry, n).view(np.float32).reshape(n, 9)

    def attributes_raw(self) -> np.ndarray:
        return _as_array(self._lib.ptw_attributes(self._h), abi.TriangleAttribute, self.triangle_count())

    def bvh_nodes(self) -> np.ndarray:
        """(node_count, 8) uint32 view: aabb_min bits, left_first, aabb_max bits, tri_count."""
        n = self.node_count()
        return _as_array(self._lib.ptw_bvh_nodes(self._h), abi.BvhNode, n).view(np.uint32).reshape(n, 8)

    def bvh_order(self) -> np.ndarray:
        n = self.triangle_count()
        return np.ctypeslib.as_array(self._lib.ptw_bvh_order(self._h), shape=(n,)).copy()

    def materials(self) -> list[abi.Material]:
        n = self.material_count()
        p = self._lib.ptw_materials(self._h)
        return [abi.Material.from_buffer_copy(p[i]) for i in range(n)]


def default_material() -> abi.Material:
    m = abi.Material()
    load().ptw_default_material(C.byref(m))
    return m


def alias_table(weights) -> np.ndarray:
    """Vose alias table of world.rs:542-575 as a structured array."""
    w = np.ascontiguousarray(weights, dtype=np.float64)
    out = (abi.SkyboxAliasEntry * max(1, w.size))()
    n = load().ptw_alias_table(w.ctypes.data, w.size, C.addressof(out))
    dt = np.dtype([("threshold", "<f4"), ("alias_index", "<u4"), ("selection_probability", "<f4")])
    return np.frombuffer(bytes(out), dtype=dt)[:n].copy()


WIDE_NODE_DTYPE = np.dtype([("origin", "<f4", 3), ("exponent", "u1", 3), ("child_count", "u1"),
                            ("lo", "u1", (3, 8)), ("hi", "u1", (3, 8)), ("child", "<u4", 8),
                            ("tri_count", "<u2", 8), ("source_node", "<u4"), ("pad", "<u4", 3)])


def build_wide_bvh(nodes: np.ndarray, max_leaf_triangles: int = 0):
    """8-wide quantised BVH of the precision form from binary nodes ((m, 8) uint32 as World.bvh_nodes())
    -> (structured array of WIDE_NODE_DTYPE, depth); subtrees of at most max_leaf_triangles become leaves."""
    lib = load()
    b = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 8)
    bp = b.ctypes.data_as(C.POINTER(abi.BvhNode))
    count, depth = C.c_uint64(), C.c_uint32()
    rc = lib.pt_build_wide_bvh(bp, b.shape[0], max_leaf_triangles, None, 0, C.byref(count), C.byref(depth))
    if rc:
        raise PathTracerError(rc, "pt_build_wide_bvh rejected the tree")
    out = np.zeros(count.value, dtype=WIDE_NODE_DTYPE)
    rc = lib.pt_build_wide_bvh(bp, b.shape[0], max_leaf_triangles, out.ctypes.data, count.value, C.byref(count),
                               C.byref(depth))
    if rc:
        raise PathTracerError(rc, "pt_build_wide_bvh failed")
    return out, depth.value


def half_attributes(attributes: np.ndarray) -> np.ndarray:
    """FP16 attribute records (64 B each, as uint16 / uint32 fields) of FP32 TriangleAttribute records."""
    a = np.ascontiguousarray(attributes)
    n = a.size
    out = np.zeros(n * 64, dtype=np.uint8)
    load().pt_half_attributes(a.ctypes.data_as(C.POINTER(abi.TriangleAttribute)), n, out.ctypes.data)
    return out.reshape(n, 64)


def read_image(path) -> np.ndarray:
    """A Radiance .hdr or OpenEXR .exr file as (height, width, 4) float32 linear RGBA."""
    lib = load()
    err = C.create_string_buffer(512)
    w, h = C.c_uint32(), C.c_uint32()
    rc = lib.ptw_read_image_rgba(str(path).encode(), None, 0, C.byref(w), C.byref(h), err, len(err))
    if rc != abi.PT_OK:
        raise PathTracerError(rc, f"{path}: {err.value.decode(errors="replace")}")
    out = np.empty((h.value, w.value, 4), np.float32)
    rc = lib.ptw_read_image_rgba(str(path).encode(), out.ctypes.data, out.size, C.byref(w), C.byref(h), err, len(err))
    if rc != abi.PT_OK:
        raise PathTracerError(rc, f"{path}: {err.value.decode(errors="replace")}")
    return out


def write_image(path, rgb: np.ndarray) -> None:
    """Save (height, width, 3) uint8 pixels as .png, .jpg/.jpeg, .webp (lossless) or .ppm."""
    a = np.ascontiguousarray(rgb, dtype=np.uint8)
    err = C.create_string_buffer(512)
    rc = load().ptw_write_image(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0], err, len(err))
    if rc != abi.PT_OK:
        raise PathTracerError(rc, err.value.decode(errors="replace"))


def decode_texture(data: bytes) -> np.ndarray:
    """A PNG or JPEG image in memory as (height, width, 4) uint8 RGBA, converted as the glTF importer does."""
    lib = load()
    err = C.create_string_buffer(512)
    w, h = C.c_uint32(), C.c_uint32()
    buf = C.create_string_buffer(bytes(data), len(data))
    rc = lib.ptw_decode_texture_rgba8(buf, len(data), None, 0, C.byref(w), C.byref(h), err, len(err))
    if rc != abi.PT_OK:
        raise PathTracerError(rc, err.value.decode(errors="replace"))
    out = np.empty((h.value, w.value, 4), np.uint8)
    rc = lib.ptw_decode_texture_rgba8(buf, len(data), out.ctypes.data, out.size, C.byref(w), C.byref(h), err, len(err))
    if rc != abi.PT_OK:
        raise PathTracerError(rc, err.value.decode(errors="replace"))
    return out


def build_bvh(triangles: np.ndarray):
    """Binned SAH BVH of world.rs:1430-1591 over (n, 9) float32 triangles -> (nodes (m, 8) uint32, order)."""
    t = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
    n = t.shape[0]
    nodes = np.zeros((max(1, 2 * n - 1), 8), dtype=np.uint32)
    order = np.zeros(n, dtype=np.uint32)
    m = load().ptw_build_bvh(t.ctypes.data, n, nodes.ctypes.data, order.ctypes.data)
    return nodes[:m].copy(), order


@dataclass
class KernelTimes:
    launches: dict
    milliseconds: dict


class PathTracer:
    """GPU trace pass for one tile (src/render/path_tracer.rs)."""

    DEFAULT_MAX_BOUNCES = abi.PT_DEFAULT_MAX_BOUNCES
    MAX_BOUNCES_LIMIT = abi.PT_MAX_BOUNCES_LIMIT
    MAX_SAMPLES_PER_TRACE = abi.PT_MAX_SAMPLES_PER_TRACE

    def __init__(self, updates: abi.WorldUpdates, tile_size, device: int = 0):
        self._lib = load()
        h = C.c_void_p()
        rc = self._lib.pt_create(device, C.byref(updates), int(tile_size[0]), int(tile_size[1]), C.byref(h))
        if rc != abi.PT_OK:
            raise PathTracerError(rc, "pt_create failed (see stderr)")
        self._h = h
        self.tile_size = (int(tile_size[0]), int(tile_size[1]))

    def _check(self, rc: int) -> None:
        if rc != abi.PT_OK:
            raise PathTracerError(rc, self._lib.pt_last_error(self._h).decode(errors="replace"))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pt_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def apply_updates(self, updates: abi.WorldUpdates) -> None:
        self._check(self._lib.pt_apply_updates(self._h, C.byref(updates)))

    def set_tile(self, image_size, origin, size) -> None:
        a = (C.c_uint32 * 2)(*image_size)
        o = (C.c_uint32 * 2)(*origin)
        s = (C.c_uint32 * 2)(*size)
        self._check(self._lib.pt_set_tile(self._h, a, o, s))
        self.tile_size = (int(size[0]), int(size[1]))

    def set_max_bounces(self, n: int) -> None:
        self._check(self._lib.pt_set_max_bounces(self._h, n))

    def max_bounces(self) -> int:
        return self._lib.pt_max_bounces(self._h)

    def sample_count(self) -> int:
        return self._lib.pt_sample_count(self._h)

    def set_kernel(self, kernel: int) -> None:
        self._check(self._lib.pt_set_kernel(self._h, kernel))

    def set_precision(self, flags: int) -> None:
        """PT_PRECISION_* bits (wide BVH, FP16/BF16 attributes, Kahan); resets the accumulation."""
        self._check(self._lib.pt_set_precision(self._h, flags))

    def precision(self) -> int:
        return self._lib.pt_precision(self._h)

    def precision_active(self) -> int:
        return self._lib.pt_precision_active(self._h)

    def trace(self, sample_count: int) -> int:
        traced = C.c_uint32()
        self._check(self._lib.pt_trace(self._h, sample_count, C.byref(traced)))
        return traced.value

    def trace_recorded(self, sample_count: int) -> np.ndarray:
        n = min(sample_count, self.MAX_SAMPLES_PER_TRACE)
        tw, th = self.tile_size
        recs = (abi.PathRecord * (n * tw * th))()
        traced = C.c_uint32()
        self._check(self._lib.pt_trace_recorded(self._h, sample_count, C.byref(traced), C.addressof(recs)))
        return records_to_numpy(recs, traced.value * tw * th)

    def trace_counted(self, sample_count: int, totals: dict | None = None) -> tuple[int, dict]:
        """pt_trace_counted: returns (samples traced, totals dict added into `totals`)."""
        arr = (C.c_uint64 * len(abi.COUNT_FIELDS))()
        traced = C.c_uint32()
        self._check(self._lib.pt_trace_counted(self._h, sample_count, C.byref(traced), arr))
        out = dict(totals) if totals else {k: 0 for k in abi.COUNT_FIELDS}
        for k, v in zip(abi.COUNT_FIELDS, arr):
            out[k] = out.get(k, 0) + int(v)
        return traced.value, out

    def render_fp64(self, sample_first: int, sample_count: int) -> np.ndarray:
        """FP64 reference render of the current tile (pt_render_fp64): per-pixel radiance sums over
        samples sample_first .. sample_first + sample_count - 1, shape (tile_h, tile_w, 3) float64."""
        tw, th = self.tile_size
        out = np.zeros((th, tw, 3), dtype=np.float64)
        self._check(self._lib.pt_render_fp64(self._h, sample_first, sample_count, out.ctypes.data))
        return out

    def synchronize(self, timeout_ms: int = 0) -> None:
        self._check(self._lib.pt_synchronize(self._h, timeout_ms))

    def read_tile(self, which: int = abi.PT_TILE_IMAGE) -> np.ndarray:
        tw, th = self.tile_size
        out = np.empty((th, tw, 4), dtype=np.float32)
        self._check(self._lib.pt_read_tile(self._h, which, out.ctypes.data))
        return out

    def display_tile(self) -> np.ndarray:
        tw, th = self.tile_size
        out = np.empty((th, tw, 4), dtype=np.uint8)
        self._check(self._lib.pt_display_tile(self._h, out.ctypes.data))
        return out

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(self._lib.pt_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def set_profiling(self, enabled: bool) -> None:
        self._check(self._lib.pt_set_profiling(self._h, 1 if enabled else 0))

    def kernel_times(self) -> KernelTimes:
        n = (C.c_uint64 * abi.PT_KERNEL_CLASS_COUNT)()
        ms = (C.c_double * abi.PT_KERNEL_CLASS_COUNT)()
        self._check(self._lib.pt_get_kernel_times(self._h, n, ms))
        return KernelTimes(dict(zip(abi.KERNEL_CLASSES, list(n))), dict(zip(abi.KERNEL_CLASSES, list(ms))))

    def reset_kernel_times(self) -> None:
        self._check(self._lib.pt_reset_kernel_times(self._h))

    def launch_count(self) -> int:
        return self._lib.pt_launch_count(self._h)

    def debug_intersect(self, origins, directions, t_max=None, records: bool = True):
        """Closest hits of opaque rays -> (hit, t, records or None).  Without records and with
        PT_PRECISION_WIDE_BVH selected the rays traverse the 8-wide BVH."""
        o = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(directions, dtype=np.float32).reshape(-1, 3)
        n = o.shape[0]
        tm = np.full(n, np.finfo(np.float32).max, dtype=np.float32) if t_max is None else np.ascontiguousarray(t_max, np.float32)
        hit = np.empty(n, dtype=np.int32)
        ht = np.empty(n, dtype=np.float32)
        recs = (abi.PathRecord * max(1, n))() if records else None
        self._check(self._lib.pt_debug_intersect(self._h, n, o.ctypes.data, d.ctypes.data, tm.ctypes.data,
                                                 hit.ctypes.data, ht.ctypes.data,
                                                 C.addressof(recs) if records else None))
        return hit, ht, (records_to_numpy(recs, n) if records else None)


RECORD_DTYPE = np.dtype([("visit_hash", "<u8"), ("hit", "<i4", (abi.PT_RECORD_MAX_BOUNCES,)),
                         ("extend_rays", "<u4"), ("shadow_rays", "<u4"), ("interior_visits", "<u4"),
                         ("leaf_visits", "<u4"), ("triangle_tests", "<u4"), ("shadow_interior_visits", "<u4"),
                         ("shadow_leaf_visits", "<u4"), ("shadow_triangle_tests", "<u4"), ("rand_draws", "<u4"),
                         ("hits", "<u4"), ("sky_misses", "<u4"), ("light_samples", "<u4"),
                         ("sky_light_samples", "<u4"), ("radiance", "<f4", (3,)), ("pad", "<u4")])
assert RECORD_DTYPE.itemsize == 144


def records_to_numpy(recs, count: int) -> np.ndarray:
    return np.frombuffer(bytes(recs), dtype=RECORD_DTYPE)[:count].copy()


def render_tiles(tracer: PathTracer, width: int, height: int, samples: int, tile_size: int) -> np.ndarray:
    """headless::render_tiles (headless.rs:207-285): every tile row-major, all
    samples, then the display tonemap; returns (height, width, 3) uint8."""
    tile = (min(tile_size, width), min(tile_size, height))
    out = np.zeros((height, width, 3), dtype=np.uint8)
    for y in range(0, height, tile[1]):
        for x in range(0, width, tile[0]):
            vis = (min(tile[0], width - x), min(tile[1], height - y))
            tracer.set_tile((width, height), (x, y), tile)
            remaining = samples
            while remaining > 0:
                remaining -= tracer.trace(remaining)
            rgba = tracer.display_tile()
            out[y:y + vis[1], x:x + vis[0]] = rgba[:vis[1], :vis[0], :3]
    return out


__all__ = ["World", "PathTracer", "PathTracerError", "render_tiles", "default_material", "alias_table",
           "build_bvh", "abi", "load", "RECORD_DTYPE"]
