"""pt_trace_noalloc: tracing for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc themselves or let a library call it for
them: a host application whose allocator owns all device memory and hands its
plug-ins ready-made buffers, or a latency-critical render thread that must not
hit the device-wide synchronisation of cudaMalloc / cudaFree.  For them the
library offers pt_trace_noalloc: the caller passes the world and the tile
buffers as its own device memory, and the library works in a fixed static
scratch array instead of allocating.

These tests play such a caller.  The caller's device memory is allocated here
with torch, standing in for the host application's allocator; the entry point
itself allocates nothing.  Two calls in a row must give exactly the bits that
pt_trace, the existing entry point, gives for the same samples.  The file
sorts last so that a run stopping at the first failure has already run every
other test.
"""
import ctypes as C

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi
from worlds import non_opaque_world

pytestmark = pytest.mark.gpu


def device_copy(torch, ptr, nbytes, keep):
    """Copy nbytes of host memory at ptr into caller-owned device memory."""
    host = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(max(nbytes, 1),)).copy()
    dev = torch.from_numpy(host).to("cuda")
    keep.append(dev)
    return dev.data_ptr()


def device_world(torch, updates, keep):
    s = updates.scene.contents
    k = updates.skybox.contents
    dw = abi.DeviceWorld()
    dw.geometries = device_copy(torch, s.geometries, 36 * s.triangle_count, keep)
    dw.attributes = device_copy(torch, s.attributes, 112 * s.triangle_count, keep)
    dw.triangle_count = s.triangle_count
    dw.materials = device_copy(torch, s.materials, 224 * s.material_count, keep)
    dw.material_count = s.material_count
    dw.bvh_nodes = device_copy(torch, s.bvh_nodes, 32 * s.node_count, keep)
    dw.node_count = s.node_count
    dw.skybox_rgba = device_copy(torch, k.rgba, 16 * k.uniforms.width * k.uniforms.height, keep)
    if k.alias_count:
        dw.skybox_aliases = device_copy(torch, k.alias_table, 12 * k.alias_count, keep)
    if updates.scene_alias_count:
        dw.scene_aliases = device_copy(torch, updates.scene_alias_table, 16 * updates.scene_alias_count, keep)
    dw.camera = updates.camera.contents
    dw.scene_uniforms = updates.scene_uniforms.contents
    dw.skybox_uniforms = updates.skybox_uniforms.contents
    mats = [s.materials[i] for i in range(s.material_count)]
    dw.any_non_opaque = int(any(m.alpha_mode != abi.PT_ALPHA_MODE_OPAQUE for m in mats))
    return dw


def noalloc(lib, dw, image, origin, tile, max_bounces, done, samples, accum, out):
    params = abi.TraceParameters()
    params.image_size[:] = image
    params.tile_origin[:] = origin
    params.max_bounces = max_bounces
    params.sample_count = done
    err = C.create_string_buffer(256)
    rc = lib.pt_trace_noalloc(C.byref(dw), C.byref(params), tile[0], tile[1], samples, accum.data_ptr(),
                              out.data_ptr(), None, err, len(err))
    return rc, err.value.decode()


@pytest.mark.parametrize("scene", ["cornell", "procedural", "non_opaque"])
def test_noalloc_matches_pt_trace_on_two_calls_in_a_row(scene):
    """Opaque worlds run the wavefront kernels with a separate shadow stage; the non-opaque one (BLEND
    and MASK materials, whose any-hit tests draw random numbers in the caller's triangle and material
    buffers) traces its shadow rays inline."""
    torch = pytest.importorskip("torch")
    lib = pt.load()
    if scene == "cornell":
        world = pt.World.cornell_box()
        image, origin, tile, bounces, spp = (256, 256), (64, 32), (128, 128), 8, 4
    elif scene == "procedural":
        world = pt.World.procedural(grid_x=128, grid_z=64, boxes=100, spheres=10, sphere_subdivision=3,
                                    emissive_triangles=16, skybox_width=256, skybox_height=128)
        image, origin, tile, bounces, spp = (640, 360), (290, 150), (100, 80), 8, 3
    else:
        world = non_opaque_world()
        image, origin, tile, bounces, spp = (200, 200), (40, 60), (96, 96), 6, 4
    world.set_aspect_ratio(image[0] / image[1])
    updates = world.take_updates()
    mats = [updates.scene.contents.materials[i] for i in range(updates.scene.contents.material_count)]
    assert any(m.alpha_mode != abi.PT_ALPHA_MODE_OPAQUE for m in mats) == (scene == "non_opaque")

    # the existing entry point
    tracer = pt.PathTracer(updates, tile)
    tracer.set_kernel(abi.PT_KERNEL_WAVEFRONT)
    tracer.set_max_bounces(bounces)
    tracer.set_tile(image, origin, tile)
    want = []
    for _ in range(2):
        assert tracer.trace(spp) == spp
        want.append((tracer.read_tile(abi.PT_TILE_ACCUMULATION), tracer.read_tile(abi.PT_TILE_IMAGE)))
    tracer.close()

    # the caller's own device memory
    keep = []
    dw = device_world(torch, updates, keep)
    accum = torch.full((tile[1], tile[0], 4), float("nan"), dtype=torch.float32, device="cuda")
    out = torch.zeros((tile[1], tile[0], 4), dtype=torch.float32, device="cuda")
    vis = (min(tile[0], image[0] - origin[0]), min(tile[1], image[1] - origin[1]))
    for call in range(2):
        rc, msg = noalloc(lib, dw, image, origin, tile, bounces, call * spp, spp, accum, out)
        assert rc == abi.PT_OK, msg
        torch.cuda.synchronize()
        got_acc = accum.cpu().numpy()[:vis[1], :vis[0]]
        got_img = out.cpu().numpy()[:vis[1], :vis[0]]
        np.testing.assert_array_equal(got_acc.view(np.uint32), want[call][0][:vis[1], :vis[0]].view(np.uint32))
        np.testing.assert_array_equal(got_img.view(np.uint32), want[call][1][:vis[1], :vis[0]].view(np.uint32))
    assert float(out.max()) > 0.0


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = pt.load()
    world = pt.World.cornell_box()
    updates = world.take_updates()
    keep = []
    dw = device_world(torch, updates, keep)
    tile = (512, 512)
    accum = torch.zeros((tile[1], tile[0], 4), dtype=torch.float32, device="cuda")
    out = torch.zeros_like(accum)
    # 512 x 512 x 1 = 262144 paths fits, one more sample does not
    rc, msg = noalloc(lib, dw, (512, 512), (0, 0), tile, 2, 0, 1, accum, out)
    assert rc == abi.PT_OK, msg
    rc, msg = noalloc(lib, dw, (512, 512), (0, 0), tile, 2, 1, 2, accum, out)
    assert rc == abi.PT_ERR_OUT_OF_LIMITS and "262144" in msg
    # a request whose paths would wrap a 64-bit product (2^40 pixels x 2^24 samples) is refused on the host
    # before anything is launched (the small buffers are never touched)
    side = 1 << 20
    rc, msg = noalloc(lib, dw, (side, side), (0, 0), (side, side), 2, 0, 1 << 24, accum, out)
    assert rc == abi.PT_ERR_OUT_OF_LIMITS and "262144" in msg
    torch.cuda.synchronize()


def test_noalloc_rejects_unaligned_nodes_on_the_host():
    # the nodes are read in place with 32-byte loads: a 16-byte aligned array is refused before any launch
    torch = pytest.importorskip("torch")
    lib = pt.load()
    world = pt.World.cornell_box()
    updates = world.take_updates()
    keep = []
    dw = device_world(torch, updates, keep)
    s = updates.scene.contents
    host = np.ctypeslib.as_array(C.cast(s.bvh_nodes, C.POINTER(C.c_uint8)), shape=(32 * s.node_count,)).copy()
    shifted = torch.zeros(32 * s.node_count + 16, dtype=torch.uint8, device="cuda")
    shifted[16:] = torch.from_numpy(host).to("cuda")
    keep.append(shifted)
    dw.bvh_nodes = shifted.data_ptr() + 16
    accum = torch.zeros((8, 8, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros_like(accum)
    rc, msg = noalloc(lib, dw, (8, 8), (0, 0), (8, 8), 2, 0, 1, accum, out)
    assert rc == abi.PT_ERR_INVALID_ARG and "32-byte aligned" in msg
    torch.cuda.synchronize()


def test_noalloc_reads_attributes_at_any_alignment():
    # the caller's attribute records may start at any 4-byte boundary: 16-byte pieces are read only from
    # a 16-byte aligned array, others are read by fields, with the same bits as pt_trace
    torch = pytest.importorskip("torch")
    lib = pt.load()
    world = pt.World.cornell_box()
    image, origin, tile, bounces, spp = (128, 128), (16, 24), (64, 64), 8, 2
    world.set_aspect_ratio(1.0)
    updates = world.take_updates()
    tracer = pt.PathTracer(updates, tile)
    tracer.set_kernel(abi.PT_KERNEL_WAVEFRONT)
    tracer.set_max_bounces(bounces)
    tracer.set_tile(image, origin, tile)
    assert tracer.trace(spp) == spp
    want = tracer.read_tile(abi.PT_TILE_ACCUMULATION)
    tracer.close()
    keep = []
    dw = device_world(torch, updates, keep)
    s = updates.scene.contents
    host = np.ctypeslib.as_array(C.cast(s.attributes, C.POINTER(C.c_uint8)), shape=(112 * s.triangle_count,)).copy()
    shifted = torch.zeros(112 * s.triangle_count + 16, dtype=torch.uint8, device="cuda")
    shifted[4:4 + host.size] = torch.from_numpy(host).to("cuda")
    keep.append(shifted)
    dw.attributes = shifted.data_ptr() + 4
    accum = torch.zeros((tile[1], tile[0], 4), dtype=torch.float32, device="cuda")
    out = torch.zeros_like(accum)
    rc, msg = noalloc(lib, dw, image, origin, tile, bounces, 0, spp, accum, out)
    assert rc == abi.PT_OK, msg
    torch.cuda.synchronize()
    np.testing.assert_array_equal(accum.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert float(out.max()) > 0.0
