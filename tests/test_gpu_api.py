"""Behaviour of the C ABI that mirrors path_tracer.rs / world_resources.rs,
including the host-side rejection of worlds that could make a kernel fault."""
import ctypes as C

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi

pytestmark = pytest.mark.gpu


@pytest.fixture
def tracer(cornell):
    _, updates, _ = cornell
    tr = pt.PathTracer(updates, (16, 16))
    yield tr
    tr.close()


def test_initial_parameters(tracer):
    # PathTracer::new, path_tracer.rs:232-239
    assert tracer.max_bounces() == abi.PT_DEFAULT_MAX_BOUNCES
    assert tracer.sample_count() == 0


def test_trace_caps_samples_per_call(tracer):
    assert tracer.trace(40) == abi.PT_MAX_SAMPLES_PER_TRACE
    assert tracer.sample_count() == 16
    assert tracer.trace(3) == 3
    assert tracer.sample_count() == 19
    assert tracer.trace(0) == 0


def test_set_tile_rules(tracer):
    tracer.trace(2)
    with pytest.raises(pt.PathTracerError) as e:
        tracer.set_tile((16, 16), (16, 0), (16, 16))
    assert e.value.code == abi.PT_ERR_INVALID_ARG and "origin" in e.value.message
    assert tracer.sample_count() == 2  # a rejected call changes nothing
    tracer.set_tile((64, 64), (16, 16), (16, 16))
    assert tracer.sample_count() == 0
    with pytest.raises(pt.PathTracerError) as e:
        tracer.set_tile((64, 64), (0, 0), (0, 16))
    assert e.value.code == abi.PT_ERR_OUT_OF_LIMITS
    with pytest.raises(pt.PathTracerError):
        tracer.set_tile((100000, 64), (0, 0), (20000, 16))


def test_max_bounces_rules(tracer):
    tracer.trace(1)
    tracer.set_max_bounces(abi.PT_DEFAULT_MAX_BOUNCES)
    assert tracer.sample_count() == 1  # unchanged value keeps accumulation
    tracer.set_max_bounces(3)
    assert tracer.sample_count() == 0
    with pytest.raises(pt.PathTracerError):
        tracer.set_max_bounces(17)


def test_apply_updates_reset(cornell):
    w = pt.World.cornell_box()
    tr = pt.PathTracer(w.take_updates(), (16, 16))
    tr.trace(4)
    first = tr.read_tile(abi.PT_TILE_ACCUMULATION)
    w.edit_camera(yaw=0.2)
    tr.apply_updates(w.take_updates())
    assert tr.sample_count() == 0
    tr.trace(4)
    assert not np.array_equal(first, tr.read_tile(abi.PT_TILE_ACCUMULATION))
    w.edit_camera(yaw=0.0)
    tr.apply_updates(w.take_updates())
    tr.trace(4)
    np.testing.assert_array_equal(first, tr.read_tile(abi.PT_TILE_ACCUMULATION))
    tr.close()


def _corrupt_updates(updates, field, value):
    """A copy of the scene upload with one BVH node field replaced."""
    s = updates.scene.contents
    nodes = (abi.BvhNode * s.node_count)()
    C.memmove(nodes, s.bvh_nodes, C.sizeof(nodes))
    setattr(nodes[0], field, value)
    scene = abi.SceneUpload.from_buffer_copy(s)
    scene.bvh_nodes = C.cast(nodes, C.POINTER(abi.BvhNode))
    u = abi.WorldUpdates.from_buffer_copy(updates)
    u.scene = C.pointer(scene)
    return u, (nodes, scene)


@pytest.mark.parametrize("field,value", [("left_first", 0), ("left_first", 10_000), ("tri_count", 1000)])
def test_malformed_bvh_rejected_on_host(cornell, field, value):
    _, updates, _ = cornell
    bad, keep = _corrupt_updates(updates, field, value)
    with pytest.raises(pt.PathTracerError):
        pt.PathTracer(bad, (8, 8))
    tr = pt.PathTracer(updates, (8, 8))
    tr.set_tile((256, 256), (120, 120), (8, 8))
    tr.trace(2)
    want = tr.read_tile(abi.PT_TILE_ACCUMULATION)
    with pytest.raises(pt.PathTracerError):
        tr.apply_updates(bad)
    # the rejected upload was staged, never made live: the same world renders the same bits
    tr.set_tile((256, 256), (120, 120), (8, 8))
    tr.trace(2)
    np.testing.assert_array_equal(tr.read_tile(abi.PT_TILE_ACCUMULATION).view(np.uint32), want.view(np.uint32))
    tr.apply_updates(updates)  # a valid full upload after a rejected one
    tr.set_tile((256, 256), (120, 120), (8, 8))
    tr.trace(2)
    np.testing.assert_array_equal(tr.read_tile(abi.PT_TILE_ACCUMULATION).view(np.uint32), want.view(np.uint32))
    tr.close()


def _scene_with_nodes(updates, nodes):
    s = updates.scene.contents
    scene = abi.SceneUpload.from_buffer_copy(s)
    scene.bvh_nodes = C.cast(nodes, C.POINTER(abi.BvhNode))
    scene.node_count = len(nodes)
    u = abi.WorldUpdates.from_buffer_copy(updates)
    u.scene = C.pointer(scene)
    return u, (nodes, scene)


def _chain_nodes(levels):
    """A degenerate tree: node 2k + 1 interior, node 2k + 2 a one-triangle leaf, `levels` deep."""
    nodes = (abi.BvhNode * (2 * levels + 1))()
    for i in range(len(nodes)):
        n = nodes[i]
        n.aabb_min[:] = (-1.0, -1.0, -1.0)
        n.aabb_max[:] = (1.0, 1.0, 1.0)
    for k in range(levels):
        i = 0 if k == 0 else 2 * k - 1
        nodes[i].left_first, nodes[i].tri_count = 2 * k + 1, 0
        nodes[2 * k + 2].left_first, nodes[2 * k + 2].tri_count = 0, 1
    last = 2 * levels - 1
    nodes[last].left_first, nodes[last].tri_count = 0, 1
    return nodes


def test_bvh_validation_messages(cornell):
    """Each malformed BVH is rejected with its own code and message, by the same checks whether the
    tree is in the builder's order (the forward pass) or not (the general walk)."""
    _, updates, _ = cornell
    s = updates.scene.contents
    tr = pt.PathTracer(updates, (8, 8))
    base = (abi.BvhNode * s.node_count)()
    C.memmove(base, s.bvh_nodes, C.sizeof(base))
    assert base[1].tri_count == 0 and base[2].tri_count == 0

    def expect(nodes, code, text):
        bad, keep = _scene_with_nodes(updates, nodes)
        with pytest.raises(pt.PathTracerError) as e:
            tr.apply_updates(bad)
        assert e.value.code == code and text in e.value.message, (e.value.code, e.value.message)

    twice = (abi.BvhNode * s.node_count)()
    C.memmove(twice, base, C.sizeof(base))
    twice[2].left_first = twice[1].left_first  # two parents for one child pair
    expect(twice, abi.PT_ERR_INVALID_ARG, "reached twice")
    leaf = (abi.BvhNode * s.node_count)()
    C.memmove(leaf, base, C.sizeof(base))
    leaf[1].tri_count, leaf[1].left_first = 5, s.triangle_count - 2
    expect(leaf, abi.PT_ERR_INVALID_ARG, "leaf triangle range")
    expect(_chain_nodes(70), abi.PT_ERR_OUT_OF_LIMITS, "deeper than the 64-entry")
    # 64 interior levels are accepted (a traversal defers at most one entry per level)
    tr.apply_updates(_scene_with_nodes(updates, _chain_nodes(64))[0])
    tr.apply_updates(updates)
    tr.close()


def test_skybox_alias_validation(cornell):
    w = pt.World.procedural(grid_x=16, grid_z=8, boxes=4, spheres=1, sphere_subdivision=1, emissive_triangles=2,
                            skybox_width=32, skybox_height=16)
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    tr = pt.PathTracer(u, (8, 8))
    k = u.skybox.contents
    assert k.alias_count == 32 * 16
    table = (abi.SkyboxAliasEntry * k.alias_count)()
    C.memmove(table, k.alias_table, C.sizeof(table))
    table[7].alias_index = k.alias_count
    sky = abi.SkyboxUpload.from_buffer_copy(k)
    sky.alias_table = C.cast(table, C.POINTER(abi.SkyboxAliasEntry))
    bad = abi.WorldUpdates.from_buffer_copy(u)
    bad.skybox = C.pointer(sky)
    with pytest.raises(pt.PathTracerError) as e:
        tr.apply_updates(bad)  # with the scene: the scan runs beside the BVH walk
    assert e.value.code == abi.PT_ERR_INVALID_ARG and "skybox alias index" in e.value.message
    bad.scene = None
    with pytest.raises(pt.PathTracerError) as e:
        tr.apply_updates(bad)  # skybox alone
    assert "skybox alias index" in e.value.message
    sky.alias_table = None
    with pytest.raises(pt.PathTracerError) as e:
        tr.apply_updates(bad)
    assert "alias table is NULL" in e.value.message
    tr.apply_updates(u)
    tr.close()


def test_inconsistent_lights_rejected(cornell):
    _, updates, _ = cornell
    u = abi.WorldUpdates.from_buffer_copy(updates)
    s = abi.SceneUniforms.from_buffer_copy(updates.scene_uniforms.contents)
    s.light_probabilities[0] = 0.5
    s.light_probabilities[1] = 0.5  # the black skybox has no alias table
    u.scene_uniforms = C.pointer(s)
    with pytest.raises(pt.PathTracerError) as e:
        pt.PathTracer(u, (8, 8))
    assert e.value.code == abi.PT_ERR_INVALID_ARG


def test_display_tile_matches_tonemap(tracer):
    tracer.trace(4)
    img = tracer.read_tile(abi.PT_TILE_IMAGE)[..., :3].astype(np.float64)
    a, b, c, d, e = 2.51, 0.03, 2.43, 0.59, 0.14
    m = np.clip((img * (a * img + b)) / (img * (c * img + d) + e), 0, 1)
    s = np.where(m > 0.0031308, np.power(m, 1 / 2.4) * 1.055 - 0.055, m * 12.92)
    want = np.floor(np.clip(s, 0, 1) * 255 + 0.5)
    got = tracer.display_tile()
    assert np.abs(got[..., :3].astype(int) - want).max() <= 1
    assert (got[..., 3] == 255).all()


def test_synchronize_and_profiling(tracer):
    tracer.set_profiling(True)
    tracer.set_kernel(abi.PT_KERNEL_PLAIN)
    tracer.trace(4)
    tracer.synchronize(timeout_ms=60000)
    times = tracer.kernel_times()
    assert times.launches["plain"] == 4 and times.milliseconds["plain"] > 0
    tracer.set_kernel(abi.PT_KERNEL_WAVEFRONT)
    tracer.trace(2)
    times = tracer.kernel_times()
    assert times.launches["extend"] == tracer.max_bounces() + 1 and times.launches["raygen"] == 1
    tracer.reset_kernel_times()
    assert tracer.kernel_times().launches["plain"] == 0
    assert tracer.launch_count() >= 4
    assert tracer.stream() != 0


def test_render_tiles_headless():
    # EXPOSURE (trace.slang:25) suits an 8000-nit sky: give the lamp the
    # reference box.glb's emissive strength (4e5) so the image is not black
    w = pt.World.cornell_box()
    w.set_aspect_ratio(100 / 60)
    m = w.materials()[3]
    m.emission_color_and_luminance[3] = 4.0e5
    w.edit_material(3, m)
    tr = pt.PathTracer(w.take_updates(), (48, 48))
    tr.set_max_bounces(3)
    rgb = pt.render_tiles(tr, 100, 60, 2, 48)
    assert rgb.shape == (60, 100, 3) and rgb.max() > 200 and rgb.min() == 0
    tr.close()
