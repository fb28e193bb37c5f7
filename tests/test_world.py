"""World builder (path-tracer_gb300/csrc/world.cpp) against the independent
restatement in oracle/world_ref.py and the golden fixtures."""
import hashlib
import json
import math
from pathlib import Path

import numpy as np
import pytest

import pathtracer as pt
from oracle import world_ref

GOLDEN = Path(__file__).resolve().parent / "golden"


def soup(seed, n):
    rng = np.random.default_rng(seed)
    centers = rng.uniform(-10, 10, (n, 1, 3))
    offsets = rng.normal(0, 0.5, (n, 3, 3))
    return (centers + offsets).reshape(n, 9).astype(np.float32)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_cornell_bvh_matches_golden_node_for_node():
    g = json.loads((GOLDEN / "bvh.json").read_text())["cornell"]
    tris = np.array(g["triangles"], dtype=np.uint32).view(np.float32).reshape(-1, 9)
    nodes, order = pt.build_bvh(tris)
    np.testing.assert_array_equal(nodes, np.array(g["nodes"], dtype=np.uint32))
    np.testing.assert_array_equal(order, np.array(g["order"], dtype=np.uint32))


@pytest.mark.parametrize("seed,n", [(7, 300), (11, 2000)])
def test_soup_bvh_matches_golden(seed, n):
    g = json.loads((GOLDEN / "bvh.json").read_text())[f"soup_{seed}_{n}"]
    nodes, order = pt.build_bvh(soup(seed, n))
    assert nodes.shape[0] == g["node_count"]
    assert digest(nodes) == g["nodes_sha256"]
    assert digest(order) == g["order_sha256"]


@pytest.mark.parametrize("seed,n", [(1, 3), (2, 17), (3, 150), (4, 700)])
def test_bvh_matches_python_restatement(seed, n):
    t = soup(seed, n)
    if seed == 4:  # degenerate axes: all centroids share z
        t[:, 2::3] = 1.0
    nodes, order = pt.build_bvh(t)
    ref_nodes, ref_order = world_ref.build_bvh(t)
    np.testing.assert_array_equal(nodes, world_ref.nodes_as_u32(ref_nodes))
    np.testing.assert_array_equal(order, ref_order)


def test_bvh_invariants_on_cornell():
    w = pt.World.cornell_box()
    nodes = w.bvh_nodes()
    geo = w.geometries()
    assert w.triangle_count() == 36
    lo = nodes[:, 0:3].view(np.float32)
    hi = nodes[:, 4:7].view(np.float32)
    leaves = nodes[:, 7] > 0
    covered = np.zeros(36, dtype=int)
    for i in np.nonzero(leaves)[0]:
        a, c = nodes[i, 3], nodes[i, 7]
        assert 1 <= c <= 36
        covered[a:a + c] += 1
        tri = geo[a:a + c].reshape(-1, 3, 3)
        assert (tri.min(axis=(0, 1)) >= lo[i]).all() and (tri.max(axis=(0, 1)) <= hi[i]).all()
    assert (covered == 1).all()
    for i in np.nonzero(~leaves)[0]:
        l = nodes[i, 3]
        assert l % 2 == 1  # children allocated pairwise after the root
        for ch in (l, l + 1):
            assert (lo[ch] >= lo[i]).all() and (hi[ch] <= hi[i]).all()
    assert w.bvh_max_depth() <= 64


def test_alias_tables_match_golden_and_restatement():
    for case in json.loads((GOLDEN / "alias.json").read_text()):
        got = pt.alias_table(case["weights"])
        want = case["entries"]
        assert len(got) == len(want)
        for (t, a, p), e in zip(want, got):
            assert np.float32(t) == e["threshold"] and a == e["alias_index"] and np.float32(p) == e["selection_probability"]
        ref = world_ref.alias_table(case["weights"])
        assert [(float(t), a, float(p)) for t, a, p in ref] == [(float(t), a, float(p)) for t, a, p in want]


def test_alias_table_samples_proportionally():
    w = np.array([1.0, 0.0, 3.0, 6.0])
    e = pt.alias_table(w)
    probs = np.zeros(4)
    for i, row in enumerate(e):
        probs[i] += row["threshold"] / 4
        probs[row["alias_index"]] += (1 - row["threshold"]) / 4
    np.testing.assert_allclose(probs, w / w.sum(), atol=1e-7)
    assert len(pt.alias_table([0.0, 0.0])) == 0


def test_cornell_lights_and_camera():
    w = pt.World.cornell_box()
    w.set_aspect_ratio(1.0)
    u = w.take_updates()
    s = u.scene_uniforms.contents
    assert s.emissive_triangles_count == 2
    # flux = 2 pi * area * luminance(17, 12, 4); the lamp is 0.25 x 0.25
    lum = 17 * 0.2126 + 12 * 0.7152 + 4 * 0.0722
    assert s.total_luminous_flux == pytest.approx(2 * math.pi * 0.0625 * lum, rel=1e-6)
    assert list(s.light_probabilities) == [1.0, 0.0]  # black skybox
    k = u.skybox.contents
    assert (k.uniforms.width, k.uniforms.height, k.alias_count) == (1, 1, 0)
    assert u.skybox_uniforms.contents.total_luminous_flux == 0.0
    cam = u.camera.contents
    # auto camera, world.rs:2178-2193: (cx, cy, max.z + 0.6 * max(dx, dy)), looking -Z, fov 90 degrees
    assert list(cam.position)[:3] == pytest.approx([0.5, 0.5, 1.6])
    assert list(cam.lower_left_corner_minus_position)[:3] == pytest.approx([-1, 1, -1], rel=1e-6)
    assert list(cam.horizontal)[:3] == pytest.approx([2, 0, 0], rel=1e-6)
    assert list(cam.vertical)[:3] == pytest.approx([0, -2, 0], rel=1e-6)
    alias = np.ctypeslib.as_array(u.scene_alias_table, shape=(2,))
    assert u.scene_alias_count == 2 and u.reset_accumulation == 1


def test_take_updates_change_tracking():
    w = pt.World.cornell_box()
    u = w.take_updates()
    assert u.scene and u.skybox and u.camera and u.reset_accumulation
    u = w.take_updates()  # nothing pending
    assert not u.scene and not u.skybox and not u.camera and not u.reset_accumulation
    w.edit_camera(yaw=0.3)
    u = w.take_updates()
    assert u.camera and not u.scene and u.reset_accumulation
    w.edit_skybox_average_luminance(5.0)
    u = w.take_updates()
    assert u.skybox_uniforms and u.skybox_uniforms.contents.average_luminance == 5.0 and u.reset_accumulation
    m = w.materials()[3]
    m.emission_color_and_luminance[3] = 2.0
    w.edit_material(3, m)
    u = w.take_updates()
    assert u.material_update_count == 1 and u.scene_alias_table and u.scene_uniforms
    assert u.scene_uniforms.contents.total_luminous_flux == pytest.approx(2 * 2 * math.pi * 0.0625 * (17 * 0.2126 + 12 * 0.7152 + 4 * 0.0722), rel=1e-6)
    bad = w.materials()[0]
    bad.base_weight = float("nan")
    with pytest.raises(pt.PathTracerError):
        w.edit_material(0, bad)


def test_skybox_normalisation_and_probabilities():
    w = pt.World.cornell_box()
    sky = np.zeros((8, 16, 4), np.float32)
    sky[..., :3] = 2.0
    sky[1, 3, :3] = 50.0
    w.set_skybox_rgba(sky)
    u = w.take_updates()
    k = u.skybox.contents
    rgba = np.ctypeslib.as_array(k.rgba, shape=(8 * 16 * 4,)).reshape(8, 16, 4)
    # solid-angle-weighted mean luminance of the normalised sky is 1
    rows = np.array([math.cos(y * math.pi / 8) - math.cos((y + 1) * math.pi / 8) for y in range(8)])
    lum = (rgba[..., :3].astype(np.float64) * [0.2126, 0.7152, 0.0722]).sum(-1)
    assert (lum * rows[:, None]).sum() / 32 == pytest.approx(1.0, rel=1e-6)
    assert k.alias_count == 128
    s = u.scene_uniforms.contents
    sky_flux = u.skybox_uniforms.contents.total_luminous_flux
    want = world_ref.light_probabilities(s.total_luminous_flux, s.emissive_triangles_count, sky_flux)
    assert tuple(s.light_probabilities) == tuple(float(x) for x in want)
    assert sum(s.light_probabilities) == pytest.approx(1.0)


def test_procedural_scene_small():
    w = pt.World.procedural(grid_x=32, grid_z=16, boxes=20, spheres=3, sphere_subdivision=2,
                            emissive_triangles=5, skybox_width=64, skybox_height=32)
    assert w.triangle_count() == 32 * 16 * 2 + 20 * 12 + 3 * 320 + 5
    assert w.bvh_max_depth() <= 64
    u = w.take_updates()
    s = u.scene_uniforms.contents
    assert s.emissive_triangles_count == 5
    assert 0 < s.light_probabilities[0] < 1 and 0 < s.light_probabilities[1] < 1
    # deterministic: same seed, same bytes
    w2 = pt.World.procedural(grid_x=32, grid_z=16, boxes=20, spheres=3, sphere_subdivision=2,
                             emissive_triangles=5, skybox_width=64, skybox_height=32)
    np.testing.assert_array_equal(w.geometries(), w2.geometries())
    np.testing.assert_array_equal(w.bvh_nodes(), w2.bvh_nodes())


def test_edit_emission_scale():
    # World::edit_emission_scale (world.rs:655-692)
    w = pt.World.cornell_box()
    mats = w.materials()
    emissive = [i for i, m in enumerate(mats) if m.emission_weight > 0 and max(m.emission_color_and_luminance[:3]) > 0]
    assert emissive and w.emission_scale() == 1.0
    w.take_updates()
    w.edit_emission_scale(3.0)
    u = w.take_updates()
    assert u.material_update_count == len(emissive) and u.reset_accumulation == 1
    for k in range(u.material_update_count):
        upd = u.materials[k]
        assert upd.index in emissive
        assert upd.material.emission_color_and_luminance[3] == np.float32(mats[upd.index].emission_color_and_luminance[3] * 3.0)
    # an individual edit of the strength is overwritten by the next scale; scale 1 restores the built value
    m = w.materials()[emissive[0]]
    m.emission_color_and_luminance[3] = 123.0
    w.edit_material(emissive[0], m)
    w.edit_emission_scale(1.0)
    u = w.take_updates()
    assert w.materials()[emissive[0]].emission_color_and_luminance[3] == mats[emissive[0]].emission_color_and_luminance[3]
    w.edit_emission_scale(-2.0)  # clamped at 0
    assert w.emission_scale() == 0.0
    u = w.take_updates()
    assert all(w.materials()[i].emission_color_and_luminance[3] == 0.0 for i in emissive)
    w.close()


def test_scene_and_skybox_from_bytes(tmp_path):
    from test_gltf import MATERIAL, write_gltf
    from test_image_io import random_planes, write_exr
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [MATERIAL], binary=True)
    a = pt.World.from_gltf(path)
    b = pt.World.from_gltf_bytes(path.read_bytes())
    np.testing.assert_array_equal(a.geometries(), b.geometries())
    rng = np.random.default_rng(2)
    write_exr(tmp_path / "sky.exr", random_planes(rng, 16, 32, {"R": "half", "G": "half", "B": "half"}), 3)
    a.set_skybox_file(tmp_path / "sky.exr")
    b.set_skybox_bytes((tmp_path / "sky.exr").read_bytes())
    ua, ub = a.take_updates(), b.take_updates()
    n = 16 * 32 * 4
    np.testing.assert_array_equal(np.ctypeslib.as_array(ua.skybox.contents.rgba, (n,)),
                                  np.ctypeslib.as_array(ub.skybox.contents.rgba, (n,)))
    with pytest.raises(pt.PathTracerError):
        b.set_skybox_bytes(b"not an image")
    with pytest.raises(pt.PathTracerError):
        pt.World.from_gltf_bytes(b"glTF\x02\x00\x00\x00\x0c\x00\x00\x00")
    a.close()
    b.close()
