"""glTF 2.0 import (ptw_load_gltf): node transforms, the reference's LIFO node
order, attribute defaults, material conversion (world.rs:1992-2155) and the
refusals, on small files written here (.gltf with a base64 buffer and .glb)."""
import base64
import json
import struct

import numpy as np
import pytest

import pathtracer as pt
from pathtracer import abi


def quad(z=0.0):
    pos = np.array([[0, 0, z], [1, 0, z], [1, 1, z], [0, 1, z]], np.float32)
    nor = np.array([[0, 0, 2]] * 4, np.float32)  # not unit: the import normalises after transforming
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    return pos, nor, uv, idx


def write_gltf(tmp_path, nodes, scene_nodes, materials, binary=False, extra_prims=None):
    """One mesh (the quad, indexed uint16, with normals and uvs) plus optional extra primitives."""
    pos, nor, uv, idx = quad()
    blobs = [pos.tobytes(), nor.tobytes(), uv.tobytes(), idx.tobytes() + b"\0\0"]
    views, accessors, off = [], [], 0
    specs = [(4, "VEC3", 5126), (4, "VEC3", 5126), (4, "VEC2", 5126), (6, "SCALAR", 5123)]
    for b, (count, typ, ctype) in zip(blobs, specs):
        views.append({"buffer": 0, "byteOffset": off, "byteLength": len(b)})
        accessors.append({"bufferView": len(views) - 1, "componentType": ctype, "count": count, "type": typ})
        off += len(b)
    prims = [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3, "material": 0}]
    prims += extra_prims or []
    data = b"".join(blobs)
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": scene_nodes}], "nodes": nodes,
           "meshes": [{"primitives": prims}], "materials": materials, "accessors": accessors,
           "bufferViews": views, "buffers": [{"byteLength": len(data)}]}
    if binary:
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        data += b"\0" * (-len(data) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(data), 0x004E4942) + data
        path = tmp_path / "scene.glb"
        path.write_bytes(struct.pack("<4sII", b"glTF", 2, 12 + len(body)) + body)
    else:
        doc["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(data).decode()
        path = tmp_path / "scene.gltf"
        path.write_text(json.dumps(doc))
    return path


MATERIAL = {"pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.25, 1.0, 1.0], "metallicFactor": 0.0,
                                     "roughnessFactor": 0.75},
            "emissiveFactor": [1.0, 0.5, 0.0],
            "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 40.0},
                           "KHR_materials_ior": {"ior": 1.33},
                           "KHR_materials_specular": {"specularFactor": 0.5, "specularColorFactor": [1, 0.5, 0.5]}},
            "alphaMode": "MASK", "alphaCutoff": 0.25,
            "extras": {"OpenPBR_specular_roughness": 0.6, "OpenPBR_base_weight": 2.0}}


@pytest.mark.parametrize("binary", [False, True])
def test_transforms_order_and_material(tmp_path, binary):
    # root 0 (translated, child 2 rotated 90 degrees about z and scaled), root 1 (matrix)
    s = np.sqrt(0.5)
    nodes = [{"translation": [10, 0, 0], "children": [2]},
             {"matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 5, 1], "mesh": 0},
             {"rotation": [0, 0, s, s], "scale": [2, 2, 2], "mesh": 0}]
    path = write_gltf(tmp_path, nodes, [0, 1], [MATERIAL], binary)
    w = pt.World.from_gltf(path, build=False)
    w.build()
    assert w.triangle_count() == 4
    g = w.geometries()[np.argsort(w.bvh_order())]  # intake order
    # the LIFO walk: root 1 (z = 5) first, then root 0, then its child (x' = 10 - 2y, y' = 2x)
    np.testing.assert_allclose(g[0].reshape(3, 3), [[0, 0, 5], [1, 0, 5], [1, 1, 5]], atol=1e-6)
    np.testing.assert_allclose(g[2].reshape(3, 3), [[10, 0, 0], [10, 2, 0], [8, 2, 0]], atol=1e-5)
    a = w.attributes_raw()[np.argsort(w.bvh_order())].view(np.float32).reshape(4, 28)
    np.testing.assert_allclose(a[:, 1:4], np.tile([0, 0, 1], (4, 1)), atol=1e-6)  # unit normals
    mats = w.materials()
    assert len(mats) == 1  # one glTF material, cached across both instances
    m = mats[0]
    np.testing.assert_allclose(list(m.base_color), [0.5, 0.25, 1.0, 1.0])
    assert m.base_metalness == 0.0 and m.base_diffuse_roughness == 0.75
    np.testing.assert_allclose(list(m.emission_color_and_luminance), [1.0, 0.5, 0.0, 40.0])
    np.testing.assert_allclose(list(m.specular_color_and_weight), [1.0, 0.5, 0.5, 0.5])
    assert abs(m.specular_ior - 1.33) < 1e-6 and abs(m.specular_roughness - 0.6) < 1e-6
    assert m.base_weight == 1.0  # out-of-range extras are ignored
    assert m.alpha_mode == abi.PT_ALPHA_MODE_MASK and m.alpha_cutoff == 0.25
    assert m.base_color_tex_layer == -1 and list(m.base_color_uv) == [0, 0, 0, 0]


def test_defaults_without_normals_uvs_or_material(tmp_path):
    # a non-indexed primitive with positions only: flat normals, the reference's dummy uvs, default material
    extra = [{"attributes": {"POSITION": 0}}]
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [MATERIAL], extra_prims=extra)
    # POSITION of 4 vertices is not a multiple of 3 without indices: refused
    with pytest.raises(pt.PathTracerError):
        pt.World.from_gltf(path)
    extra = [{"attributes": {"POSITION": 0}, "indices": 3}]
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [MATERIAL], extra_prims=extra)
    w = pt.World.from_gltf(path)
    assert w.triangle_count() == 4
    mats = w.materials()
    assert len(mats) == 2
    d = mats[1]  # glTF default material: white, metallic 1, roughness 1
    assert list(d.base_color) == [1, 1, 1, 1] and d.base_metalness == 1.0 and d.base_diffuse_roughness == 1.0
    a = w.attributes_raw()[np.argsort(w.bvh_order())].view(np.float32).reshape(4, 28)
    # without TEXCOORD_0 vertex i gets (0,0), (1,0), (0,1)[i % 3]: triangles (0,1,2) and (0,2,3)
    np.testing.assert_array_equal(a[2:, 10:16], [[0, 0, 1, 0, 0, 1], [0, 0, 0, 1, 0, 0]])


def test_refusals(tmp_path):
    textured = dict(MATERIAL, pbrMetallicRoughness={"baseColorTexture": {"index": 0}})
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [textured])
    with pytest.raises(pt.PathTracerError, match="textured"):
        pt.World.from_gltf(path)
    (tmp_path / "bad.glb").write_bytes(b"glTF\x01\x00\x00\x00\x0c\x00\x00\x00")
    with pytest.raises(pt.PathTracerError, match="2.0"):
        pt.World.from_gltf(tmp_path / "bad.glb")
    (tmp_path / "broken.gltf").write_text("{\"asset\": {\"version\": \"2.0\"}, \"nodes\": [")
    with pytest.raises(pt.PathTracerError, match="JSON"):
        pt.World.from_gltf(tmp_path / "broken.gltf")
    with pytest.raises(pt.PathTracerError, match="cannot read"):
        pt.World.from_gltf(tmp_path / "missing.glb")
