"""glTF 2.0 import (ptw_load_gltf): node transforms, the reference's LIFO node
order, attribute defaults, material conversion (world.rs:1992-2155) and the
refusals, texture images packed into atlas layers, on small files written
here (.gltf with a base64 buffer and .glb)."""
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


def write_gltf(tmp_path, nodes, scene_nodes, materials, binary=False, extra_prims=None, images=None, textures=None):
    """One mesh (the quad, indexed uint16, with normals and uvs) plus optional extra primitives.
    images: list of (encoded bytes, how) with how "view" (a buffer view), "data" (a data URI) or "file"."""
    pos, nor, uv, idx = quad()
    blobs = [pos.tobytes(), nor.tobytes(), uv.tobytes(), idx.tobytes() + b"\0\0"]
    views, accessors, off = [], [], 0
    specs = [(4, "VEC3", 5126), (4, "VEC3", 5126), (4, "VEC2", 5126), (6, "SCALAR", 5123)]
    for b, (count, typ, ctype) in zip(blobs, specs):
        views.append({"buffer": 0, "byteOffset": off, "byteLength": len(b)})
        accessors.append({"bufferView": len(views) - 1, "componentType": ctype, "count": count, "type": typ})
        off += len(b)
    image_docs = []
    for k, (enc, how) in enumerate(images or []):
        mime = "image/png" if enc[:4] == b"\x89PNG" else "image/jpeg"
        if how == "view":
            enc = enc + b"\0" * (-len(enc) % 4)
            blobs.append(enc)
            views.append({"buffer": 0, "byteOffset": off, "byteLength": len(enc)})
            off += len(enc)
            image_docs.append({"bufferView": len(views) - 1, "mimeType": mime})
        elif how == "data":
            image_docs.append({"uri": f"data:{mime};base64," + base64.b64encode(enc).decode()})
        else:
            (tmp_path / f"image{k}.bin").write_bytes(enc)
            image_docs.append({"uri": f"image{k}.bin"})
    prims = [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3, "material": 0}]
    prims += extra_prims or []
    data = b"".join(blobs)
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": scene_nodes}], "nodes": nodes,
           "meshes": [{"primitives": prims}], "materials": materials, "accessors": accessors,
           "bufferViews": views, "buffers": [{"byteLength": len(data)}]}
    if images:
        doc["images"] = image_docs
        doc["textures"] = textures if textures is not None else [{"source": i} for i in range(len(images))]
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
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [textured], images=[(b"GIF89a....", "view")])
    with pytest.raises(pt.PathTracerError, match="unsupported image encoding"):
        pt.World.from_gltf(path)
    (tmp_path / "bad.glb").write_bytes(b"glTF\x01\x00\x00\x00\x0c\x00\x00\x00")
    with pytest.raises(pt.PathTracerError, match="2.0"):
        pt.World.from_gltf(tmp_path / "bad.glb")
    (tmp_path / "broken.gltf").write_text("{\"asset\": {\"version\": \"2.0\"}, \"nodes\": [")
    with pytest.raises(pt.PathTracerError, match="JSON"):
        pt.World.from_gltf(tmp_path / "broken.gltf")
    with pytest.raises(pt.PathTracerError, match="cannot read"):
        pt.World.from_gltf(tmp_path / "missing.glb")


def _atlases(updates, srgb):
    sc = updates.scene.contents
    ptr, count = (sc.srgb_texture_atlases, sc.srgb_atlas_count) if srgb else (sc.linear_texture_atlases,
                                                                              sc.linear_atlas_count)
    n = abi.PT_ATLAS_SIZE
    return np.ctypeslib.as_array(ptr, (count * n * n * 4,)).reshape(count, n, n, 4) if count else None


@pytest.mark.parametrize("binary", [False, True])
def test_textures_into_atlases(tmp_path, binary):
    from test_texture_io import QUANT, _test_image, encode_jpeg, write_png
    rng = np.random.default_rng(8)
    img0 = write_png(rng.integers(0, 256, size=(30, 40, 3)), 2, 8)                  # base colour (sRGB)
    img1 = write_png(rng.integers(0, 65536, size=(16, 16, 4)), 6, 16)               # metallic-roughness (linear)
    img2, _ = encode_jpeg(_test_image(20, 24, 1)[..., 0], [(1, 1)], QUANT, grey=True)  # normal (linear)
    img3 = write_png(rng.integers(0, 256, size=(8, 12, 2)), 4, 8)                   # emission and specular factor
    img4 = write_png(rng.integers(0, 256, size=(5, 7, 1)), 0, 8)                    # used by no material
    mat = {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicRoughnessTexture": {"index": 1}},
           "normalTexture": {"index": 2, "scale": 0.5}, "emissiveTexture": {"index": 3},
           "extensions": {"KHR_materials_specular": {"specularTexture": {"index": 3}}}}
    hows = ["view", "data", "file", "view", "data"] if binary else ["data", "file", "data", "file", "data"]
    images = list(zip([img0, img1, img2, img3, img4], hows))
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [mat], binary, images=images)
    w = pt.World.from_gltf(path)
    m = w.materials()[0]
    u = w.take_updates()
    assert u.scene.contents.srgb_atlas_count == 1 and u.scene.contents.linear_atlas_count == 1
    srgb, linear = _atlases(u, True), _atlases(u, False)
    n = abi.PT_ATLAS_SIZE
    rects = {True: [], False: []}

    def check(layer, uv, enc, is_srgb):
        want = pt.decode_texture(enc)
        h, wd = want.shape[:2]
        assert layer == 0
        x, y = int(round(uv[0] * n)), int(round(uv[1] * n))
        assert list(uv) == [np.float32(x) / n, np.float32(y) / n, np.float32(wd) / n, np.float32(h) / n]
        atlas = srgb if is_srgb else linear
        np.testing.assert_array_equal(atlas[0, y:y + h, x:x + wd], want)
        rects[is_srgb].append((x, y, wd, h))

    check(m.base_color_tex_layer, m.base_color_uv, img0, True)
    check(m.metallic_roughness_tex_layer, m.metallic_roughness_uv, img1, False)
    check(m.normal_tex_layer, m.normal_uv, img2, False)
    check(m.emission_tex_layer, m.emission_uv, img3, True)
    # an image in the sRGB set is not in the linear atlases: the specular-factor slot has none
    assert m.specular_weight_tex_layer == -1 and list(m.specular_weight_uv) == [0, 0, 0, 0]
    assert m.specular_color_tex_layer == -1
    assert m.normal_scale == 0.5
    # the unused image went to the linear layer too, and no two placements overlap
    for r in rects.values():
        for i in range(len(r)):
            for j in range(i + 1, len(r)):
                a, b = r[i], r[j]
                assert a[0] + a[2] <= b[0] or b[0] + b[2] <= a[0] or a[1] + a[3] <= b[1] or b[1] + b[3] <= a[1]
    # 16-bit RGBA keeps the high bytes; grey-alpha becomes (l, a, 0, 255)
    d3 = pt.decode_texture(img3)
    assert (d3[..., 2] == 0).all() and (d3[..., 3] == 255).all()
    w.close()


def test_atlas_packing_opens_layers(tmp_path):
    # three 5000x5000 images cannot share an 8192^2 layer: one layer each; an image above 8192 is refused
    big = write_png_solid(5000, 5000)
    images = [(big, "data")] * 3
    mat = {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [mat], images=images)
    w = pt.World.from_gltf(path)
    u = w.take_updates()
    assert u.scene.contents.srgb_atlas_count == 1 and u.scene.contents.linear_atlas_count == 2
    w.close()
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [mat], images=[(write_png_solid(8193, 2), "data")])
    with pytest.raises(pt.PathTracerError, match="larger"):
        pt.World.from_gltf(path)


def write_png_solid(w, h):
    import zlib
    from test_texture_io import _chunk
    raw = (b"\0" + b"\x10\x20\x30" * w) * h
    return (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
            + _chunk(b"IDAT", zlib.compress(raw, 1)) + _chunk(b"IEND", b""))


def test_sparse_accessors(tmp_path):
    # POSITION with a sparse substitution of vertices 1 and 3, and a sparse-only (no bufferView) TEXCOORD_0
    pos, nor, uv, idx = quad()
    sp_idx = np.array([1, 3], np.uint16).tobytes()
    sp_pos = np.array([[2, 0, 0], [0, 3, 0]], np.float32).tobytes()
    sp_uv_idx = np.array([2], np.uint8).tobytes() + b"\0\0\0"
    sp_uv = np.array([[0.25, 0.75]], np.float32).tobytes()
    blobs = [pos.tobytes(), nor.tobytes(), idx.tobytes() + b"\0\0", sp_idx, sp_pos, sp_uv_idx, sp_uv]
    views, off = [], 0
    for b in blobs:
        views.append({"buffer": 0, "byteOffset": off, "byteLength": len(b)})
        off += len(b)
    accessors = [
        {"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3",
         "sparse": {"count": 2, "indices": {"bufferView": 3, "componentType": 5123},
                    "values": {"bufferView": 4}}},
        {"bufferView": 1, "componentType": 5126, "count": 4, "type": "VEC3"},
        {"bufferView": 2, "componentType": 5123, "count": 6, "type": "SCALAR"},
        {"componentType": 5126, "count": 4, "type": "VEC2",
         "sparse": {"count": 1, "indices": {"bufferView": 5, "componentType": 5121}, "values": {"bufferView": 6}}},
    ]
    data = b"".join(blobs)
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
           "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 3}, "indices": 2}]}],
           "accessors": accessors, "bufferViews": views,
           "buffers": [{"byteLength": len(data), "uri": "data:application/octet-stream;base64," +
                        base64.b64encode(data).decode()}]}
    path = tmp_path / "sparse.gltf"
    path.write_text(json.dumps(doc))
    w = pt.World.from_gltf(path)
    g = w.geometries()[np.argsort(w.bvh_order())].reshape(2, 3, 3)
    np.testing.assert_array_equal(g[0], [[0, 0, 0], [2, 0, 0], [1, 1, 0]])  # triangle (0, 1, 2)
    np.testing.assert_array_equal(g[1], [[0, 0, 0], [1, 1, 0], [0, 3, 0]])  # triangle (0, 2, 3)
    a = w.attributes_raw()[np.argsort(w.bvh_order())].view(np.float32).reshape(2, 28)
    np.testing.assert_array_equal(a[0, 10:16], [0, 0, 0, 0, 0.25, 0.75])  # uv of vertex 2 from the sparse values
    w.close()


def _edit_glb(path, edit):
    """Rewrite the JSON chunk of a .glb written by write_gltf through edit(doc)."""
    data = path.read_bytes()
    jl = struct.unpack("<I", data[12:16])[0]
    doc = json.loads(data[20:20 + jl])
    rest = data[20 + jl:]
    edit(doc)
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    body = struct.pack("<II", len(js), 0x4E4F534A) + js + rest
    path.write_bytes(struct.pack("<4sII", b"glTF", 2, 12 + len(body)) + body)


@pytest.mark.parametrize("field,value,message", [
    # a count no long can hold, a count far beyond any buffer, a negative count
    (("accessors", 1, "count"), 1e30, "count out of range"),
    (("accessors", 1, "count"), 2 ** 40, "count out of range"),
    (("accessors", 3, "count"), -5, "count out of range"),
    # a stride whose product with the count wraps 64 bits, and one the format does not allow
    (("bufferViews", 1, "byteStride"), 2 ** 60, "byteStride"),
    (("bufferViews", 1, "byteStride"), 6, "byteStride"),
    # offset + length past the end of the buffer without and with 64-bit wrap-around
    (("bufferViews", 2, "byteOffset"), 2 ** 62, "out of range"),
    (("bufferViews", 2, "byteLength"), 2 ** 63 - 1, "out of range"),
    (("bufferViews", 2, "byteOffset"), -8, "out of range"),
    # node indices that are not integers a long can hold
    (("scenes", 0, "nodes"), [1e300], "node out of range"),
])
def test_hostile_numbers_are_refused(tmp_path, field, value, message):
    """Accessor counts, strides, offsets and node indices taken from the file are checked before any
    allocation or read they would size: a hostile file gets an error, never a crash or a read outside
    the buffers (found by fuzzing the importer: a count of 1e30 once escaped as an exception)."""
    path = write_gltf(tmp_path, [{"mesh": 0}], [0], [{}], True)
    path.write_bytes(path.read_bytes())

    def edit(doc):
        obj = doc
        for k in field[:-1]:
            obj = obj[k]
        obj[field[-1]] = value
        if field[-1] == "byteStride":
            doc["accessors"][1]["count"] = 17  # with a 2^60 stride, 16 x stride wraps to 0

    _edit_glb(path, edit)
    with pytest.raises(pt.PathTracerError, match=message):
        pt.World.from_gltf(path)
