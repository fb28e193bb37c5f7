"""Seeded mutation fuzzing of the host-side decoders of untrusted files.

Valid PNG and JPEG textures, Radiance HDR and OpenEXR skyboxes (every
compression) and .glb scenes are written by the encoders of the other tests,
then damaged at random: flipped bits, overwritten bytes, truncations,
insertions, deletions, and 32-bit fields set to extreme values; for the
scenes also numbers, types and keys of the JSON document.  Every damaged
file must either decode or be refused with an error: a crash, an abort or an
exception escaping the C ABI fails the run.  The same generator under
AddressSanitizer (tens of thousands of cases per format) found one defect,
an accessor count of 1e30 in a glTF file; these few hundred cases per format
run with the CPU suite.
"""
import json
import random
import struct

import numpy as np
import pytest

import pathtracer as pt
from test_gltf import write_gltf
from test_image_io import random_planes, write_exr, write_hdr
from test_texture_io import QUANT, _test_image, encode_jpeg, write_png

CASES = 300


def mutate(r: random.Random, data: bytes) -> bytes:
    b = bytearray(data)
    if len(b) < 8:
        return bytes(b) + bytes(r.randrange(256) for _ in range(8))
    kind = r.randrange(6)
    if kind == 0:
        for _ in range(r.randint(1, 8)):
            i = r.randrange(len(b))
            b[i] ^= 1 << r.randrange(8)
    elif kind == 1:
        for _ in range(r.randint(1, 4)):
            b[r.randrange(len(b))] = r.choice([0, 0xff, 0x7f, 0x80, r.randrange(256)])
    elif kind == 2:
        b = b[: r.randrange(len(b))]
    elif kind == 3:
        i = r.randrange(len(b))
        b[i:i] = bytes(r.randrange(256) for _ in range(r.randint(1, 16)))
    elif kind == 4:
        i = r.randrange(len(b))
        del b[i:i + r.randint(1, 64)]
    else:
        i = r.randrange(max(1, len(b) - 4))
        v = r.choice([0, 1, 0x7fffffff, 0xffffffff, 0x10000, 0xffff, 0x80000000])
        b[i:i + 4] = v.to_bytes(4, r.choice(["little", "big"]))
    return bytes(b)


def texture_seeds():
    rng = np.random.default_rng(11)
    out = []
    for ctype, depth, ch in [(0, 8, 1), (2, 8, 3), (4, 8, 2), (6, 8, 4), (6, 16, 4), (0, 1, 1), (2, 16, 3)]:
        s = rng.integers(0, 1 << depth, size=(13, 17, ch))
        out += [write_png(s, ctype, depth), write_png(s, ctype, depth, interlace=True)]
    out.append(write_png(rng.integers(0, 4, size=(9, 11, 1)), 3, 8, palette=rng.integers(0, 256, size=(4, 3))))
    img = _test_image(24, 40, 3)
    for kw in (dict(), dict(progressive=True), dict(restart=2)):
        for sampling in ([(1, 1), (1, 1), (1, 1)], [(2, 2), (1, 1), (1, 1)]):
            out.append(encode_jpeg(img, sampling, QUANT, **kw)[0])
    return out


def skybox_seeds(tmp_path):
    rng = np.random.default_rng(12)
    out = []
    for rle in (False, True):
        px = np.zeros((9, 40, 4), np.uint8)
        px[..., :3] = rng.integers(0, 256, size=(9, 40, 3))
        px[..., 3] = rng.integers(120, 140, size=(9, 40))
        p = tmp_path / f"seed{int(rle)}.hdr"
        write_hdr(p, px, rle=rle)
        out.append((p.read_bytes(), ".hdr"))
    for comp in (0, 1, 2, 3, 4):  # NONE, RLE, ZIPS, ZIP, PIZ
        p = tmp_path / f"seed{comp}.exr"
        write_exr(p, random_planes(rng, 20, 33, {"B": "half", "G": "half", "R": "half"}), comp)
        out.append((p.read_bytes(), ".exr"))
    return out


def test_texture_decoders_survive_damaged_files():
    r = random.Random(5)
    seeds = texture_seeds()
    decoded = refused = 0
    for k in range(CASES):
        data = mutate(r, seeds[k % len(seeds)])
        if r.random() < 0.3:
            data = mutate(r, data)
        try:
            pt.decode_texture(data)
            decoded += 1
        except pt.PathTracerError:
            refused += 1
    assert decoded + refused == CASES and refused > 0


def test_skybox_decoders_survive_damaged_files(tmp_path):
    r = random.Random(6)
    seeds = skybox_seeds(tmp_path)
    decoded = refused = 0
    for k in range(CASES):
        data, ext = seeds[k % len(seeds)]
        data = mutate(r, data)
        path = tmp_path / f"case{k}{ext}"
        path.write_bytes(data)
        try:
            pt.read_image(path)
            decoded += 1
        except pt.PathTracerError:
            refused += 1
    assert decoded + refused == CASES and refused > 0


def _json_mutate(r: random.Random, doc):
    paths = []

    def walk(x, p):
        if isinstance(x, dict):
            for k, v in x.items():
                paths.append(p + [k])
                walk(v, p + [k])
        elif isinstance(x, list):
            for i, v in enumerate(x):
                paths.append(p + [i])
                walk(v, p + [i])

    walk(doc, [])
    for _ in range(r.randint(1, 3)):
        p = r.choice(paths)
        parent = doc
        try:
            for k in p[:-1]:
                parent = parent[k]
            k = p[-1]
            choice = r.randrange(6)
            if choice == 0:
                parent[k] = r.choice([-1, 0, 1, 3, 255, 65535, 2 ** 31 - 1, 2 ** 32 - 1, 2 ** 53, -2 ** 31, 1e30])
            elif choice == 1:
                parent[k] = r.choice([0.5, -0.5, 1e-30, -1e30])
            elif choice == 2:
                parent[k] = "x" * r.randint(0, 3)
            elif choice == 3:
                parent[k] = [] if r.random() < 0.5 else {}
            elif choice == 4:
                if isinstance(parent, dict):
                    del parent[k]
                else:
                    parent.pop(k)
            else:
                parent[k] = None
        except (KeyError, IndexError, TypeError):
            pass
    return doc


def test_gltf_import_survives_damaged_files(tmp_path):
    r = random.Random(7)
    png = write_png(np.random.default_rng(13).integers(0, 256, size=(8, 8, 3)), 2, 8)
    s2 = 0.7071
    configs = [
        ([{"mesh": 0}], [0], [{"pbrMetallicRoughness": {"baseColorFactor": [1, 0.5, 0.2, 1]}}], None),
        ([{"mesh": 0, "children": [1]}, {"mesh": 0, "rotation": [s2, 0, 0, s2], "translation": [1, 2, 3]}], [0],
         [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "metallicFactor": 0.5},
           "emissiveFactor": [1, 1, 1]}], [(png, "view")]),
    ]
    seeds = []
    for k, (nodes, roots, mats, images) in enumerate(configs):
        d = tmp_path / f"seed{k}"
        d.mkdir()
        seeds.append(write_gltf(d, nodes, roots, mats, True, images=images).read_bytes())
    loaded = refused = 0
    for k in range(CASES):
        data = seeds[k % len(seeds)]
        if r.random() < 0.7:
            jl = struct.unpack("<I", data[12:16])[0]
            doc = _json_mutate(r, json.loads(data[20:20 + jl]))
            js = json.dumps(doc).encode()
            js += b" " * (-len(js) % 4)
            body = struct.pack("<II", len(js), 0x4E4F534A) + js + data[20 + jl:]
            data = struct.pack("<4sII", b"glTF", 2, 12 + len(body)) + body
        else:
            data = mutate(r, data)
        path = tmp_path / f"case{k}.glb"
        path.write_bytes(data)
        try:
            pt.World.from_gltf(path, build=False).close()
            loaded += 1
        except pt.PathTracerError:
            refused += 1
    assert loaded + refused == CASES and refused > 0 and loaded > 0
