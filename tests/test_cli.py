"""The headless `pt-render render` command (the reference's `render`
subcommand, headless.rs:15-285): flag validation on the host, and on the GPU
an image equal to the one the library renders through the same tile loop
(render_tiles) for the built-in room and for a glTF scene under an OpenEXR
sky, written as PNG, lossless WebP or PPM that decode back to the same
bytes."""
import subprocess

import numpy as np
import pytest

import pathtracer as pt
from pathtracer.build import CLI


def run(*args, timeout=300):
    return subprocess.run([str(CLI), *args], capture_output=True, text=True, timeout=timeout)


@pytest.mark.parametrize("args,words", [
    ([], "expected the `render` command"),
    (["render", "--max-bounces", "17"], "--max-bounces"),
    (["render", "--camera-pitch", "91"], "--camera-pitch must be from -90 to 90"),
    (["render", "--camera-fov", "180"], "--camera-fov must be strictly between 0 and 180"),
    (["render", "--camera-position", "1,2"], "three comma-separated"),
    (["render", "--camera-yaw", "inf"], "must be finite"),
    (["render", "--skybox-luminance", "-1"], "nonnegative"),
    (["render", "--width", "0"], "--width"),
    (["render", "--samples", "-3"], "--samples"),
    (["render", "--output", "x.bmp"], "must have a .png, .jpg, .jpeg, or .webp extension"),
    (["render", "--frobnicate", "1"], "unknown flag"),
    (["render", "--scene"], "missing value"),
])
def test_flag_errors(args, words):
    r = run(*args)
    assert r.returncode == 2
    assert words in r.stderr and "usage: pt-render render" in r.stderr


def _png_rgb(path):
    return pt.decode_texture(path.read_bytes())[..., :3]


@pytest.mark.gpu
@pytest.mark.parametrize("ext", ["png", "webp"])
def test_cornell_render_matches_library(tmp_path, ext):
    out = tmp_path / f"room.{ext}"
    r = run("render", "--scene", "cornell", "--width", "72", "--height", "40", "--samples", "5",
            "--max-bounces", "3", "--tile-size", "32", "--camera-yaw", "10", "--output", str(out))
    assert r.returncode == 0, r.stderr
    w = pt.World.cornell_box()
    w.set_aspect_ratio(72 / 40)
    w.edit_skybox_average_luminance(8000.0)
    w.edit_camera(yaw=np.float32(10.0) * (np.float32(np.pi) / np.float32(180.0)))  # the command's float degrees
    tr = pt.PathTracer(w.take_updates(), (32, 32))
    tr.set_max_bounces(3)
    want = pt.render_tiles(tr, 72, 40, 5, 32)
    tr.close()
    if ext == "png":
        got = _png_rgb(out)
    else:
        from test_image_out import webp_pixels
        got = webp_pixels(out.read_bytes())
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
def test_gltf_scene_under_exr_sky(tmp_path):
    from test_gltf import write_gltf
    from test_image_io import random_planes, write_exr
    rng = np.random.default_rng(6)
    write_exr(tmp_path / "sky.exr", random_planes(rng, 32, 64, {"R": "half", "G": "half", "B": "half"}), 4,
              force=True)
    s2 = np.sqrt(0.5)
    nodes = [{"mesh": 0}, {"mesh": 0, "rotation": [s2, 0, 0, s2]}]
    mat = {"pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.5, 0.3, 1.0], "metallicFactor": 0.0}}
    scene = write_gltf(tmp_path, nodes, [0, 1], [mat], binary=True)
    out = tmp_path / "scene.ppm"
    r = run("render", "--scene", str(scene), "--skybox", str(tmp_path / "sky.exr"), "--skybox-luminance", "2",
            "--width", "48", "--height", "48", "--samples", "3", "--max-bounces", "4", "--tile-size", "48",
            "--output", str(out))
    assert r.returncode == 0, r.stderr
    data = out.read_bytes()
    assert data.startswith(b"P6\n48 48\n255\n")
    got = np.frombuffer(data[len(b"P6\n48 48\n255\n"):], np.uint8).reshape(48, 48, 3)
    w = pt.World.from_gltf(scene)
    w.set_skybox_file(tmp_path / "sky.exr")
    w.set_aspect_ratio(1.0)
    w.edit_skybox_average_luminance(2.0)
    tr = pt.PathTracer(w.take_updates(), (48, 48))
    tr.set_max_bounces(4)
    want = pt.render_tiles(tr, 48, 48, 3, 48)
    tr.close()
    np.testing.assert_array_equal(got, want)
    assert got.max() > 0
