"""The C ABI: struct layouts, exported symbols, library loading (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import pathtracer as pt
from pathtracer import abi

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        for m in re.finditer(r"\b(pt[we]?_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_struct_sizes_match_reference_layouts():
    for struct, size in abi.STRUCT_SIZES.items():
        assert C.sizeof(struct) == size, struct.__name__


def test_field_offsets():
    assert abi.Material.alpha_mode.offset == 92
    assert abi.Material.base_color_uv.offset == 128
    assert abi.Material.specular_weight_uv.offset == 208
    assert abi.TriangleAttribute.t0.offset == 64
    assert abi.BvhNode.tri_count.offset == 28
    assert abi.EngineConfig.shade_threads.offset == 44
    assert abi.JobDesc.continue_job.offset == 88
    assert abi.EngineStats.gpu_ms.offset == 80 and abi.EngineStats.shade_threads.offset == 116
    dw = abi.DeviceWorld
    assert (dw.triangle_count.offset, dw.bvh_nodes.offset, dw.srgb_atlas_count.offset) == (16, 40, 64)
    assert (dw.linear_texture_atlases.offset, dw.skybox_rgba.offset, dw.camera.offset) == (72, 88, 112)
    assert (dw.scene_uniforms.offset, dw.skybox_uniforms.offset, dw.any_non_opaque.offset) == (176, 192, 208)


def test_library_exports_every_declared_symbol():
    lib = pt.load()
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # every declared entry point also has a ctypes signature
    assert names <= set(abi.SIGNATURES), sorted(names - set(abi.SIGNATURES))


def test_library_is_the_in_tree_build():
    assert abi.library_path().parent.name == "_build"
    assert abi.library_path().exists()


def test_create_rejects_missing_upload():
    lib = pt.load()
    h = C.c_void_p()
    u = abi.WorldUpdates()
    rc = lib.pt_create(0, C.byref(u), 8, 8, C.byref(h))
    assert rc != abi.PT_OK and not h.value


def test_world_errors_carry_messages():
    w = pt.World.empty()
    with pytest.raises(pt.PathTracerError) as e:
        w.build()
    assert e.value.code == abi.PT_ERR_INVALID_ARG
    assert "no triangles" in e.value.message
