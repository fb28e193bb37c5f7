"""The Rust binding (include/pt_ffi.rs) against the C header it binds.

No Rust toolchain exists on the build machine, so the binding is checked by
parsing: every #[repr(C)] descriptor has the C struct's fields in the same
order with corresponding types, every extern "C" function exists in the
header with the same parameter types, the binding's compile-time size
assertions equal the C layouts (which pt_layout_check.cpp asserts in C and
the ctypes mirror measures here), and the marshalling fills every field of
pt_world_updates.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

from pathtracer import abi

ROOT = Path(__file__).resolve().parent.parent
RUST = (ROOT / "include" / "pt_ffi.rs").read_text()
HEADER = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "pt.h").read_text(), flags=re.S)
HEADER += re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "pt_precision.h").read_text(), flags=re.S)

# Rust type -> C type of the same layout (the reference's Gpu* structs are byte-identical to pt_*)
TYPES = {
    "u8": "uint8_t", "u32": "uint32_t", "u64": "uint64_t", "i32": "int32_t", "f32": "float", "c_char": "char",
    "usize": "size_t",
    "GpuTriangleGeometry": "pt_triangle_geometry", "GpuTriangleAttribute": "pt_triangle_attribute",
    "GpuBvhNode": "pt_bvh_node", "GpuMaterial": "pt_material", "GpuCamera": "pt_camera",
    "GpuSceneUniforms": "pt_scene_uniforms", "GpuSceneAliasEntry": "pt_scene_alias_entry",
    "GpuSkyboxUniforms": "pt_skybox_uniforms", "GpuSkyboxAliasEntry": "pt_skybox_alias_entry",
    "PtSceneUpload": "pt_scene_upload", "PtSkyboxUpload": "pt_skybox_upload",
    "PtMaterialUpdate": "pt_material_update", "PtWorldUpdates": "pt_world_updates", "PtCtx": "pt_ctx",
}
STRUCTS = {"PtSceneUpload": "pt_scene_upload", "PtSkyboxUpload": "pt_skybox_upload",
           "PtMaterialUpdate": "pt_material_update", "PtWorldUpdates": "pt_world_updates"}
CTYPES = {"pt_scene_upload": abi.SceneUpload, "pt_skybox_upload": abi.SkyboxUpload,
          "pt_material_update": abi.MaterialUpdate, "pt_world_updates": abi.WorldUpdates,
          "pt_material": abi.Material, "pt_camera": abi.Camera}


def rust_type(t: str) -> str:
    """'*const GpuMaterial' -> 'const pt_material*', '*mut u32' -> 'uint32_t*', 'u64' -> 'uint64_t'."""
    t = t.strip()
    m = re.fullmatch(r"\*(const|mut)\s+(\w+)", t)
    if m:
        base = TYPES[m.group(2)]
        return ("const " if m.group(1) == "const" else "") + base + "*"
    m = re.fullmatch(r"\*mut\s+\*mut\s+(\w+)", t)
    if m:
        return TYPES[m.group(1)] + "**"
    return TYPES[t]


def c_norm(t: str) -> str:
    t = re.sub(r"\s+", " ", t.replace(" *", "*")).strip()
    return re.sub(r"\bint\b", "int32_t", t)  # the header's plain int is 32-bit on every target


def c_struct_fields(name: str) -> list[tuple[str, str]]:
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", HEADER, re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m = re.fullmatch(r"(.*?)(\w+)", decl)
        out.append((m.group(2), c_norm(m.group(1))))
    return out


def rust_struct_fields(name: str) -> list[tuple[str, str]]:
    body = re.search(r"pub struct " + name + r" \{(.*?)\n\}", RUST, re.S).group(1)
    return [(f, rust_type(t)) for f, t in re.findall(r"pub (\w+): ([^,\n]+),", body)]


@pytest.mark.parametrize("rust,c", sorted(STRUCTS.items()))
def test_descriptors_match_the_header(rust, c):
    assert re.search(r"#\[repr\(C\)\]\s*pub struct " + rust + r"\b", RUST)
    assert rust_struct_fields(rust) == c_struct_fields(c)


def test_size_assertions_match_the_c_layouts():
    sizes = dict(re.findall(r"size_of::<(\w+)>\(\) == (\d+)", RUST))
    assert set(sizes) >= set(STRUCTS)
    for rust, n in sizes.items():
        assert C.sizeof(CTYPES[TYPES[rust]]) == int(n), rust
    layout = (ROOT / "path-tracer_gb300" / "csrc" / "pt_layout_check.cpp").read_text()
    for rust, c in STRUCTS.items():
        assert f"CHECK_SIZE({c}, {sizes[rust]});" in layout


def c_functions() -> dict[str, tuple[str, list[str]]]:
    out = {}
    for m in re.finditer(r"\n([\w\s\*]+?)\b(pt_\w+)\s*\(([^)]*)\)\s*;", HEADER):
        params = [p.strip() for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
        types = []
        for p in params:
            p = " ".join(p.split())
            arr = p.endswith("]")
            p = re.sub(r"\[\w*\]$", "", p)
            t = c_norm(re.fullmatch(r"(.*?)(\w+)", p).group(1))
            types.append(t + ("*" if arr else ""))
        out[m.group(2)] = (c_norm(m.group(1)), types)
    return out


def test_extern_functions_match_the_header():
    decls = re.search(r'extern "C" \{(.*?)\n\}', RUST, re.S).group(1)
    header = c_functions()
    found = 0
    for name, params, ret in re.findall(r"pub fn (\w+)\(([^)]*)\)(?:\s*->\s*([^;]+))?;", decls, re.S):
        assert name in header, name
        c_ret, c_params = header[name]
        rust_params = [rust_type(p.split(":", 1)[1]) for p in params.split(",") if p.strip()]
        # C array parameters (uint32_t image_size[2]) decay to pointers
        assert [t.replace("const uint32_t*", "uint32_t*") for t in rust_params] == \
            [t.replace("const uint32_t*", "uint32_t*") for t in c_params], name
        want_ret = "void" if not ret else rust_type(ret)
        assert c_ret.replace("const ", "") == want_ret.replace("const ", ""), name
        found += 1
    assert found >= 13


def test_marshalling_sets_every_field():
    """Marshalled::view fills every pt_world_updates field, null for None (no todo!() left)."""
    assert "todo!" not in RUST and "unimplemented!" not in RUST
    view = re.search(r"\n        PtWorldUpdates \{\n(.*?)\n        \}", RUST, re.S).group(1)
    assigned = re.findall(r"^\s*(\w+): ", view, re.M)
    assert assigned == [f for f, _ in c_struct_fields("pt_world_updates")]
    scene = re.search(r"m\.scene = Some\(PtSceneUpload \{(.*?)\}\);", RUST, re.S).group(1)
    assert re.findall(r"^\s*(\w+): ", scene, re.M) == [f for f, _ in c_struct_fields("pt_scene_upload")]
    assert "ptr::null()" in view or "opt_ptr" in view
