"""Worlds built in code for tests that need materials the scene generators do not make."""
import ctypes as C

import numpy as np

import pathtracer as pt
from pathtracer import abi


def non_opaque_world():
    """Three screens of 8x8 quads in front of a floor, under an emissive quad and a gradient sky; the quads'
    materials cycle through BLEND at alpha 0.35 and 0.7, MASK at alpha 0.45 (cut out) and 0.55 (kept) with
    cutoff 0.5, and opaque.  The extend and shadow traversals draw one random number per BLEND candidate
    (trace.slang:446-454), so the wavefront kernels shade with inline shadow rays."""
    w = pt.World.empty()

    def material(rgb, mode=abi.PT_ALPHA_MODE_OPAQUE, alpha=1.0, emission=None):
        m = pt.default_material()
        m.base_color[:] = [*rgb, alpha]
        m.alpha_mode = mode
        m.alpha_cutoff = 0.5
        m.base_diffuse_roughness = 0.5
        if emission is not None:
            m.emission_color_and_luminance[:] = [*emission, 1.0]
            m.emission_weight = 1.0
        return w.add_material(m)

    def quad(c, du, dv, mi):
        c, du, dv = (np.asarray(v, np.float32) for v in (c, du, dv))
        pos = np.array([c - du - dv, c + du - dv, c + du + dv, c - du + dv], np.float32)
        uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
        w.add_mesh(pos, mi, uvs=uv, indices=[0, 1, 2, 0, 2, 3])

    cycle = [material((0.8, 0.3, 0.2), abi.PT_ALPHA_MODE_BLEND, 0.35),
             material((0.2, 0.7, 0.3), abi.PT_ALPHA_MODE_BLEND, 0.7),
             material((0.3, 0.3, 0.9), abi.PT_ALPHA_MODE_MASK, 0.45),
             material((0.9, 0.9, 0.2), abi.PT_ALPHA_MODE_MASK, 0.55),
             material((0.7, 0.7, 0.7))]
    quad((0, -1.2, 0), (4, 0, 0), (0, 0, 4), material((0.6, 0.6, 0.6)))
    quad((0, 2.5, 0), (0.6, 0, 0), (0, 0, 0.6), material((0, 0, 0), emission=(12.0, 10.0, 8.0)))
    k = 0
    for z in (-1.0, 0.0, 1.0):
        for iy in range(8):
            for ix in range(8):
                quad((-1.4 + 0.4 * ix + 0.1 * z, -1.0 + 0.3 * iy, z), (0.19, 0, 0), (0, 0.14, 0.02), cycle[k % 5])
                k += 1
    w.build()
    y = np.linspace(0.2, 1.0, 16, dtype=np.float32)[:, None, None]
    sky = np.concatenate([np.broadcast_to(y * np.array([0.5, 0.7, 1.0], np.float32), (16, 32, 3)),
                          np.ones((16, 32, 1), np.float32)], axis=2)
    w.set_skybox_rgba(sky)
    w.edit_skybox_average_luminance(1.0)
    w.set_aspect_ratio(1.0)
    w.edit_camera(position=(0.0, 0.2, 3.2), yaw=0.0, pitch=0.0, fov=1.2)
    return w


def sphere(center, radius, nu=48, nv=24):
    """UV sphere: positions, normals, UVs, tangents (+u direction, w = 1), indices."""
    j, i = np.mgrid[0:nv + 1, 0:nu + 1]
    th, ph = np.pi * j / nv, 2 * np.pi * i / nu
    n = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1).reshape(-1, 3)
    uv = np.stack([i / nu, j / nv], -1).reshape(-1, 2)
    t = np.stack([-np.sin(ph), np.zeros_like(ph), np.cos(ph), np.ones_like(ph)], -1).reshape(-1, 4)
    a = (j[:-1, :-1] * (nu + 1) + i[:-1, :-1]).ravel()
    b = a + nu + 1
    idx = np.stack([a, b, a + 1, a + 1, b, b + 1], -1).ravel()
    f = np.float32
    return (np.asarray(center, f) + radius * n).astype(f), n.astype(f), uv.astype(f), t.astype(f), idx


def material_zoo_world():
    """Spheres of OpenPBR materials the scene generators leave out, on a floor under an emissive quad and a
    gradient sky: anisotropic GGX metal, a tinted dielectric coat at IOR 2.4 over a half-weight base, a
    half metal, a sphere with a texture in every material slot (base colour, metallic-roughness, normal map
    at scale 0.7, emission, specular colour, specular weight), and an emitter at half emission weight with
    an emission texture.  Textures are 512^2 regions of one sRGB and one linear 8192^2 atlas layer."""
    lib = pt.load()
    w = pt.World.empty()
    size = 8192
    r = 512
    y, x = np.mgrid[0:r, 0:r]
    checker = ((x // 64 + y // 64) % 2).astype(np.float32)
    srgb = np.zeros((size, size, 4), np.uint8)
    srgb[0:r, 0:r] = np.stack([40 + 200 * checker, 60 + 150 * x / r, 90 + 120 * y / r, 255 + 0 * x], -1)
    srgb[0:r, r:2 * r] = np.stack([255 * checker, 180 + 0 * x, 255 * (1 - checker), 255 + 0 * x], -1)
    srgb[r:2 * r, 0:r] = np.stack([120 + 130 * x / r, 200 + 0 * x, 250 - 200 * y / r, 255 + 0 * x], -1)
    lin = np.zeros((size, size, 4), np.uint8)
    lin[0:r, 0:r] = np.stack([0 * x, 30 + 220 * x / r, 255 * checker, 255 + 0 * x], -1)
    bump = np.sin(x / 20.0) * np.cos(y / 27.0)
    lin[0:r, r:2 * r] = np.stack([128 + 70 * bump, 128 + 70 * np.cos(x / 13.0), 230 + 0 * x, 255 + 0 * x], -1)
    lin[r:2 * r, 0:r] = np.stack([0 * x, 0 * x, 0 * x, 40 + 215 * checker], -1)
    layers = []
    for is_srgb, img in ((1, srgb), (0, lin)):
        lay = C.c_int32()
        buf = np.ascontiguousarray(img.astype(np.uint8))
        rc = lib.ptw_add_atlas_layer(w.handle, is_srgb, buf.ctypes.data, C.byref(lay))
        assert rc == abi.PT_OK
        layers.append(lay.value)
    s = r / size

    def slot(col, row):
        return [col * s, row * s, s, s]

    def material(**fields):
        m = pt.default_material()
        m.base_color[:] = [0.8, 0.8, 0.8, 1.0]
        m.emission_color_and_luminance[:] = [0.0, 0.0, 0.0, 1.0]
        for k, v in fields.items():
            if k == "specular":
                m.specular_color_and_weight[:] = v
            elif k in ("base_color", "emission_color_and_luminance") or k.endswith("_uv"):
                getattr(m, k)[:] = v
            else:
                setattr(m, k, v)
        return w.add_material(m)

    zoo = [
        material(base_metalness=1.0, specular_roughness=0.4, specular_roughness_anisotropy=0.8,
                 specular=[1.0, 1.0, 1.0, 1.0], base_color=[0.9, 0.7, 0.5, 1.0]),
        material(base_metalness=0.0, base_weight=0.5, specular_ior=2.4, specular_roughness=0.15,
                 specular=[0.9, 0.6, 0.3, 0.7], base_color=[0.2, 0.4, 0.8, 1.0], base_diffuse_roughness=0.3),
        material(base_metalness=0.5, specular_roughness=0.2, base_diffuse_roughness=0.7,
                 specular=[1.0, 1.0, 1.0, 1.0], base_color=[0.7, 0.2, 0.2, 1.0]),
        material(base_metalness=1.0, specular_roughness=1.0, base_diffuse_roughness=0.5, normal_scale=0.7,
                 specular=[1.0, 1.0, 1.0, 1.0], base_color=[1.0, 1.0, 1.0, 1.0],
                 emission_color_and_luminance=[0.5, 0.4, 0.3, 1.0], emission_weight=1.0,
                 base_color_tex_layer=layers[0], base_color_uv=slot(0, 0),
                 emission_tex_layer=layers[0], emission_uv=slot(1, 0),
                 specular_color_tex_layer=layers[0], specular_color_uv=slot(0, 1),
                 metallic_roughness_tex_layer=layers[1], metallic_roughness_uv=slot(0, 0),
                 normal_tex_layer=layers[1], normal_uv=slot(1, 0),
                 specular_weight_tex_layer=layers[1], specular_weight_uv=slot(0, 1)),
        material(emission_color_and_luminance=[6.0, 5.0, 4.0, 1.0], emission_weight=0.5,
                 emission_tex_layer=layers[0], emission_uv=slot(1, 0), base_metalness=0.0),
    ]
    for k, mi in enumerate(zoo):
        pos, nor, uv, tan, idx = sphere((-2.0 + 1.0 * k, 0.0, 0.2 * (k % 2)), 0.42)
        w.add_mesh(pos, mi, normals=nor, uvs=uv, tangents=tan, indices=idx)
    floor = material(base_color=[0.5, 0.5, 0.5, 1.0], base_metalness=0.0, base_diffuse_roughness=1.0)
    w.add_mesh(np.array([[-4, -0.45, -3], [4, -0.45, -3], [4, -0.45, 3], [-4, -0.45, 3]], np.float32), floor,
               uvs=np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32), indices=[0, 2, 1, 0, 3, 2])
    lamp = material(emission_color_and_luminance=[10.0, 9.0, 8.0, 1.0], emission_weight=1.0, base_metalness=0.0)
    w.add_mesh(np.array([[-0.5, 2.5, -0.5], [0.5, 2.5, -0.5], [0.5, 2.5, 0.5], [-0.5, 2.5, 0.5]], np.float32),
               lamp, indices=[0, 1, 2, 0, 2, 3])
    w.build()
    yy = np.linspace(0.2, 1.0, 16, dtype=np.float32)[:, None, None]
    sky = np.concatenate([np.broadcast_to(yy * np.array([0.5, 0.7, 1.0], np.float32), (16, 32, 3)),
                          np.ones((16, 32, 1), np.float32)], axis=2)
    w.set_skybox_rgba(sky)
    w.edit_skybox_average_luminance(1.0)
    w.set_aspect_ratio(2.0)
    w.edit_camera(position=(0.0, 0.3, 3.0), yaw=0.0, pitch=-0.1, fov=1.1)
    return w
