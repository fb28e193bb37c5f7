"""Worlds built in code for tests that need materials the scene generators do not make."""
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
