"""The oracle's shading math against a second, independent restatement of the
shader (tests/shading_ref.py, numpy, FP64) on random inputs.

* FP64 oracle vs numpy: both are double-precision readings of the same
  shader lines, so they must agree to rounding (a mis-read formula, a wrong
  constant, a swapped argument or a different number or order of random
  draws shows at once, far above 1e-11).
* FP32 oracle (the parity mode, whose bits the CUDA kernels reproduce) vs
  numpy FP64: within FP32 rounding for nearly every point; a small fraction
  may take a different discrete decision (a VNDF sample landing on the
  horizon, `wi.z <= 0`, is dropped in one precision and kept in the other).

Functions: estimate_e_dielectric, the OpenPBR setup, evaluate_lobes and BSDF
sampling (trace.slang:229-411, 1097-1260), and sample_light with the
triangle and skybox pdfs (trace.slang:467-592).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import pathtracer as pt
from pathtracer import abi
import shading_ref as R

N = 100_000


def hemisphere(rng, n, min_z=0.02):
    v = rng.normal(size=(n, 3))
    v[:, 2] = np.abs(v[:, 2]) + min_z
    return v / np.linalg.norm(v, axis=1, keepdims=True)


@pytest.fixture(scope="module")
def shading():
    rng = np.random.default_rng(2024)
    c = np.zeros(N, oracle.SHADE_CASE)
    c["base_color"] = rng.uniform(0, 1, (N, 3))
    c["base_weight"] = rng.uniform(0, 1, N)
    c["base_metalness"] = np.where(rng.random(N) < 0.3, 1.0, rng.uniform(0, 1, N))
    c["base_diffuse_roughness"] = np.where(rng.random(N) < 0.1, 0.0, rng.uniform(0, 1, N))
    c["specular_color"] = rng.uniform(0, 1, (N, 3))
    c["specular_weight"] = rng.uniform(0, 1, N)
    c["specular_roughness"] = rng.uniform(0.02, 1, N)
    c["specular_anisotropy"] = np.where(rng.random(N) < 0.5, 0.0, rng.uniform(0, 1, N))
    c["specular_ior"] = rng.uniform(1.0, 3.0, N)
    c["wo"] = hemisphere(rng, N)
    c["wi"] = hemisphere(rng, N)
    c["rng"] = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32) | 1
    f64 = lambda k: c[k].astype(np.float64)  # noqa: E731
    draws = R.Rng(c["rng"])
    b = R.Bsdf(draws, f64("base_color"), f64("base_weight"), f64("base_metalness"), f64("base_diffuse_roughness"),
               f64("specular_color"), f64("specular_weight"), f64("specular_roughness"), f64("specular_anisotropy"),
               f64("specular_ior"), f64("wo"))
    f, pdf = b.evaluate(f64("wi"))
    ws = b.sample(draws)
    sf, spdf = b.evaluate(ws)
    ref = {"e_dielectric": b.e_dielectric, "p_ggx": b.p_ggx, "p_u": b.p_u, "f": f, "pdf": pdf, "sampled_wi": ws,
           "sampled_f": sf, "sampled_pdf": spdf, "rng_after": draws.s}
    return c, ref, oracle.shade_cases(c, 64), oracle.shade_cases(c, 32)


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


@pytest.mark.parametrize("key", ["e_dielectric", "p_ggx", "p_u", "f", "pdf", "sampled_wi", "sampled_f",
                                 "sampled_pdf"])
def test_fp64_oracle_equals_independent_restatement(shading, key):
    _, ref, o64, _ = shading
    assert np.isfinite(ref[key]).all()
    if key == "sampled_wi":
        np.testing.assert_allclose(o64[key], ref[key], rtol=0, atol=1e-11)
    elif key in ("f", "sampled_f"):  # the EON single-scatter term can cancel to ~1e-7: absolute slack there
        np.testing.assert_allclose(o64[key], ref[key], rtol=1e-11, atol=1e-12)
    else:
        np.testing.assert_allclose(o64[key], ref[key], rtol=1e-11, atol=1e-300)


def test_fp64_oracle_draws_the_same_random_numbers(shading):
    _, ref, o64, o32 = shading
    np.testing.assert_array_equal(o64["rng_after"], ref["rng_after"])  # 32 + 3 draws per shading point
    np.testing.assert_array_equal(o32["rng_after"], ref["rng_after"])


@pytest.mark.parametrize("key,typical,rare", [("f", 1e-6, 1e-4), ("pdf", 1e-6, 1e-4), ("e_dielectric", 1e-6, 1e-3),
                                              ("p_ggx", 1e-6, 1e-4), ("sampled_pdf", 1e-6, 1e-3)])
def test_fp32_parity_mode_within_fp32_rounding(shading, key, typical, rare):
    """Median error a few FP32 ulps; at most 1 in 1000 points beyond `rare` (decision flips)."""
    _, ref, _, o32 = shading
    err = rel(o32[key], ref[key])
    if err.ndim > 1:
        err = err.max(axis=1)
    assert np.median(err) < typical
    assert np.mean(err > rare) < 1e-3, (key, float(np.mean(err > rare)))


def light_world(updates) -> R.LightWorld:
    s = updates.scene.contents
    k = updates.skybox.contents
    n = s.triangle_count
    geo = np.ctypeslib.as_array(C.cast(s.geometries, C.POINTER(C.c_float)), shape=(n * 9,))
    attr = np.ctypeslib.as_array(C.cast(s.attributes, C.POINTER(C.c_uint8)), shape=(n * 112,)).reshape(n, 112)
    mat_index = attr[:, 0:4].copy().view(np.uint32).ravel()
    uv = attr[:, 40:64].copy().view(np.float32).reshape(n, 6)
    mats = [s.materials[i] for i in range(s.material_count)]
    assert all(m.alpha_mode == abi.PT_ALPHA_MODE_OPAQUE and m.emission_tex_layer < 0 for m in mats)
    erg = np.array([list(m.emission_color_and_luminance)[:3] for m in mats], np.float64)
    elum = np.array([m.emission_color_and_luminance[3] for m in mats], np.float64)
    ew = np.array([m.emission_weight for m in mats], np.float64)
    alias_dt = np.dtype([("threshold", "<f4"), ("alias_index", "<u4"), ("triangle_index", "<u4"),
                         ("selection_probability", "<f4")])
    live = updates.scene_uniforms.contents.emissive_triangles_count
    alias = np.ctypeslib.as_array(C.cast(updates.scene_alias_table, C.POINTER(C.c_uint8)),
                                  shape=(max(updates.scene_alias_count, 1) * 16,)).view(alias_dt)[:live].copy()
    W, H = k.uniforms.width, k.uniforms.height
    sky = np.ctypeslib.as_array(k.rgba, shape=(W * H * 4,)).reshape(H, W, 4).copy()
    sky_dt = np.dtype([("threshold", "<f4"), ("alias_index", "<u4"), ("selection_probability", "<f4")])
    sky_alias = (np.ctypeslib.as_array(C.cast(k.alias_table, C.POINTER(C.c_uint8)), shape=(k.alias_count * 12,))
                 .view(sky_dt).copy() if k.alias_count else np.zeros(1, sky_dt))
    su = updates.scene_uniforms.contents
    return R.LightWorld(geo, uv, (mat_index, erg, elum, ew), alias, list(su.light_probabilities), live, sky,
                        sky_alias, updates.skybox_uniforms.contents.average_luminance)


@pytest.fixture(scope="module", params=["cornell", "terrain"])
def lights(request):
    if request.param == "cornell":
        w = pt.World.cornell_box()  # one emissive quad, black sky: triangle lights only
        lo, hi = np.array([-0.45, 0.02, -0.45]), np.array([0.45, 0.9, 0.45])
    else:
        w = pt.World.procedural(grid_x=96, grid_z=48, boxes=60, spheres=6, sphere_subdivision=2,
                                emissive_triangles=24, skybox_width=128, skybox_height=64)
        lo, hi = np.array([-20.0, 0.5, -10.0]), np.array([20.0, 8.0, 10.0])
    u = w.take_updates()
    rng = np.random.default_rng(7)
    origins = rng.uniform(lo, hi, (N, 3)).astype(np.float32)
    states = rng.integers(0, 2 ** 32, N, dtype=np.uint64).astype(np.uint32) | 1
    ow = oracle.world_from_updates(u)
    lw = light_world(u)
    draws = R.Rng(states)
    d, dist, em, pdf, tri = lw.sample(origins.astype(np.float64), draws)
    ref = {"direction": d, "distance": dist, "emission": em, "pdf": pdf, "triangle_index": tri, "rng_after": draws.s}
    return request.param, w, ref, oracle.sample_lights(ow, origins, states, 64), oracle.sample_lights(ow, origins,
                                                                                                       states, 32)


def test_light_samples_fp64_equal(lights):
    name, _, ref, o64, _ = lights
    np.testing.assert_array_equal(o64["triangle_index"], ref["triangle_index"])
    np.testing.assert_array_equal(o64["rng_after"], ref["rng_after"])
    assert (ref["pdf"] > 0).mean() > 0.9
    if name == "terrain":  # both light categories are drawn
        assert 0.05 < (ref["triangle_index"] >= 0).mean() < 0.95
    for key in ("direction", "distance", "emission", "pdf"):
        np.testing.assert_allclose(o64[key], ref[key], rtol=1e-11, atol=1e-13, err_msg=key)


def test_light_samples_fp32_within_rounding(lights):
    _, _, ref, _, o32 = lights
    same = o32["triangle_index"] == ref["triangle_index"]
    assert same.mean() > 0.999  # an alias slot decided by a draw within rounding of the threshold may flip
    for key, typical, rare in (("direction", 1e-6, 1e-4), ("pdf", 1e-5, 1e-3), ("emission", 1e-6, 1e-3)):
        a, b = o32[key][same], ref[key][same]
        err = np.abs(a - b) / np.maximum(np.abs(b), 1e-20)  # exact zeros (a black sky) compare as 0
        if err.ndim > 1:
            err = err.max(axis=1)
        assert np.median(err) < typical, key
        assert np.mean(err > rare) < 1e-3, (key, float(np.mean(err > rare)))
