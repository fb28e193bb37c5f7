"""A second, independent FP64 restatement of the shading math of
src/render/trace.slang, in numpy, vectorised over many shading points.

Written from the shader source, not from the oracle (oracle/trace_oracle.cpp)
or the kernels, so that the oracle's reading of the shader is checked by a
second reading: tests/test_shading_restatement.py compares the two on 10^5
random shading points.  Every quantity is float64; the shader's f32 literals
are widened exactly (F below), and the random numbers are the shader's own
f32 draws (rand, trace.slang:195-202), widened.

Covered: rand (195-202), fresnel_exact (330-341), ggx_lambda (347-352),
sample_VNDF (356-364), alpha_anisotropic (369-375), specular_ior_modulated
(379-391), estimate_e_dielectric (396-411), E_FON_exact (318-323),
evaluate_lobes (229-315), the OpenPBR setup of compute_main (1097-1181), BSDF
sampling (1212-1260) and sample_light with its skybox and triangle pdfs
(467-592).
"""
from __future__ import annotations

import numpy as np


def F(x: float) -> float:
    """An f32 literal of the shader, widened to float64 without rounding."""
    return float(np.float32(x))


PI = F(3.14159265359)
INV_PI = F(0.31830988618)
INV_2PI = F(0.15915494309189535)
TWO_PI = float(np.float32(2.0) * np.float32(3.14159265359))  # 2.0 * PI, folded in f32
FLT_MAX = float(np.finfo(np.float32).max)
ONE_BELOW_1 = float(np.uint32(0x3F7FFFFF).view(np.float32))  # asfloat(0x3f800000u - 1u)


# ------------------------------------------------------------------------ RNG

class Rng:
    """PCG-RXS-M-XS of rand(), one uint32 state per lane."""

    def __init__(self, states):
        self.s = np.asarray(states, dtype=np.uint32).copy()

    def __call__(self, mask=None) -> np.ndarray:
        """Draw for the lanes in `mask` (all lanes if None); other lanes keep their state, return 0."""
        with np.errstate(over="ignore"):
            s = (self.s * np.uint32(747796405) + np.uint32(2891336453)).astype(np.uint32)
            word = (((s >> ((s >> np.uint32(28)) + np.uint32(4))) ^ s) * np.uint32(277803737)).astype(np.uint32)
        bits = np.uint32(0x3F800000) | (((word >> np.uint32(22)) ^ word) >> np.uint32(9))
        f = bits.view(np.float32).astype(np.float64) - 1.0  # exact: the f32 subtraction of 1.0 is exact here
        if mask is None:
            self.s = s
            return f
        self.s = np.where(mask, s, self.s)
        return np.where(mask, f, 0.0)


# -------------------------------------------------------------------- vectors

def dot(a, b):
    return np.sum(a * b, axis=-1)


def normalize(v):
    return v / np.sqrt(dot(v, v))[..., None]


def reflect(i, n):
    return i - 2.0 * dot(n, i)[..., None] * n


def lerp(a, b, t):
    return a * (1.0 - t) + b * t


def saturate(x):
    return np.clip(x, 0.0, 1.0)


# ------------------------------------------------------------------ BSDF parts

def fresnel_exact(ior, cos_i):
    s = (1.0 - cos_i * cos_i) / (ior * ior)
    tir = s >= 1.0
    cos_t = np.sqrt(np.where(tir, 0.0, 1.0 - s))
    rs = (cos_i - ior * cos_t) / (cos_i + ior * cos_t)
    rp = (cos_t - ior * cos_i) / (cos_t + ior * cos_i)
    return np.where(tir, 1.0, 0.5 * (rs * rs + rp * rp))


def ggx_lambda(v, a):
    return 0.5 * np.sqrt(1.0 + (a[..., 0] ** 2 * v[..., 0] ** 2 + a[..., 1] ** 2 * v[..., 1] ** 2) / v[..., 2] ** 2) - 0.5


def sample_vndf(wo, a, r, two_pi_r):
    ww = normalize(np.stack([wo[..., 0] * a[..., 0], wo[..., 1] * a[..., 1], wo[..., 2]], -1))
    z = (1.0 - r) * (1.0 + ww[..., 2]) - ww[..., 2]
    sin_theta = np.sqrt(saturate(1.0 - z * z))
    h = np.stack([sin_theta * np.cos(two_pi_r), sin_theta * np.sin(two_pi_r), z], -1) + ww
    return normalize(np.stack([h[..., 0] * a[..., 0], h[..., 1] * a[..., 1], h[..., 2]], -1))


def alpha_anisotropic(roughness, anisotropy):
    iso = 1.0 - anisotropy
    at = roughness * roughness * F(1.41421356237) / np.sqrt(iso * iso + 1.0)
    return np.stack([np.maximum(at, F(1e-4)), np.maximum(at * iso, F(1e-4))], -1)


def specular_ior_modulated(ior, weight):
    f0 = (ior - 1.0) ** 2 / (ior + 1.0) ** 2
    f0s = np.sign(ior - 1.0) * np.sqrt(np.minimum(weight * f0, ONE_BELOW_1))
    return (1.0 + f0s) / (1.0 - f0s)


def estimate_e_dielectric(rng, wo, opl, alpha, ior_m, spec_color):
    total = np.zeros(wo.shape[:-1])
    for _ in range(16):
        r1 = rng()
        tpr = TWO_PI * rng()
        h = sample_vndf(wo, alpha, r1, tpr)
        wi = reflect(-wo, h)
        ok = wi[..., 2] > 0.0
        f = fresnel_exact(ior_m, dot(h, wo))
        with np.errstate(divide="ignore", invalid="ignore"):
            term = f * opl / (opl + ggx_lambda(wi, alpha))
        total += np.where(ok, term, 0.0)
    return spec_color * (total / 16.0)[..., None]


def e_fon_exact(mu, r):
    af = 1.0 / (F(0.28779340921) * r + 1.0)
    si = np.sqrt(1.0 - mu * mu)
    g = si * (np.arccos(mu) - si * mu) + F(float.fromhex("0x1.555556p-1")) * ((si / mu) * (1.0 - si ** 3) - si)
    return af + r * af * INV_PI * g


class Bsdf:
    """The per-shading-point state of compute_main (trace.slang:1097-1181)."""

    def __init__(self, rng, base_color, base_weight, metalness, diffuse_roughness, spec_color, spec_weight,
                 roughness, anisotropy, ior, wo):
        self.wo = wo
        self.alpha = alpha_anisotropic(roughness, anisotropy)
        self.ior_m = specular_ior_modulated(ior, spec_weight)
        self.f0 = base_weight[..., None] * base_color
        self.opl = 1.0 + ggx_lambda(wo, self.alpha)
        r, z = diffuse_roughness, wo[..., 2]
        self.ltc = np.stack([
            1.0 + r * (F(0.303392) + (F(-0.518982) + F(0.111709) * z) * z + (F(-0.276266) + F(0.335918) * z) * r),
            r * (F(-1.16407) + F(1.15859) * z + (F(0.150815) - F(0.150105) * z) * r) / (z ** 3 - F(1.43545)),
            1.0 + r * (F(0.20013) + (F(-0.506373) + F(0.261777) * z) * z),
            r * (F(0.540852) + (F(-1.01625) + F(0.475392) * z) * z) / (F(-1.0743) + (F(0.0725628) + z) * z)], -1)
        ls = wo[..., 0] ** 2 + wo[..., 1] ** 2
        safe = np.where(ls > 0.0, ls, 1.0)
        x = np.where((ls > 0.0)[..., None], np.stack([wo[..., 0], wo[..., 1], np.zeros_like(z)], -1)
                     / np.sqrt(safe)[..., None], np.array([1.0, 0.0, 0.0]))
        # float3x3(X, (-X.y, X.x, 0), (0, 0, 1)): rows of the LTC frame
        self.rows = np.stack([x, np.stack([-x[..., 1], x[..., 0], np.zeros_like(z)], -1),
                              np.broadcast_to(np.array([0.0, 0.0, 1.0]), x.shape)], -2)
        self.e_dielectric = estimate_e_dielectric(rng, wo, self.opl, self.alpha, self.ior_m, spec_color)
        luma = np.array([F(0.2126), F(0.7152), F(0.0722)])
        albedo_gloss = dot(self.e_dielectric, luma)
        albedo_diffuse = (1.0 - albedo_gloss) * base_weight * dot(base_color, luma)
        fsm = self.f0 + (1.0 - self.f0) * ((1.0 - z) ** 5)[..., None]
        w_ggx = lerp(albedo_gloss, dot(fsm, luma), metalness)
        w_diffuse = (1.0 - metalness) * albedo_diffuse
        self.p_ggx = np.clip(w_ggx / np.maximum(w_ggx + w_diffuse, F(1e-7)), F(0.1), F(0.9))
        self.p_diffuse = 1.0 - self.p_ggx
        self.p_u = r ** F(0.1) * (F(0.162925) + (F(-0.372058) + (F(0.538233) - F(0.290822) * z) * z) * z)
        self.p_c = 1.0 - self.p_u
        self.base_color, self.base_weight, self.metalness = base_color, base_weight, metalness
        self.r, self.spec_color, self.spec_weight = diffuse_roughness, spec_color, spec_weight

    def evaluate(self, wi):
        """evaluate_lobes (trace.slang:229-315): (f_total, pdf_total)."""
        wo, a = self.wo, self.alpha
        h = normalize(wo + wi)
        hw = dot(h, wo)
        g1 = 1.0 / self.opl
        g2 = 1.0 / (self.opl + ggx_lambda(wi, a))
        dh = h[..., 0] ** 2 / a[..., 0] ** 2 + h[..., 1] ** 2 / a[..., 1] ** 2 + h[..., 2] ** 2
        D = INV_PI / (a[..., 0] * a[..., 1] * dh * dh)
        ts = D * g2 / (4.0 * wi[..., 2] * wo[..., 2])
        omh = 1.0 - hw
        f0 = self.f0
        f82 = f0 - (omh ** 5)[..., None] * (
            (F(0.00105024005) * hw * omh)[..., None] * (1.0 - self.spec_color) * (9031.0 * f0 + 7776.0) + (f0 - 1.0))
        f_conductor = saturate(self.spec_weight[..., None] * f82) * ts[..., None]
        f_dielectric = self.spec_color * (fresnel_exact(self.ior_m, hw) * ts)[..., None]
        r = self.r
        s_f = wi[..., 0] * wo[..., 0] + wi[..., 1] * wo[..., 1]
        sovert = np.where(s_f > 0.0, s_f / np.maximum(wo[..., 2], wi[..., 2]), s_f)
        af = 1.0 / (F(0.28779340921) * r + 1.0)
        f_ss = self.base_color * (INV_PI * af * (r * sovert + 1.0))[..., None]
        efo, efi = e_fon_exact(wo[..., 2], r), e_fon_exact(wi[..., 2], r)
        avg = af * (F(0.07248821245) * r + 1.0)
        rho = self.base_color
        rho_ms = rho * rho * avg[..., None] / (1.0 - rho * (1.0 - avg)[..., None])
        f_ms = rho_ms * INV_PI * (np.maximum(F(1e-7), 1.0 - efo) * np.maximum(F(1e-7), 1.0 - efi)
                                  / np.maximum(F(1e-7), 1.0 - avg))[..., None]
        f_diffuse = self.base_weight[..., None] * (f_ss + f_ms)
        f_gd = f_dielectric + (1.0 - self.e_dielectric) * f_diffuse
        f_total = lerp(f_gd, f_conductor, self.metalness[..., None])
        pdf_ggx = D * g1 / (4.0 * wo[..., 2])
        wl = np.einsum("...ij,...j->...i", self.rows, wi)  # mul(basis, wi)
        la, lb, lc, ld = (self.ltc[..., k] for k in range(4))
        det = lc * (la - lb * ld)
        wh = np.stack([lc * (wl[..., 0] - lb * wl[..., 2]), (la - lb * ld) * wl[..., 1],
                       -lc * (ld * wl[..., 0] - la * wl[..., 2])], -1)
        len2 = dot(wh, wh)
        s_pdf = 0.5 / np.sqrt(ld * ld + 1.0) + 0.5
        pdf_c = det * det / (len2 * len2) * np.maximum(wh[..., 2], 0.0) / (PI * s_pdf)
        pdf_eon = self.p_u * F(0.15915494309) + self.p_c * pdf_c
        return f_total, self.p_ggx * pdf_ggx + self.p_diffuse * pdf_eon

    def sample(self, rng):
        """BSDF sampling (trace.slang:1212-1260): wi from the next three draws."""
        tpr = TWO_PI * rng()
        r1 = rng()
        use_ggx = rng() < self.p_ggx
        wo = self.wo
        ggx = reflect(-wo, sample_vndf(wo, self.alpha, r1, tpr))
        with np.errstate(divide="ignore", invalid="ignore"):
            u1 = r1 / self.p_u
            st = np.sqrt(1.0 - u1 * u1)
            uniform = np.stack([st * np.cos(tpr), st * np.sin(tpr), u1], -1)
            u1c = (r1 - self.p_u) / self.p_c
            la, lb, lc, ld = (self.ltc[..., k] for k in range(4))
            R = np.sqrt(u1c)
            y = R * np.sin(tpr)
            s = 0.5 / np.sqrt(ld * ld + 1.0) + 0.5
            x = -lerp(np.sqrt(1.0 - y * y), R * np.cos(tpr), s)
            wh = np.stack([x, y, np.sqrt(np.maximum(1.0 - (x * x + y * y), 0.0))], -1)
            wu = np.stack([la * wh[..., 0] + lb * wh[..., 2], lc * wh[..., 1], ld * wh[..., 0] + wh[..., 2]], -1)
            cltc = normalize(np.einsum("...i,...ij->...j", wu, self.rows))  # mul(wu, basis)
        diffuse = np.where((r1 < self.p_u)[..., None], uniform, cltc)
        return np.where(use_ggx[..., None], ggx, diffuse)


# ------------------------------------------------------------- light sampling

class LightWorld:
    """The parts of bind group 1 that sample_light reads, as float64 numpy arrays."""

    def __init__(self, geometries, attributes_uv, materials, scene_alias, light_probabilities, emissive_count,
                 sky_rgba, sky_alias, sky_average_luminance):
        self.v = np.asarray(geometries, np.float64).reshape(-1, 3, 3)
        self.uv = np.asarray(attributes_uv, np.float64).reshape(-1, 3, 2)
        self.mat = materials  # (material index per triangle, emission rgb, luminance, weight) arrays
        self.alias = scene_alias  # structured: triangle_index, alias_index, threshold, selection_probability
        self.p = np.asarray(light_probabilities, np.float64)
        self.count = int(emissive_count)
        self.sky = np.asarray(sky_rgba, np.float64)  # H x W x 4
        self.sky_alias = sky_alias  # structured: alias_index, threshold, selection_probability
        self.avg_lum = float(sky_average_luminance)

    # skybox_uv / evaluate_skybox / skybox_texel_solid_angle / skybox_light_pdf (trace.slang:467-489)
    def skybox_uv(self, d):
        u = np.arctan2(d[..., 2], d[..., 0]) * INV_2PI + 0.5
        return np.stack([u - np.floor(u), np.arctan2(np.sqrt(d[..., 0] ** 2 + d[..., 2] ** 2), d[..., 1]) * INV_PI], -1)

    def skybox(self, d):
        """Bilinear, clamp-to-edge sample (world_resources.rs:451-456) times the average luminance."""
        H, W = self.sky.shape[:2]
        uv = self.skybox_uv(d)
        x, y = uv[..., 0] * W - 0.5, uv[..., 1] * H - 0.5
        x0, y0 = np.floor(x), np.floor(y)
        fx, fy = (x - x0)[..., None], (y - y0)[..., None]
        ix0, iy0 = np.clip(x0, 0, W - 1).astype(np.int64), np.clip(y0, 0, H - 1).astype(np.int64)
        ix1, iy1 = np.clip(x0 + 1, 0, W - 1).astype(np.int64), np.clip(y0 + 1, 0, H - 1).astype(np.int64)
        s = self.sky[..., :3]
        top = lerp(s[iy0, ix0], s[iy0, ix1], fx)
        bottom = lerp(s[iy1, ix0], s[iy1, ix1], fx)
        return lerp(top, bottom, fy) * self.avg_lum

    def texel_solid_angle(self, row):
        H, W = self.sky.shape[:2]
        step = PI / H
        pole = np.minimum(row, H - 1 - row)
        return (TWO_PI / W) * 2.0 * np.sin((pole + 0.5) * step) * np.sin(0.5 * step)

    def skybox_pdf(self, d, prob):
        H, W = self.sky.shape[:2]
        uv = self.skybox_uv(d)
        px = np.minimum(np.floor(uv[..., 0] * W), W - 1).astype(np.int64)
        py = np.minimum(np.floor(uv[..., 1] * H), H - 1).astype(np.int64)
        sel = self.sky_alias["selection_probability"].astype(np.float64)[py * W + px]
        return np.where(prob > 0.0, prob * sel / self.texel_solid_angle(py), 0.0)

    def sample(self, origins, rng):
        """sample_light (trace.slang:531-592) for every lane: (direction, distance, emission, pdf, triangle)."""
        n = origins.shape[0]
        direction = np.zeros((n, 3))
        distance = np.zeros(n)
        emission = np.zeros((n, 3))
        pdf = np.zeros(n)
        tri = np.full(n, -1, np.int64)
        p0, p1 = self.p
        if p0 + p1 <= 0.0:
            return direction, distance, emission, pdf, tri
        pick = rng()
        is_tri = pick < p0
        is_sky = ~is_tri
        if self.count:
            c = self.count
            slot = np.minimum(np.floor(rng(is_tri) * c), c - 1).astype(np.int64)
            cand = self.alias[slot]
            entry = self.alias[np.where(rng(is_tri) < cand["threshold"], slot, cand["alias_index"])]
            t = entry["triangle_index"].astype(np.int64)
            v = self.v[t]
            root = np.sqrt(rng(is_tri))
            bu = 1.0 - root
            bv = root * (1.0 - rng(is_tri))
            bw = 1.0 - bu - bv
            delta = bu[:, None] * v[:, 0] + bv[:, None] * v[:, 1] + bw[:, None] * v[:, 2] - origins
            d2 = dot(delta, delta)
            ok = is_tri & (d2 > 0.0)
            dist = np.sqrt(np.where(ok, d2, 1.0))
            dirn = delta / dist[:, None]
            area = 0.5 * np.abs(dot(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), dirn))
            prob = p0 * entry["selection_probability"].astype(np.float64)
            tpdf = np.where((prob > 0.0) & (area > 0.0), prob * d2 / np.where(area > 0.0, area, 1.0), 0.0)
            mi, erg, elum, ew = self.mat
            m = mi[t]
            em = (ew[m] * elum[m])[:, None] * erg[m]  # opaque, untextured emitters: coverage 1
            direction = np.where(ok[:, None], dirn, direction)
            distance = np.where(ok, dist, distance)
            pdf = np.where(ok, tpdf, pdf)
            emission = np.where(ok[:, None], em, emission)
            tri = np.where(ok, t, tri)
        if is_sky.any():
            H, W = self.sky.shape[:2]
            cnt = W * H
            slot = np.minimum(np.floor(rng(is_sky) * cnt), cnt - 1).astype(np.int64)
            cand = self.sky_alias[slot]
            index = np.where(rng(is_sky) < cand["threshold"], slot, cand["alias_index"]).astype(np.int64)
            row, col = index // W, index % W
            phi = ((col + rng(is_sky)) / W - 0.5) * TWO_PI
            north = row < H // 2
            pole = np.where(north, row, H - 1 - row)
            half = 0.5 * PI / H
            a, b = np.sin(pole * half), np.sin((pole + 1) * half)
            shs = lerp(a * a, b * b, rng(is_sky))
            cos_t = 1.0 - 2.0 * shs
            sin_t = 2.0 * np.sqrt(np.maximum(0.0, shs * (1.0 - shs)))
            d = np.stack([sin_t * np.cos(phi), np.where(north, cos_t, -cos_t), sin_t * np.sin(phi)], -1)
            direction = np.where(is_sky[:, None], d, direction)
            distance = np.where(is_sky, FLT_MAX, distance)
            pdf = np.where(is_sky, self.skybox_pdf(d, p1), pdf)
            emission = np.where(is_sky[:, None], self.skybox(d), emission)
        return direction, distance, emission, pdf, tri
