"""CPU oracle of the environment-map renderer (numpy, FP64). Parity unpinned: the reference
renders with Mitsuba 3 (not installed) under fig/ennis.exr (missing), so no golden images
exist; this is a restatement of the scene and of the direct-illumination algorithm.

TEST INFRASTRUCTURE ONLY (tests). Restates, step by step, the direct-illumination renderer
that svbrdf_envmap_render runs on the GPU for the reference's novel-view video
(src/mitsubarender.py:7-105, src/scripts.py:44-59): the reference's scene (camera at (0, 0, 1),
fov 50, a 0.3-scaled rectangle turned Ry(angle) Rx(-15) Rz(-5), a normal map over a 0.5 / 0.5
GGX conductor + diffuse blend, a lat-long environment), one environment and one BSDF sample
per camera sample, the power heuristic, and the same counter-based random numbers. The
reference itself needs Mitsuba 3 (not installed) and fig/ennis.exr (missing from its
repository), so parity is pinned to this restatement, not to Mitsuba's images.
Vectorised over pixels; one loop over samples. Small images only.
"""
from __future__ import annotations

import math

import numpy as np

PI = math.pi


def pcg_hash(v):
    """The PCG hash of Jarzynski and Olano (JCGT 2020) on uint32 arrays (wrapping)."""
    v = np.asarray(v, dtype=np.uint64) & 0xFFFFFFFF
    state = (v * 747796405 + 2891336453) & 0xFFFFFFFF
    word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
    return ((word >> 22) ^ word) & 0xFFFFFFFF


def rnd(seed, pixel, sample, dim):
    h = pcg_hash((pcg_hash((pcg_hash(np.uint64(seed) ^ pixel) + sample) & 0xFFFFFFFF) + dim) & 0xFFFFFFFF)
    return (h >> 8).astype(np.float64) / 16777216.0


def rotation(angle_deg):
    k = PI / 180.0
    a, b, c = angle_deg * k, -15.0 * k, -5.0 * k
    ry = np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])
    rx = np.array([[1, 0, 0], [0, math.cos(b), -math.sin(b)], [0, math.sin(b), math.cos(b)]])
    rz = np.array([[math.cos(c), -math.sin(c), 0], [math.sin(c), math.cos(c), 0], [0, 0, 1]])
    return ry @ (rx @ rz)


def _norm(v):
    return v / np.sqrt((v * v).sum(-1, keepdims=True))


def _dot(a, b):
    return (a * b).sum(-1)


def _srgb_to_linear(c):
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)


def _bilinear(plane, s, t):
    h, w = plane.shape
    x = s * w - 0.5
    y = t * h - 0.5
    fx, fy = np.floor(x), np.floor(y)
    ax, ay = x - fx, y - fy
    x0 = fx.astype(np.int64) % w
    y0 = fy.astype(np.int64) % h
    x1 = (x0 + 1) % w
    y1 = (y0 + 1) % h
    return (1 - ay) * ((1 - ax) * plane[y0, x0] + ax * plane[y0, x1]) + ay * ((1 - ax) * plane[y1, x0] +
                                                                             ax * plane[y1, x1])


def _env_eval(env, row_pdf, col_pdf, d, intensity):
    he, we = env.shape[:2]
    u = np.arctan2(d[..., 0], -d[..., 2]) / (2 * PI)
    u = np.where(u < 0, u + 1.0, u)
    v = np.arccos(np.clip(d[..., 1], -1.0, 1.0)) / PI
    j = np.minimum((u * we).astype(np.int64), we - 1)
    i = np.minimum((v * he).astype(np.int64), he - 1)
    st = np.sin(v * PI)
    p = row_pdf[i].astype(np.float64) * col_pdf[i, j].astype(np.float64) * he * we
    pdf = np.where(st > 0, p / (2 * PI * PI * np.where(st > 0, st, 1.0)), 0.0)
    return env[i, j].astype(np.float64) * intensity, pdf


def _bsdf(kd, ks, alpha, wi, wo):
    valid = (wi[..., 2] > 0) & (wo[..., 2] > 0)
    a2 = alpha * alpha
    h = _norm(wi + wo)
    t = h[..., 2] ** 2 * (a2 - 1) + 1
    D = a2 / (PI * t * t)

    def g1(w):
        c2 = w[..., 2] ** 2
        t2 = np.maximum(1 - c2, 0) / np.maximum(c2, 1e-20)
        return 2 / (1 + np.sqrt(1 + a2 * t2))

    g1i = g1(wi)
    G = g1i * g1(wo)
    wiz = np.where(valid, wi[..., 2], 1.0)
    spec = D * G / (4 * wiz)
    diff = wo[..., 2] / PI
    pdf = np.where(valid, 0.5 * (g1i * D / (4 * wiz)) + 0.5 * diff, 0.0)
    f = 0.5 * (ks * spec[..., None] + kd * diff[..., None])
    return np.where(valid[..., None], f, 0.0), pdf


def _vndf(wi, alpha, u1, u2):
    vh = _norm(np.stack([alpha * wi[..., 0], alpha * wi[..., 1], wi[..., 2]], -1))
    lensq = vh[..., 0] ** 2 + vh[..., 1] ** 2
    inv = np.where(lensq > 0, 1 / np.sqrt(np.where(lensq > 0, lensq, 1.0)), 0.0)
    t1 = np.where((lensq > 0)[..., None], np.stack([-vh[..., 1] * inv, vh[..., 0] * inv, np.zeros_like(inv)], -1),
                  np.array([1.0, 0.0, 0.0]))
    t2 = np.cross(vh, t1)
    r = np.sqrt(u1)
    phi = 2 * PI * u2
    p1 = r * np.cos(phi)
    p2 = r * np.sin(phi)
    s = 0.5 * (1 + vh[..., 2])
    p2 = (1 - s) * np.sqrt(np.maximum(1 - p1 * p1, 0)) + s * p2
    nh = t1 * p1[..., None] + t2 * p2[..., None] + vh * np.sqrt(np.maximum(1 - p1 * p1 - p2 * p2, 0))[..., None]
    return _norm(np.stack([alpha * nh[..., 0], alpha * nh[..., 1], np.maximum(nh[..., 2], 0)], -1))


def _power(a, b):
    s = a * a + b * b
    return np.where(s > 0, a * a / np.where(s > 0, s, 1.0), 0.0)


def render(textures, env, tables, res, angle, intensity=1.0, spp=16, seed=0):
    """[res, res, 3] display image of the material (textures [9, H, W] in [-1, 1]) under the
    environment env [He, We, 3] with the importance tables (row_cdf, row_pdf, col_cdf,
    col_pdf) of env_distribution."""
    tex = np.asarray(textures, dtype=np.float64)
    env = np.asarray(env, dtype=np.float32)
    row_cdf, row_pdf, col_cdf, col_pdf = tables
    he, we = env.shape[:2]
    R = rotation(angle)
    R0, R1, R2 = R[:, 0], R[:, 1], R[:, 2]
    tan_half = math.tan(25.0 * PI / 180.0)
    pix = np.arange(res * res, dtype=np.uint64)
    py = (pix // res).astype(np.float64)
    px = (pix % res).astype(np.float64)
    org = np.array([0.0, 0.0, 1.0])
    acc = np.zeros((res * res, 3))
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        for s in range(spp):
            acc += _sample(s, seed, pix, px, py, res, tan_half, org, R0, R1, R2, tex, env, row_cdf, row_pdf,
                           col_cdf, col_pdf, he, we, intensity)
    img = acc / spp
    return (np.clip(img, 0, 1) ** (1 / 2.2)).reshape(res, res, 3)


def _sample(s, seed, pix, px, py, res, tan_half, org, R0, R1, R2, tex, env, row_cdf, row_pdf, col_cdf, col_pdf, he,
            we, intensity):
    """Radiance of camera sample s of every pixel."""
    jx, jy = rnd(seed, pix, s, 0), rnd(seed, pix, s, 1)
    sx = (2 * (px + jx) / res - 1) * tan_half
    sy = (1 - 2 * (py + jy) / res) * tan_half
    d = _norm(np.stack([sx, sy, -np.ones_like(sx)], -1))
    dn = d @ R2
    t = np.where(np.abs(dn) > 1e-8, -(org @ R2) / np.where(np.abs(dn) > 1e-8, dn, 1.0), -1.0)
    p = org + d * t[:, None]
    lx = (p @ R0) / 0.3
    ly = (p @ R1) / 0.3
    hit = (t > 0) & (np.abs(lx) <= 1) & (np.abs(ly) <= 1) & (dn < 0)
    le_miss, _ = _env_eval(env, row_pdf, col_pdf, d, intensity)
    su = 0.5 * (lx + 1)
    tv = 1 - 0.5 * (ly + 1)
    m9 = np.stack([_bilinear(tex[c], su, tv) for c in range(9)], -1)
    kd = _srgb_to_linear(0.5 * (m9[:, 0:3] + 1))
    ks = _srgb_to_linear(0.5 * (m9[:, 6:9] + 1))
    alpha = np.maximum(_srgb_to_linear(0.5 * (m9[:, 5] + 1)), 1e-3)
    nx, ny = m9[:, 3], m9[:, 4]
    nz = np.sqrt(np.maximum(1 - nx * nx - ny * ny, 0))
    n = _norm(R0 * nx[:, None] + R1 * ny[:, None] + R2 * nz[:, None])
    ts = _norm(R0 - n * (n @ R0)[:, None])
    tt = np.cross(n, ts)
    wiw = -d
    wi = np.stack([_dot(wiw, ts), _dot(wiw, tt), _dot(wiw, n)], -1)
    L = np.zeros((res * res, 3))
    # environment sample
    u1, u2 = rnd(seed, pix, s, 2), rnd(seed, pix, s, 3)
    i = np.clip(np.searchsorted(row_cdf[1:].astype(np.float64), u1, side="right"), 0, he - 1)
    r0, r1 = row_cdf[i].astype(np.float64), row_cdf[i + 1].astype(np.float64)
    dv = np.where(r1 > r0, (u1 - r0) / np.where(r1 > r0, r1 - r0, 1.0), 0.5)
    cc = col_cdf[i].astype(np.float64)  # [P, We+1]
    j = np.clip((cc[:, 1:] <= u2[:, None]).sum(1), 0, we - 1)
    c0, c1 = cc[np.arange(len(j)), j], cc[np.arange(len(j)), j + 1]
    du = np.where(c1 > c0, (u2 - c0) / np.where(c1 > c0, c1 - c0, 1.0), 0.5)
    theta = PI * (i + dv) / he
    phi = 2 * PI * (j + du) / we
    st = np.sin(theta)
    dl = np.stack([st * np.sin(phi), np.cos(theta), -st * np.cos(phi)], -1)
    up = dl @ R2 > 0
    le, pdf_l = _env_eval(env, row_pdf, col_pdf, dl, intensity)
    wo = np.stack([_dot(dl, ts), _dot(dl, tt), _dot(dl, n)], -1)
    f, pdf_b = _bsdf(kd, ks, alpha, wi, wo)
    use = up & (pdf_l > 0)
    w = np.where(use, _power(pdf_l, pdf_b) / np.where(pdf_l > 0, pdf_l, 1.0), 0.0)
    L += np.where(use[:, None], f * le * w[:, None], 0.0)
    # BSDF sample
    uc, v1, v2 = rnd(seed, pix, s, 4), rnd(seed, pix, s, 5), rnd(seed, pix, s, 6)
    h = _vndf(wi, alpha, v1, v2)
    wo_s = h * (2 * _dot(wi, h))[:, None] - wi
    r = np.sqrt(v1)
    ph = 2 * PI * v2
    wo_d = np.stack([r * np.cos(ph), r * np.sin(ph), np.sqrt(np.maximum(1 - v1, 0))], -1)
    wo = np.where((uc < 0.5)[:, None], wo_s, wo_d)
    f, pdf_b = _bsdf(kd, ks, alpha, wi, wo)
    dw = ts * wo[:, 0:1] + tt * wo[:, 1:2] + n * wo[:, 2:3]
    le, pdf_l = _env_eval(env, row_pdf, col_pdf, dw, intensity)
    ok = (wi[:, 2] > 0) & (pdf_b > 0) & (dw @ R2 > 0)
    w = np.where(ok, _power(pdf_b, pdf_l) / np.where(pdf_b > 0, pdf_b, 1.0), 0.0)
    L += np.where(ok[:, None], f * le * w[:, None], 0.0)
    return np.where(hit[:, None], L, le_miss)
