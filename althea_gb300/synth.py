"""Seeded synthetic HDR equirect environment maps.

The reference bakes ``Content/HDRI_Skybox/<name>.hdr`` maps that are not part
of its checkout, and it names no public dataset, so every workload here uses
generated maps with the shapes and value ranges of the benchmark
configurations:

* sky: radiance(e) = 2.0 + (0.5 - 2.0) * |sin e|, e = elevation of the texel
  centre (horizon 2.0, zenith and nadir 0.5);
* noise: x one log-normal(mu=0, sigma=1) scalar per texel, applied to RGB;
* suns: + 8 Gaussian suns L_s * exp(-theta^2 / (2 sigma_s^2)),
  sigma_s ~ U[1, 3] degrees, L_s log-uniform in [1, sun_max]
  (1e4 for the plain configurations, 1e6 for the precision one),
  directions uniform on the sphere;
* alpha = 1.

Texel (x, y) of a W x H map has its centre at yaw = pi*(2(x+0.5)/W - 1),
pitch = pi*((y+0.5)/H - 0.5), direction (cos p cos yaw, sin p, cos p sin yaw)
-- the mapping of ``sampleEnvMap`` in Shaders/IBL_Precompute/
PreFilterEnvMap.comp:98-122.  Random draws come from numpy's PCG64 in a fixed
order (noise field, then per sun: direction, sigma, radiance).
"""
from __future__ import annotations

import numpy as np


def texel_directions(w: int, h: int) -> np.ndarray:
    """(H, W, 3) float64 unit directions of texel centres."""
    yaw = np.pi * (2.0 * (np.arange(w) + 0.5) / w - 1.0)
    pitch = np.pi * ((np.arange(h) + 0.5) / h - 0.5)
    cp, sp = np.cos(pitch)[:, None], np.sin(pitch)[:, None]
    cy, sy = np.cos(yaw)[None, :], np.sin(yaw)[None, :]
    return np.stack([cp * cy, np.broadcast_to(sp, (h, w)), cp * sy], axis=-1)


def make_env(w: int, h: int, seed: int = 0, sun_max: float = 1e4, n_suns: int = 8,
             with_suns: bool = True) -> np.ndarray:
    """Returns an (H, W, 4) float32 RGBA map."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pitch = np.pi * ((np.arange(h) + 0.5) / h - 0.5)
    sky = 2.0 + (0.5 - 2.0) * np.abs(np.sin(pitch))
    noise = rng.lognormal(mean=0.0, sigma=1.0, size=(h, w))
    rad = sky[:, None] * noise
    if with_suns and n_suns > 0:
        dirs = texel_directions(w, h)
        for _ in range(n_suns):
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            sigma = np.deg2rad(rng.uniform(1.0, 3.0))
            lum = float(np.exp(rng.uniform(0.0, np.log(sun_max))))
            cosang = np.clip(dirs @ d, -1.0, 1.0)
            theta = np.arccos(cosang)
            rad = rad + lum * np.exp(-theta * theta / (2.0 * sigma * sigma))
    env = np.empty((h, w, 4), dtype=np.float32)
    env[..., 0] = rad
    env[..., 1] = rad
    env[..., 2] = rad
    env[..., 3] = 1.0
    return env


def sun_params(w: int, h: int, seed: int = 0, sun_max: float = 1e4, n_suns: int = 8):
    """The suns make_env(w, h, seed, sun_max, n_suns) draws: a list of
    (unit direction, sigma in radians, radiance), replaying its PCG64 stream."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rng.lognormal(mean=0.0, sigma=1.0, size=(h, w))
    suns = []
    for _ in range(n_suns):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        sigma = np.deg2rad(rng.uniform(1.0, 3.0))
        lum = float(np.exp(rng.uniform(0.0, np.log(sun_max))))
        suns.append((d, sigma, lum))
    return suns


def draw_suns(seed: int, sun_max: float = 1e4, n_suns: int = 8):
    """n_suns suns drawn like make_env's (direction uniform on the sphere,
    sigma ~ U[1, 3] degrees, radiance log-uniform in [1, sun_max]) from their
    own PCG64 stream: the per-request suns of a re-bake of a resident sky."""
    rng = np.random.Generator(np.random.PCG64(seed))
    suns = []
    for _ in range(n_suns):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        sigma = np.deg2rad(rng.uniform(1.0, 3.0))
        lum = float(np.exp(rng.uniform(0.0, np.log(sun_max))))
        suns.append((d, sigma, lum))
    return suns


def make_tinted_env(w: int, h: int, seed: int = 0) -> np.ndarray:
    """A small map whose channels differ (tests that channels stay apart)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    env = make_env(w, h, seed=seed, sun_max=1e3)
    tint = rng.uniform(0.25, 1.0, size=(h, w, 3)).astype(np.float32)
    env[..., :3] *= tint
    return env


def make_reflection(w: int, h: int, seed: int = 0, extremes: bool = False) -> np.ndarray:
    """(H, W, 4) float16 level 0 of a reflection buffer (what the SSR pass
    writes into the RGBA16F buffer of Src/ReflectionBuffer.cpp:28-36).

    RGB: a screen-space gradient 0.2..1.5 times a log-normal(0, 0.75) texel
    noise, plus 16 Gaussian highlights (radius 1-4 % of the width, peak
    log-uniform in [1, 2000]); texels whose ray missed (10 %, in horizontal
    runs) are 0.  Alpha: the hit confidence, uniform in [0, 1], 0 on misses.
    extremes=True also plants binary16 edge values -- subnormals, -0, the
    largest finite half and its neighbours -- for the rounding paths.
    Draws: PCG64, in the order noise, highlights, misses, alpha, extremes."""
    rng = np.random.default_rng(seed)
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float64)
    u, v = (xs + 0.5) / w, (ys + 0.5) / h
    base = 0.2 + 1.3 * (0.5 * u + 0.5 * (1.0 - v))
    rgb = base[..., None] * np.array([1.0, 0.9, 0.8]) * rng.lognormal(0.0, 0.75, (h, w, 1))
    for _ in range(16):
        cx, cy = rng.uniform(0, w), rng.uniform(0, h)
        r = rng.uniform(0.01, 0.04) * w
        peak = np.exp(rng.uniform(0.0, np.log(2000.0)))
        tint = rng.uniform(0.6, 1.0, 3)
        # the Gaussian below 1e-7 of its peak (beyond 5.7 r) is left out
        x0, x1 = max(0, int(cx - 6 * r)), min(w, int(cx + 6 * r) + 1)
        y0, y1 = max(0, int(cy - 6 * r)), min(h, int(cy + 6 * r) + 1)
        d2 = (xs[y0:y1, x0:x1] - cx) ** 2 + (ys[y0:y1, x0:x1] - cy) ** 2
        rgb[y0:y1, x0:x1] += peak * tint * np.exp(-d2 / (2 * r * r))[..., None]
    miss = np.zeros((h, w), dtype=bool)
    for _ in range(max(1, (h * w) // 200)):
        y0, x0 = rng.integers(0, h), rng.integers(0, w)
        miss[y0, x0:x0 + rng.integers(1, 40)] = True
    alpha = rng.uniform(0.0, 1.0, (h, w))
    rgb[miss] = 0.0
    alpha[miss] = 0.0
    out = np.concatenate([rgb, alpha[..., None]], axis=2).astype(np.float16)
    if extremes:
        flat = out.reshape(-1)
        vals = np.array([0x0001, 0x03ff, 0x0400, 0x8000, 0x8001, 0x7bff, 0x7bfe, 0x3c00,
                         0xfbff, 0x0200], dtype=np.uint16).view(np.float16)
        idx = rng.choice(flat.size, size=min(flat.size, 64 * len(vals)), replace=False)
        flat[idx] = np.resize(vals, idx.size)
    return out
