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


def make_tinted_env(w: int, h: int, seed: int = 0) -> np.ndarray:
    """A small map whose channels differ (tests that channels stay apart)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    env = make_env(w, h, seed=seed, sun_max=1e3)
    tint = rng.uniform(0.25, 1.0, size=(h, w, 3)).astype(np.float32)
    env[..., :3] *= tint
    return env
