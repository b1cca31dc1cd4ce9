"""Radiance .hdr files and the on-disk bake cache.

``read_hdr`` / ``write_hdr`` wrap althea_ibl_hdr_read / althea_ibl_hdr_write
(RGBE, run-length scanlines).  ``BakeCache`` reproduces the reference's cache
layout and policy (Src/ImageBasedLighting.cpp:415-605):

* the env map is ``<root>/Content/HDRI_Skybox/<name>.hdr``; a missing one is an
  error (:421-425);
* the bake outputs are ``<root>/Content/PrecomputedMaps/<name>/Prefiltered{1..M}.hdr``
  and ``IrradianceMap.hdr``; if any is missing the probe is baked and every
  file written (:429-446, :58-102);
* the images handed to the renderer are then read back from those files
  (:483-568), so they carry the RGBE quantisation, as in the reference.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional

import numpy as np

from . import ibl


def _lib():
    L = ibl.load()
    if not getattr(L, "_hdr_bound", False):
        L.althea_ibl_hdr_read.restype = ctypes.c_int
        L.althea_ibl_hdr_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_float)),
                                          ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.althea_ibl_hdr_free.restype = None
        L.althea_ibl_hdr_free.argtypes = [ctypes.POINTER(ctypes.c_float)]
        L.althea_ibl_hdr_write.restype = ctypes.c_int
        L.althea_ibl_hdr_write.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_float),
                                           ctypes.c_int, ctypes.c_int]
        L._hdr_bound = True
    return L


def read_hdr(path: str) -> np.ndarray:
    """(H, W, 4) float32, alpha 1."""
    L = _lib()
    p = ctypes.POINTER(ctypes.c_float)()
    w, h = ctypes.c_int(), ctypes.c_int()
    ibl._check(L.althea_ibl_hdr_read(os.fsencode(path), ctypes.byref(p), ctypes.byref(w),
                                     ctypes.byref(h)))
    try:
        arr = np.ctypeslib.as_array(p, shape=(h.value, w.value, 4)).copy()
    finally:
        L.althea_ibl_hdr_free(p)
    return arr


def write_hdr(path: str, rgba: np.ndarray) -> None:
    a = np.ascontiguousarray(rgba, dtype=np.float32)
    if a.ndim != 3 or a.shape[2] not in (3, 4):
        raise ValueError("rgba must be (H, W, 3|4)")
    if a.shape[2] == 3:
        a = np.concatenate([a, np.ones(a.shape[:2] + (1,), np.float32)], axis=2)
    h, w = a.shape[:2]
    ibl._check(_lib().althea_ibl_hdr_write(os.fsencode(path),
                                           a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), w, h))


class BakeCache:
    """The reference's precompute cache under ``<root>/Content``."""

    def __init__(self, root: str, mip_count: int = 5):
        self.root = root
        self.mip_count = mip_count

    def env_path(self, name: str) -> str:
        return os.path.join(self.root, "Content", "HDRI_Skybox", name + ".hdr")

    def out_dir(self, name: str) -> str:
        return os.path.join(self.root, "Content", "PrecomputedMaps", name)

    def prefiltered_paths(self, name: str) -> List[str]:
        return [os.path.join(self.out_dir(name), f"Prefiltered{i + 1}.hdr")
                for i in range(self.mip_count)]

    def irradiance_path(self, name: str) -> str:
        return os.path.join(self.out_dir(name), "IrradianceMap.hdr")

    def complete(self, name: str) -> bool:
        return all(os.path.exists(p) for p in self.prefiltered_paths(name) + [self.irradiance_path(name)])

    def create_resources(self, name: str, cfg: Optional["ibl.Config"] = None, stream=None,
                         lut_size: int = 0):
        """createResources: bake when the cache is incomplete, then serve the
        cached (RGBE) images as device tensors.  Returns (IBLResources, baked)."""
        import torch
        path = self.env_path(name)
        if not os.path.exists(path):
            raise ibl.IBLError(ibl.ERR_INVALID_ARGUMENT, "Specified environment map does not exist!")
        env = read_hdr(path)
        h, w = env.shape[:2]
        baked = False
        if not self.complete(name):
            # a copy: the caller's config is left as it was
            c = (ibl.Config.from_buffer_copy(cfg) if cfg is not None
                 else ibl.reference_config(w, h))
            c.mip_count = self.mip_count
            c.lut_size = 0  # the cache holds no LUT file; the LUT is made below
            ctx = ibl.BakeContext(c)
            try:
                ctx.upload_env(torch.from_numpy(env), stream)
                irr, mips, _ = ctx.allocate_outputs()
                ctx.bake(irr, mips, None, stream)
                torch.cuda.synchronize()
                os.makedirs(self.out_dir(name), exist_ok=True)
                for p, t in zip(self.prefiltered_paths(name), mips):
                    write_hdr(p, t.cpu().numpy())
                write_hdr(self.irradiance_path(name), irr.cpu().numpy())
            finally:
                ctx.close()
            baked = True
        mips = [torch.from_numpy(read_hdr(p)).cuda() for p in self.prefiltered_paths(name)]
        irr = torch.from_numpy(read_hdr(self.irradiance_path(name))).cuda()
        lut = ibl.brdf_lut(lut_size) if lut_size > 0 else None
        res = ibl.IBLResources(environmentMap=torch.from_numpy(env).cuda(), prefilteredMap=mips,
                               irradianceMap=irr, brdfLut=lut)
        return res, baked
