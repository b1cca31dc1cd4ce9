"""Host-side API over ``libalthea_ibl.so`` (the C ABI in include/althea_ibl.h).

Mirrors the reference's interface for this path:

* ``ImageBasedLighting.createResources``  -- Include/Althea/ImageBasedLighting.h:46-49,
  Src/ImageBasedLighting.cpp:415-605 (bake, then hand out the four images);
* ``IBLResources.bind / registerToHeap / getHandles`` -- :20-52 and
  Include/Althea/ImageBasedLighting.h:24-43 (env, prefiltered, irradiance,
  BRDF LUT, in that order);
* ``IBLHandles`` -- Include/Althea/ImageBasedLighting.h:17-22.

Device memory comes from PyTorch tensors (plumbing only); every computation
runs in the CUDA library.  There is no CPU fallback: importing works without
a GPU (so host logic can be tested), but any call that computes raises if the
library or a CUDA device is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, NamedTuple, Optional

from . import build as _build

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_UNSUPPORTED = 4
ERR_BUDGET = 5
ERR_NOT_READY = 6

GEN_REF_HASH = 0
GEN_HAMMERSLEY = 1
LUT_ASSET = 0
LUT_CORRECTED = 1
MAX_MIPS = 16


class IBLError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"althea_ibl status {status}: {message}")
        self.status = status


class MipTarget(ctypes.Structure):
    _fields_ = [("out_dev", ctypes.c_void_p), ("pitch_bytes", ctypes.c_size_t),
                ("width", ctypes.c_int), ("height", ctypes.c_int), ("roughness", ctypes.c_float)]


class Config(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "env_width", "env_height", "irradiance_width", "irradiance_height", "mip_count",
        "first_mip_width", "first_mip_height", "samples", "generator", "lut_size", "lut_samples",
        "lut_orientation", "path", "out_format")]


class Outputs(ctypes.Structure):
    _fields_ = [("irradiance_dev", ctypes.c_void_p), ("irradiance_pitch_bytes", ctypes.c_size_t),
                ("mip_dev", ctypes.c_void_p * MAX_MIPS),
                ("mip_pitch_bytes", ctypes.c_size_t * MAX_MIPS),
                ("lut_dev", ctypes.c_void_p), ("lut_pitch_bytes", ctypes.c_size_t)]


class TcWork(ctypes.Structure):
    _fields_ = [("dense_pairs", ctypes.c_double), ("visible_pairs", ctypes.c_double),
                ("tensor_flops", ctypes.c_double), ("cuda_core_pairs", ctypes.c_double),
                ("tensor_launches", ctypes.c_int)]


class Probe(ctypes.Structure):
    _fields_ = [("level0_dev", ctypes.c_void_p), ("chain_dev", ctypes.c_void_p),
                ("env_width", ctypes.c_int), ("env_height", ctypes.c_int),
                ("irradiance_dev", ctypes.c_void_p), ("irradiance_width", ctypes.c_int),
                ("irradiance_height", ctypes.c_int), ("irradiance_pitch_bytes", ctypes.c_size_t),
                ("mip_count", ctypes.c_int), ("mip_dev", ctypes.c_void_p * MAX_MIPS),
                ("mip_pitch_bytes", ctypes.c_size_t * MAX_MIPS),
                ("mip_width", ctypes.c_int * MAX_MIPS), ("mip_height", ctypes.c_int * MAX_MIPS),
                ("mip_roughness", ctypes.c_float * MAX_MIPS)]


class BatchParams(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_int), ("generator", ctypes.c_int),
                ("lut_dev", ctypes.c_void_p), ("lut_size", ctypes.c_int),
                ("lut_pitch_bytes", ctypes.c_size_t), ("lut_samples", ctypes.c_int),
                ("lut_orientation", ctypes.c_int), ("flags", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "probes", "prefilter_jobs", "prefilter_tiles", "irradiance_blocks", "tile_x", "tile_y",
        "persistent_blocks", "irradiance_target_blocks", "tuned", "graph", "graph_kernels",
        "contraction_items")]


BATCH_AUTOTUNE = 1
BATCH_GRAPH = 2
BATCH_PRECISION = 4
BATCH_HALF = 8
PATH_PLAIN = 0
PATH_PRECISION = 1
FORMAT_RGBA32F = 0
FORMAT_RGBA16F = 1
TIMED_BAKES = 64  # contraction launches a context keeps the device time of


class ServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_size_t), ("max_inflight", ctypes.c_int),
                ("samples", ctypes.c_int), ("generator", ctypes.c_int),
                ("irradiance_width", ctypes.c_int), ("irradiance_height", ctypes.c_int),
                ("path", ctypes.c_int)]


MAX_SUNS = 16


class Sun(ctypes.Structure):
    _fields_ = [("dir", ctypes.c_float * 3), ("sigma", ctypes.c_float),
                ("radiance", ctypes.c_float)]


class Request(ctypes.Structure):
    _fields_ = [("env_host", ctypes.c_void_p), ("env_width", ctypes.c_int),
                ("env_height", ctypes.c_int), ("mip_count", ctypes.c_int),
                ("irradiance_host", ctypes.c_void_p), ("mips_host", ctypes.c_void_p),
                ("tag", ctypes.c_uint64), ("env_id", ctypes.c_int), ("sun_count", ctypes.c_int),
                ("suns", Sun * MAX_SUNS)]


class Completion(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("done_s", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("inflight", ctypes.c_int), ("queued", ctypes.c_int),
                ("bytes_in_use", ctypes.c_size_t), ("bytes_reserved", ctypes.c_size_t),
                ("peak_bytes_in_use", ctypes.c_size_t), ("completed", ctypes.c_uint64),
                ("rejected", ctypes.c_uint64), ("bytes_resident", ctypes.c_size_t),
                ("resident_maps", ctypes.c_int)]

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libalthea_ibl.so (building it with nvcc when absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path) or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise OSError(f"{path} missing; run althea_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    sig = {
        "althea_ibl_abi_version": (i, []),
        "althea_ibl_last_error": (ctypes.c_char_p, []),
        "althea_ibl_chain_levels": (i, [i, i]),
        "althea_ibl_chain_texels": (sz, [i, i]),
        "althea_ibl_chain_level_offset": (sz, [i, i, i]),
        "althea_ibl_build_env_chain": (i, [vp, i, i, vp, vp]),
        "althea_ibl_prefilter": (i, [vp, i, i, ctypes.POINTER(MipTarget), i, i, i, vp]),
        "althea_ibl_irradiance_workspace_size": (sz, [i, i, i, i]),
        "althea_ibl_irradiance": (i, [vp, i, i, vp, i, i, sz, vp, sz, vp]),
        "althea_ibl_brdf_lut": (i, [vp, i, sz, i, i, vp]),
        "althea_ibl_config_reference": (None, [ctypes.POINTER(Config), i, i]),
        "althea_ibl_create": (i, [ctypes.POINTER(Config), ctypes.POINTER(vp)]),
        "althea_ibl_destroy": (i, [vp]),
        "althea_ibl_mip_info": (i, [vp, i, ctypes.POINTER(i), ctypes.POINTER(i),
                                    ctypes.POINTER(ctypes.c_float)]),
        "althea_ibl_irradiance_size": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "althea_ibl_upload_env": (i, [vp, vp, i, vp]),
        "althea_ibl_env_chain": (vp, [vp]),
        "althea_ibl_bake": (i, [vp, ctypes.POINTER(Outputs), vp]),
        "althea_ibl_bake_status": (i, [vp, vp]),
        "althea_ibl_context_device_bytes": (sz, [vp]),
        "althea_ibl_contraction_times": (i, [vp, ctypes.POINTER(ctypes.c_float), i,
                                             ctypes.POINTER(i)]),
        "althea_ibl_irradiance_noalloc": (i, [vp, i, i, vp, i, i, sz, vp]),
        "althea_ibl_batch_create": (i, [ctypes.POINTER(Probe), i, ctypes.POINTER(BatchParams), vp,
                                        ctypes.POINTER(vp)]),
        "althea_ibl_batch_run": (i, [vp, vp]),
        "althea_ibl_batch_describe": (i, [vp, ctypes.POINTER(BatchInfo)]),
        "althea_ibl_batch_status": (i, [vp, vp]),
        "althea_ibl_batch_destroy": (i, [vp]),
        "althea_ibl_server_create": (i, [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]),
        "althea_ibl_server_submit": (i, [vp, ctypes.POINTER(Request)]),
        "althea_ibl_server_poll": (i, [vp, ctypes.POINTER(Completion), i, ctypes.POINTER(i)]),
        "althea_ibl_server_get_stats": (i, [vp, ctypes.POINTER(ServerStats)]),
        "althea_ibl_server_request_bytes": (sz, [vp, i, i, i]),
        "althea_ibl_server_now": (ctypes.c_double, []),
        "althea_ibl_server_register_env": (i, [vp, vp, i, i, i, ctypes.POINTER(i)]),
        "althea_ibl_server_unregister_env": (i, [vp, i]),
        "althea_ibl_apply_suns": (i, [vp, vp, i, i, ctypes.POINTER(Sun), i, vp]),
        "althea_ibl_server_destroy": (i, [vp]),
        "althea_ibl_tc_workspace_size": (sz, [i, i, ctypes.POINTER(MipTarget), i,
                                              ctypes.POINTER(i), i, i, i]),
        "althea_ibl_tc_plan": (i, [i, i, ctypes.POINTER(MipTarget), i, i, ctypes.POINTER(i),
                                   ctypes.POINTER(i)]),
        "althea_ibl_bake_tc": (i, [vp, i, i, ctypes.POINTER(MipTarget), i, ctypes.POINTER(i),
                                   vp, i, i, sz, i, vp, sz, vp]),
        "althea_ibl_tc_error": (i, [vp, vp]),
        "althea_ibl_tc_stats": (i, [i, i, ctypes.POINTER(MipTarget), i, ctypes.POINTER(i), i, i,
                                    i, ctypes.POINTER(TcWork)]),
        "althea_ibl_tc_wait_selftest": (i, [ctypes.c_ulonglong, ctypes.POINTER(i), vp]),
        "althea_ibl_bake_tc_ex": (i, [vp, i, i, ctypes.POINTER(MipTarget), i, ctypes.POINTER(i),
                                      vp, i, i, sz, i, vp, sz, i, vp]),
        "althea_ssr_level_offset": (sz, [i, i, i]),
        "althea_ssr_convolve": (i, [vp, i, i, i, vp]),
        "althea_ssr_convolve_levels": (i, [ctypes.POINTER(vp), ctypes.POINTER(sz), i, i, i, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(status: int) -> None:
    if status != OK:
        msg = load().althea_ibl_last_error()
        raise IBLError(status, msg.decode() if msg else "")


def _torch():
    import torch
    return torch


def _stream_ptr(stream) -> Optional[int]:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _require_cuda(t, name, ncomp, allow_half=False):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise IBLError(ERR_INVALID_ARGUMENT, f"{name} must be a CUDA tensor")
    if t.dtype != torch.float32 and not (allow_half and t.dtype == torch.float16):
        raise IBLError(ERR_INVALID_ARGUMENT,
                       f"{name} must be float32" + (" or float16" if allow_half else ""))
    if t.dim() != 3 or t.shape[2] != ncomp or t.stride(2) != 1 or t.stride(1) != ncomp:
        raise IBLError(ERR_INVALID_ARGUMENT, f"{name} must be (H, W, {ncomp}) with packed texels")


def _pitch(t, ncomp) -> int:
    return t.stride(0) * t.element_size()


# The C calls receive bare pointers and pitches, so they cannot see how large
# a caller's tensor is.  These checks hold the tensors to the extents the
# kernels read or write; they look only at tensor metadata (no device access).

def _require_shape(t, name, shape) -> None:
    torch = _torch()
    if not isinstance(t, torch.Tensor):
        raise IBLError(ERR_INVALID_ARGUMENT, f"{name} must be a tensor, not {type(t).__name__}")
    if tuple(t.shape) != tuple(shape):
        raise IBLError(ERR_INVALID_ARGUMENT,
                       f"{name} has shape {tuple(t.shape)}; this call writes {tuple(shape)}")


def _require_chain(chain, w: int, h: int) -> None:
    """chain must hold every level of a w x h env: chain_texels(w, h) RGBA32F
    texels, contiguous, on a CUDA device."""
    torch = _torch()
    if not isinstance(chain, torch.Tensor) or chain.dtype != torch.float32:
        raise IBLError(ERR_INVALID_ARGUMENT, "chain must be a float32 tensor")
    if not chain.is_contiguous():
        raise IBLError(ERR_INVALID_ARGUMENT, "chain must be contiguous")
    need = chain_texels(w, h)
    if chain.numel() < 4 * need:
        raise IBLError(ERR_INVALID_ARGUMENT,
                       f"chain holds {chain.numel() // 4} texels; the chain of a {w}x{h} env "
                       f"has {need}")
    if not chain.is_cuda:
        raise IBLError(ERR_INVALID_ARGUMENT, "chain must be a CUDA tensor")


def _require_counts(outs, roughness, limit=MAX_MIPS) -> None:
    if len(outs) != len(roughness):
        raise IBLError(ERR_INVALID_ARGUMENT,
                       f"{len(outs)} output mips but {len(roughness)} roughness values")
    if len(outs) > limit:
        raise IBLError(ERR_INVALID_ARGUMENT, f"{len(outs)} mips; at most {limit}")


# ---- stateless kernels -------------------------------------------------------

def chain_levels(w: int, h: int) -> int:
    return load().althea_ibl_chain_levels(w, h)


def chain_texels(w: int, h: int) -> int:
    return load().althea_ibl_chain_texels(w, h)


def chain_level_offset(w: int, h: int, level: int) -> int:
    return load().althea_ibl_chain_level_offset(w, h, level)


def build_env_chain(env, stream=None):
    """env: CUDA (H, W, 4) float32 -> chain tensor (texels, 4), every level."""
    torch = _torch()
    _require_cuda(env, "env", 4)
    env = env.contiguous()
    h, w = env.shape[:2]
    chain = torch.empty((chain_texels(w, h), 4), dtype=torch.float32, device=env.device)
    _check(load().althea_ibl_build_env_chain(env.data_ptr(), w, h, chain.data_ptr(),
                                             _stream_ptr(stream)))
    return chain


def build_env_chain_into(env, chain, stream=None) -> None:
    """Builds the chain of env (CUDA (H, W, 4)) into a preallocated chain tensor."""
    _require_cuda(env, "env", 4)
    h, w = env.shape[:2]
    _require_chain(chain, w, h)
    _check(load().althea_ibl_build_env_chain(env.contiguous().data_ptr(), w, h, chain.data_ptr(),
                                             _stream_ptr(stream)))


def chain_level(chain, w: int, h: int, level: int):
    lw, lh = max(w >> level, 1), max(h >> level, 1)
    off = chain_level_offset(w, h, level)
    return chain[off:off + lw * lh].view(lh, lw, 4)


def prefilter(chain, w: int, h: int, outs: List, roughness: List[float], samples: int,
              generator: int = GEN_REF_HASH, stream=None) -> None:
    """Writes each prefiltered mip into the given (h_m, w_m, 4) CUDA tensors."""
    _require_counts(outs, roughness)
    _require_chain(chain, w, h)
    n = len(outs)
    arr = (MipTarget * max(n, 1))()
    for k, (o, r) in enumerate(zip(outs, roughness)):
        _require_cuda(o, f"mip {k}", 4)
        arr[k] = MipTarget(o.data_ptr(), _pitch(o, 4), o.shape[1], o.shape[0], float(r))
    _check(load().althea_ibl_prefilter(chain.data_ptr(), w, h, arr, n, samples, generator,
                                       _stream_ptr(stream)))


def irradiance(chain, w: int, h: int, out, workspace=None, stream=None) -> None:
    torch = _torch()
    _require_chain(chain, w, h)
    _require_cuda(out, "irradiance", 4)
    oh, ow = out.shape[:2]
    L = load()
    need = L.althea_ibl_irradiance_workspace_size(w, h, ow, oh)
    if need == 0:
        _check(ERR_UNSUPPORTED if L.althea_ibl_last_error() else ERR_INVALID_ARGUMENT)
    if workspace is None:
        workspace = torch.empty(need, dtype=torch.uint8, device=out.device)
    _check(L.althea_ibl_irradiance(chain.data_ptr(), w, h, out.data_ptr(), ow, oh, _pitch(out, 4),
                                   workspace.data_ptr(), workspace.numel() *
                                   workspace.element_size(), _stream_ptr(stream)))


def brdf_lut(n: int, samples: int = 1024, orientation: int = LUT_ASSET, out=None, device=None,
             stream=None):
    torch = _torch()
    if out is None:
        out = torch.empty((n, n, 2), dtype=torch.float32, device=device or "cuda")
    _require_cuda(out, "brdf lut", 2)
    _check(load().althea_ibl_brdf_lut(out.data_ptr(), n, _pitch(out, 2), samples, orientation,
                                      _stream_ptr(stream)))
    return out


# ---- context: the createResources mirror ----------------------------------------

def reference_config(env_width: int, env_height: int) -> Config:
    cfg = Config()
    load().althea_ibl_config_reference(ctypes.byref(cfg), env_width, env_height)
    return cfg


def make_config(env_width, env_height, irradiance_size=None, mip_count=5, first_mip=None,
                samples=10000, generator=GEN_REF_HASH, lut_size=0, lut_samples=1024,
                lut_orientation=LUT_ASSET, path=PATH_PLAIN, out_format=FORMAT_RGBA32F) -> Config:
    """The reference's settings for this env size with the given overrides.
    path: PATH_PLAIN (the reference estimator) or PATH_PRECISION (the
    tensor-core contraction within 1e-3 of FP64); out_format: FORMAT_RGBA32F
    or, on the precision path, FORMAT_RGBA16F for the mips and irradiance."""
    cfg = reference_config(env_width, env_height)
    cfg.path = path
    cfg.out_format = out_format
    if irradiance_size is not None:
        cfg.irradiance_width, cfg.irradiance_height = irradiance_size
    cfg.mip_count = mip_count
    if first_mip is not None:
        cfg.first_mip_width, cfg.first_mip_height = first_mip
    cfg.samples = samples
    cfg.generator = generator
    cfg.lut_size = lut_size
    cfg.lut_samples = lut_samples
    cfg.lut_orientation = lut_orientation
    return cfg


class IBLHandles(NamedTuple):
    environmentMapHandle: int
    prefilteredMapHandle: int
    irradianceMapHandle: int
    brdfLutHandle: int


@dataclass
class IBLResources:
    """The four images the renderer binds (env, prefiltered, irradiance, LUT)."""
    environmentMap: object
    prefilteredMap: List[object]
    irradianceMap: object
    brdfLut: Optional[object]
    handles: Optional[IBLHandles] = None
    _heap_ids: List[int] = field(default_factory=list)

    def bind(self, assignment: list) -> list:
        # Src/ImageBasedLighting.cpp:20-26 order.
        assignment.extend([self.environmentMap, self.prefilteredMap, self.irradianceMap,
                           self.brdfLut])
        return assignment

    def registerToHeap(self, heap: list) -> None:
        ids = []
        for img in (self.environmentMap, self.prefilteredMap, self.irradianceMap, self.brdfLut):
            heap.append(img)
            ids.append(len(heap) - 1)
        self.handles = IBLHandles(*ids)

    def getHandles(self) -> IBLHandles:
        if self.handles is None:
            raise IBLError(ERR_NOT_READY, "registerToHeap has not been called")
        return self.handles


class BakeContext:
    """A resident env map plus its mip chain on one device (C context)."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        self._ctx = ctypes.c_void_p()
        _check(load().althea_ibl_create(ctypes.byref(cfg), ctypes.byref(self._ctx)))

    def close(self):
        if self._ctx:
            load().althea_ibl_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def mip_info(self, m):
        w, h, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _check(load().althea_ibl_mip_info(self._ctx, m, ctypes.byref(w), ctypes.byref(h),
                                          ctypes.byref(r)))
        return w.value, h.value, r.value

    def irradiance_size(self):
        w, h = ctypes.c_int(), ctypes.c_int()
        _check(load().althea_ibl_irradiance_size(self._ctx, ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value

    def upload_env(self, env, stream=None):
        """env: (H, W, 4) float32, CUDA tensor or pinned/any host tensor."""
        torch = _torch()
        env = env.contiguous()
        if tuple(env.shape) != (self.cfg.env_height, self.cfg.env_width, 4):
            raise IBLError(ERR_INVALID_ARGUMENT, f"env shape {tuple(env.shape)}")
        if env.dtype != torch.float32:
            raise IBLError(ERR_INVALID_ARGUMENT, "env must be float32")
        _check(load().althea_ibl_upload_env(self._ctx, env.data_ptr(), 1 if env.is_cuda else 0,
                                            _stream_ptr(stream)))

    def chain(self):
        torch = _torch()
        ptr = load().althea_ibl_env_chain(self._ctx)
        n = chain_texels(self.cfg.env_width, self.cfg.env_height)
        return _device_view(ptr, n * 4).view(n, 4)

    def _out_dtype(self):
        torch = _torch()
        return torch.float16 if self.cfg.out_format == FORMAT_RGBA16F else torch.float32

    def device_bytes(self) -> int:
        """Device memory the context holds: the resident chain and its workspaces."""
        return load().althea_ibl_context_device_bytes(self._ctx)

    def allocate_outputs(self, device="cuda"):
        torch = _torch()
        dt = self._out_dtype()
        iw, ih = self.irradiance_size()
        irr = torch.empty((ih, iw, 4), dtype=dt, device=device)
        mips = []
        for m in range(self.cfg.mip_count):
            w, h, _ = self.mip_info(m)
            mips.append(torch.empty((h, w, 4), dtype=dt, device=device))
        lut = None
        if self.cfg.lut_size > 0:
            n = self.cfg.lut_size
            lut = torch.empty((n, n, 2), dtype=torch.float32, device=device)
        return irr, mips, lut

    def bake(self, irr, mips, lut=None, stream=None, check: bool = False):
        """Bakes into caller tensors of exactly the context's sizes and format
        (as allocate_outputs makes them): irradiance (ih, iw, 4), one
        (h_m, w_m, 4) tensor per mip -- float32, or float16 for an RGBA16F
        config -- and, when the config has a LUT, (n, n, 2) float32.
        check: synchronise and raise if a precision bake's bounded waits gave up."""
        torch = _torch()
        dt = self._out_dtype()
        for k, t in enumerate([irr] + list(mips)):
            if isinstance(t, torch.Tensor) and t.dtype != dt:
                raise IBLError(ERR_INVALID_ARGUMENT,
                               f"output {k} is {t.dtype}; this context writes {dt}")
        iw, ih = self.irradiance_size()
        _require_shape(irr, "irradiance", (ih, iw, 4))
        if len(mips) != self.cfg.mip_count:
            raise IBLError(ERR_INVALID_ARGUMENT,
                           f"{len(mips)} mip tensors; this context bakes {self.cfg.mip_count}")
        for m, t in enumerate(mips):
            w, h, _ = self.mip_info(m)
            _require_shape(t, f"mip {m}", (h, w, 4))
        if self.cfg.lut_size > 0:
            n = self.cfg.lut_size
            if lut is None:
                raise IBLError(ERR_INVALID_ARGUMENT, f"this context bakes a {n}x{n} LUT: pass one")
            _require_shape(lut, "lut", (n, n, 2))
        o = Outputs()
        half = dt == torch.float16
        _require_cuda(irr, "irradiance", 4, allow_half=half)
        o.irradiance_dev = irr.data_ptr()
        o.irradiance_pitch_bytes = _pitch(irr, 4)
        for m, t in enumerate(mips):
            _require_cuda(t, f"mip {m}", 4, allow_half=half)
            o.mip_dev[m] = t.data_ptr()
            o.mip_pitch_bytes[m] = _pitch(t, 4)
        if lut is not None and self.cfg.lut_size > 0:
            _require_cuda(lut, "lut", 2)
            o.lut_dev = lut.data_ptr()
            o.lut_pitch_bytes = _pitch(lut, 2)
        sp = _stream_ptr(stream)
        _check(load().althea_ibl_bake(self._ctx, ctypes.byref(o), sp))
        if check:
            self.status(stream)

    def status(self, stream=None) -> None:
        """Synchronises the stream; raises IBLError if a precision bake's
        kernels gave up on a bounded wait."""
        _check(load().althea_ibl_bake_status(self._ctx, _stream_ptr(stream)))

    def contraction_times(self) -> List[float]:
        """Device ms of the contraction launch of the last (up to
        TIMED_BAKES) precision bakes, oldest first (CUDA events the context
        records around that launch on the bake's stream)."""
        buf = (ctypes.c_float * TIMED_BAKES)()
        n = ctypes.c_int(0)
        _check(load().althea_ibl_contraction_times(self._ctx, buf, TIMED_BAKES,
                                                   ctypes.byref(n)))
        return [float(buf[k]) for k in range(n.value)]


def _device_view(ptr: int, nfloats: int):
    """A torch float32 view of library-owned device memory (no copy)."""
    torch = _torch()

    class _Holder:
        __cuda_array_interface__ = {"shape": (nfloats,), "typestr": "<f4",
                                    "data": (ptr, False), "version": 3}
    return torch.as_tensor(_Holder(), device="cuda")


class ImageBasedLighting:
    """``ImageBasedLighting::createResources`` for the GB300 bake."""

    @staticmethod
    def createResources(env, cfg: Optional[Config] = None, stream=None) -> IBLResources:
        """env: (H, W, 4) float32 (host or CUDA).  Bakes irradiance, the
        prefiltered chain and (when cfg.lut_size > 0) the BRDF LUT, on the
        path and in the output format cfg names (default: the reference's
        estimator, RGBA32F)."""
        h, w = int(env.shape[0]), int(env.shape[1])
        cfg = cfg or reference_config(w, h)
        ctx = BakeContext(cfg)
        try:
            ctx.upload_env(env, stream)
            irr, mips, lut = ctx.allocate_outputs()
            # synchronous like the reference's bake (vkQueueWaitIdle), and
            # checked: a precision bake that gave up raises here
            ctx.bake(irr, mips, lut, stream, check=True)
            env_dev = chain_level(ctx.chain(), w, h, 0).clone()
        finally:
            ctx.close()
        return IBLResources(environmentMap=env_dev, prefilteredMap=mips, irradianceMap=irr,
                            brdfLut=lut)

    @staticmethod
    def buildLayout() -> List[str]:
        # Src/ImageBasedLighting.cpp:607-619: four texture bindings.
        return ["environmentMap", "prefilteredMap", "irradianceMap", "brdfLut"]


# ---- analytic sun lobes ---------------------------------------------------------

def make_suns(suns) -> tuple:
    """[(direction (3,), sigma rad, radiance), ...] -> (ctypes Sun array, count)."""
    n = len(suns)
    if n > MAX_SUNS:
        raise IBLError(ERR_INVALID_ARGUMENT, f"{n} suns; at most {MAX_SUNS}")
    arr = (Sun * MAX_SUNS)()
    for k, (d, sigma, lum) in enumerate(suns):
        arr[k].dir[0], arr[k].dir[1], arr[k].dir[2] = (float(d[0]), float(d[1]), float(d[2]))
        arr[k].sigma, arr[k].radiance = float(sigma), float(lum)
    return arr, n


def apply_suns(base, suns, out=None, stream=None):
    """out = base + the suns' Gaussian lobes on R, G, B (CUDA (H, W, 4) float32;
    out may be base).  suns: [(direction, sigma in radians, radiance), ...]."""
    torch = _torch()
    _require_cuda(base, "base", 4)
    if not base.is_contiguous():
        raise IBLError(ERR_INVALID_ARGUMENT, "base must be contiguous")
    if out is None:
        out = torch.empty_like(base)
    _require_cuda(out, "out", 4)
    _require_shape(out, "out", tuple(base.shape))
    if not out.is_contiguous():
        raise IBLError(ERR_INVALID_ARGUMENT, "out must be contiguous")
    arr, n = make_suns(suns)
    h, w = base.shape[:2]
    _check(load().althea_ibl_apply_suns(base.data_ptr(), out.data_ptr(), w, h, arr, n,
                                        _stream_ptr(stream)))
    return out


# ---- batches -------------------------------------------------------------------

@dataclass
class ProbeSpec:
    """One probe of a batch: its env size, chain of mips and irradiance size."""
    env_width: int
    env_height: int
    mip_sizes: List[tuple]
    roughness: List[float]
    irradiance_size: Optional[tuple] = (32, 16)


def spec_for(env_width: int, env_height: int, mip_count: Optional[int] = None,
             irradiance_size=(32, 16)) -> ProbeSpec:
    """Batch-config probe: mips from W/2, mip_count = log2(W) - 3 by default,
    roughness m/(M-1)."""
    if mip_count is None:
        mip_count = max(1, env_width.bit_length() - 1 - 3)
    sizes = [(max((env_width >> 1) >> m, 1), max((env_height >> 1) >> m, 1))
             for m in range(mip_count)]
    rough = [m / (mip_count - 1) if mip_count > 1 else 0.0 for m in range(mip_count)]
    return ProbeSpec(env_width, env_height, sizes, rough, irradiance_size)


class ProbeBatch:
    """Device buffers and a batch plan for many probes (althea_ibl_batch_*).

    ``levels0``: per-probe CUDA (H, W, 4) env tensors (the chain is rebuilt from
    them on every run).  Outputs are allocated here and exposed as
    ``chains``, ``mips`` (list of lists), ``irradiance`` and ``lut``."""

    def __init__(self, specs: List[ProbeSpec], levels0: List, samples: int = 1024,
                 generator: int = GEN_HAMMERSLEY, lut_size: int = 0, lut_samples: int = 1024,
                 lut_orientation: int = LUT_ASSET, autotune: bool = True, graph: bool = True,
                 stream=None, device="cuda", precision: bool = False, half: bool = False):
        torch = _torch()
        self.specs = specs
        # precision: mips and irradiance by the tensor-core path; half: RGBA16F outputs
        out_dtype = torch.float16 if half else torch.float32
        texel = 8 if half else 16
        self.levels0 = levels0
        self.chains, self.mips, self.irradiance = [], [], []
        n = len(specs)
        self._probes = (Probe * max(n, 1))()
        for i, (s, env) in enumerate(zip(specs, levels0)):
            _require_cuda(env, f"env {i}", 4)
            if tuple(env.shape[:2]) != (s.env_height, s.env_width):
                raise IBLError(ERR_INVALID_ARGUMENT, f"env {i} shape {tuple(env.shape)}")
            chain = torch.empty((chain_texels(s.env_width, s.env_height), 4),
                                dtype=torch.float32, device=device)
            mips = [torch.empty((h, w, 4), dtype=out_dtype, device=device)
                    for w, h in s.mip_sizes]
            irr = None
            if s.irradiance_size is not None:
                iw, ih = s.irradiance_size
                irr = torch.empty((ih, iw, 4), dtype=out_dtype, device=device)
            self.chains.append(chain)
            self.mips.append(mips)
            self.irradiance.append(irr)
            p = self._probes[i]
            p.level0_dev = env.data_ptr()
            p.chain_dev = chain.data_ptr()
            p.env_width, p.env_height = s.env_width, s.env_height
            if irr is not None:
                p.irradiance_dev = irr.data_ptr()
                p.irradiance_width, p.irradiance_height = s.irradiance_size
                p.irradiance_pitch_bytes = irr.stride(0) * irr.element_size()
            p.mip_count = len(mips)
            for m, (t, r) in enumerate(zip(mips, s.roughness)):
                p.mip_dev[m] = t.data_ptr()
                p.mip_pitch_bytes[m] = t.stride(0) * t.element_size()
                p.mip_width[m], p.mip_height[m] = t.shape[1], t.shape[0]
                p.mip_roughness[m] = float(r)
        self.lut = None
        params = BatchParams()
        params.samples, params.generator = samples, generator
        if lut_size > 0:
            self.lut = torch.empty((lut_size, lut_size, 2), dtype=torch.float32, device=device)
            params.lut_dev, params.lut_size = self.lut.data_ptr(), lut_size
            params.lut_pitch_bytes = _pitch(self.lut, 2)
            params.lut_samples, params.lut_orientation = lut_samples, lut_orientation
        params.flags = ((BATCH_AUTOTUNE if autotune else 0) | (BATCH_GRAPH if graph else 0) |
                        (BATCH_PRECISION if precision else 0) | (BATCH_HALF if half else 0))
        del texel
        self._plan = ctypes.c_void_p()
        _check(load().althea_ibl_batch_create(self._probes, n, ctypes.byref(params),
                                              _stream_ptr(stream), ctypes.byref(self._plan)))

    def run(self, stream=None) -> None:
        _check(load().althea_ibl_batch_run(self._plan, _stream_ptr(stream)))

    def status(self, stream=None) -> None:
        """Synchronises `stream`; raises when a bounded wait of the last run's
        contraction gave up (its outputs are then undefined)."""
        _check(load().althea_ibl_batch_status(self._plan, _stream_ptr(stream)))

    def info(self) -> BatchInfo:
        inf = BatchInfo()
        _check(load().althea_ibl_batch_describe(self._plan, ctypes.byref(inf)))
        return inf

    def close(self) -> None:
        if self._plan:
            load().althea_ibl_batch_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- precision path (tensor cores) ------------------------------------------------

def tc_plan(w: int, h: int, mip_sizes: List[tuple], roughness: List[float],
            irradiance_width: int = 0):
    """Source level chosen per mip (-1: roughness 0, plain path) and for the
    irradiance."""
    n = len(mip_sizes)
    arr = (MipTarget * max(n, 1))()
    for k, ((mw, mh), r) in enumerate(zip(mip_sizes, roughness)):
        arr[k] = MipTarget(0, mw * 16, mw, mh, float(r))
    lv = (ctypes.c_int * max(n, 1))()
    il = ctypes.c_int()
    _check(load().althea_ibl_tc_plan(w, h, arr, n, irradiance_width, lv, ctypes.byref(il)))
    return [lv[k] for k in range(n)], il.value


def tc_stats(w: int, h: int, mip_sizes: List[tuple], roughness: List[float],
             irradiance_size=None) -> TcWork:
    """The planned work of a precision bake with the planner's levels: dense
    and visible (output, source) pairs, tensor-core flops issued, CUDA-core
    pairs, contraction launches (host only)."""
    n = len(mip_sizes)
    arr = (MipTarget * max(n, 1))()
    for k, ((mw, mh), r) in enumerate(zip(mip_sizes, roughness)):
        arr[k] = MipTarget(0, mw * 16, mw, mh, float(r))
    iw, ih = irradiance_size or (0, 0)
    out = TcWork()
    _check(load().althea_ibl_tc_stats(w, h, arr, n, None, iw, ih, -1, ctypes.byref(out)))
    return out


def tc_wait_selftest(limit_ms: float = 20.0, stream=None) -> int:
    """Runs the precision kernel's bounded wait against a barrier nothing
    completes; raises IBLError unless it gave up and reported.  Returns the
    milliseconds it waited."""
    waited = ctypes.c_int(0)
    _check(load().althea_ibl_tc_wait_selftest(int(limit_ms * 1e6), ctypes.byref(waited),
                                              _stream_ptr(stream)))
    return waited.value


def bake_tc(chain, w: int, h: int, outs: List, roughness: List[float], irradiance=None,
            levels: Optional[List[int]] = None, irradiance_level: int = -1, workspace=None,
            stream=None, check: bool = True):
    """Precision-path bake into CUDA tensors (mips and optional irradiance):
    float32 outputs are RGBA32F, float16 outputs RGBA16F (all of one type)."""
    torch = _torch()
    _require_counts(outs, roughness)
    if levels is not None and len(levels) != len(outs):
        raise IBLError(ERR_INVALID_ARGUMENT,
                       f"{len(levels)} source levels for {len(outs)} output mips")
    _require_chain(chain, w, h)
    n = len(outs)
    arr = (MipTarget * max(n, 1))()
    all_out = list(outs) + ([irradiance] if irradiance is not None else [])
    half = bool(all_out) and all_out[0].dtype == torch.float16
    if any((t.dtype == torch.float16) != half for t in all_out):
        raise IBLError(ERR_INVALID_ARGUMENT, "precision outputs must all be float32 or float16")
    for k, (o, r) in enumerate(zip(outs, roughness)):
        _require_cuda(o, f"mip {k}", 4, allow_half=True)
        arr[k] = MipTarget(o.data_ptr(), _pitch(o, 4), o.shape[1], o.shape[0], float(r))
    lv = None
    if levels is not None:
        lv = (ctypes.c_int * max(n, 1))(*levels)
    iw = ih = 0
    ip = 0
    ipitch = 0
    if irradiance is not None:
        _require_cuda(irradiance, "irradiance", 4, allow_half=True)
        ih, iw = irradiance.shape[:2]
        ip, ipitch = irradiance.data_ptr(), _pitch(irradiance, 4)
    L = load()
    need = L.althea_ibl_tc_workspace_size(w, h, arr, n, lv, iw, ih, irradiance_level)
    if need == 0:
        raise IBLError(ERR_UNSUPPORTED, L.althea_ibl_last_error().decode())
    if workspace is None or workspace.numel() < need:
        workspace = torch.empty(need, dtype=torch.uint8, device=chain.device)
    sp = _stream_ptr(stream)
    _check(L.althea_ibl_bake_tc_ex(chain.data_ptr(), w, h, arr, n, lv, ip, iw, ih, ipitch,
                                   irradiance_level, workspace.data_ptr(), need,
                                   FORMAT_RGBA16F if half else FORMAT_RGBA32F, sp))
    if check:
        _check(L.althea_ibl_tc_error(workspace.data_ptr(), sp))
    return workspace


# ---- reflection-buffer glossy convolution ------------------------------------

def ssr_level_offset(w: int, h: int, level: int) -> int:
    """Texel offset of level `level` in a packed reflection-buffer chain."""
    return load().althea_ssr_level_offset(w, h, level)


def ssr_convolve(chain, w: int, h: int, mip_count: int = 5, stream=None) -> None:
    """Convolves levels 1..mip_count-1 of a packed RGBA16F chain in place.

    chain: contiguous CUDA float16 tensor holding ssr_level_offset(w, h,
    mip_count) texels (4 halfs each), level 0 first."""
    torch = _torch()
    if not isinstance(chain, torch.Tensor) or not chain.is_cuda or chain.dtype != torch.float16:
        raise IBLError(ERR_INVALID_ARGUMENT, "chain must be a CUDA float16 tensor")
    if not chain.is_contiguous() or chain.numel() < 4 * ssr_level_offset(w, h, mip_count):
        raise IBLError(ERR_INVALID_ARGUMENT, "chain tensor too small or not contiguous")
    _check(load().althea_ssr_convolve(chain.data_ptr(), w, h, mip_count, _stream_ptr(stream)))


def ssr_convolve_levels(levels, stream=None) -> None:
    """levels: list of CUDA (H_l, W_l, 4) float16 tensors, level 0 first, each
    max(1, W >> l) x max(1, H >> l); fills levels 1.. from level 0."""
    torch = _torch()
    n = len(levels)
    if n < 1:
        raise IBLError(ERR_INVALID_ARGUMENT, "need at least one level")
    for l, t in enumerate(levels):
        if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float16:
            raise IBLError(ERR_INVALID_ARGUMENT, f"level {l} must be a CUDA float16 tensor")
        if t.dim() != 3 or t.shape[2] != 4 or t.stride(2) != 1 or t.stride(1) != 4:
            raise IBLError(ERR_INVALID_ARGUMENT, f"level {l} must be (H, W, 4) with packed texels")
    h, w = levels[0].shape[:2]
    for l, t in enumerate(levels):
        if tuple(t.shape[:2]) != (max(1, h >> l), max(1, w >> l)):
            raise IBLError(ERR_INVALID_ARGUMENT, f"level {l} has shape {tuple(t.shape[:2])}")
    ptrs = (ctypes.c_void_p * n)(*[t.data_ptr() for t in levels])
    pitch = (ctypes.c_size_t * n)(*[t.stride(0) * 2 for t in levels])
    _check(load().althea_ssr_convolve_levels(ptrs, pitch, w, h, n, _stream_ptr(stream)))


class ReflectionBuffer:
    """The reflection buffer of Src/ReflectionBuffer.cpp:20-100 as device
    memory: an RGBA16F chain of `mip_count` levels at the swapchain extent,
    packed in one tensor.  `level(0)` is where the SSR pass writes;
    convolveReflectionBuffer() fills the glossy levels 1.. from it
    (Src/ReflectionBuffer.cpp:163-275)."""

    def __init__(self, width: int, height: int, mip_count: int = 5, device="cuda"):
        torch = _torch()
        self.width, self.height, self.mip_count = width, height, mip_count
        self.chain = torch.zeros(4 * ssr_level_offset(width, height, mip_count),
                                 dtype=torch.float16, device=device)

    def level(self, l: int):
        w, h = max(1, self.width >> l), max(1, self.height >> l)
        off = 4 * ssr_level_offset(self.width, self.height, l)
        return self.chain[off:off + 4 * w * h].view(h, w, 4)

    def convolveReflectionBuffer(self, stream=None) -> None:
        ssr_convolve(self.chain, self.width, self.height, self.mip_count, stream)
