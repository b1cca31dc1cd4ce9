"""CPU oracle for the IBL precompute -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package.  The product library never calls it.

* ``lib()``      -- ctypes handle on ``oracle/libibl_oracle.so`` (the plain-C
  restatement, ``ibl_oracle.c``); built on demand with gcc.
* ``ref_lib()``  -- ctypes handle on ``oracle/_ref/libref_ibl.so``, the
  reference's own shader source mechanically rewritten to C++
  (``make_ref.py``); ``None`` when it was never generated on this machine.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libibl_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB_PATH = os.path.join(REF_DIR, "libref_ibl.so")

GEN_REF_HASH = 0
GEN_HAMMERSLEY = 1
LUT_ASSET = 0
LUT_CORRECTED = 1

_lock = threading.Lock()
_lib = None
_ref = None

_F = ctypes.POINTER(ctypes.c_float)
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile ibl_oracle.c and ssr_oracle.c into a shared library (gcc, OpenMP)."""
    src = os.path.join(HERE, "ibl_oracle.c")
    ssr = os.path.join(HERE, "ssr_oracle.c")
    deps = [src, ssr, os.path.join(HERE, "ibl_oracle.h"),
            os.path.join(HERE, "..", "althea_gb300", "csrc", "glsl_builtins.h")]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp",
                           "-ffp-contract=off", "-o", tmp, src, ssr, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref() -> str | None:
    """Compile oracle/_ref from generated sources if they exist here."""
    if os.path.exists(os.path.join(REF_DIR, "ref_prefilter_hash.cpp")):
        subprocess.check_call(["python3", os.path.join(HERE, "make_ref.py"), "--compile-only"])
        return REF_LIB_PATH
    return None


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            L.oracle_level_count.restype = ctypes.c_int
            L.oracle_chain_texels.restype = ctypes.c_size_t
            L.oracle_level_offset.restype = ctypes.c_size_t
            L.oracle_max_threads.restype = ctypes.c_int
            _lib = L
        return _lib


def ref_lib():
    global _ref
    with _lock:
        if _ref is None and os.path.exists(REF_LIB_PATH):
            _ref = ctypes.CDLL(REF_LIB_PATH)
            _ref.ref_level_count.restype = ctypes.c_int
        return _ref


def _fp(a):
    return a.ctypes.data_as(_F)


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def level_count(w: int, h: int) -> int:
    return lib().oracle_level_count(w, h)


def chain_texels(w: int, h: int) -> int:
    return lib().oracle_chain_texels(w, h)


def level_offset(w: int, h: int, level: int) -> int:
    return lib().oracle_level_offset(w, h, level)


def build_chain(env: np.ndarray) -> np.ndarray:
    """env: (H, W, 4) float32 -> chain (texels, 4) float32."""
    env = np.ascontiguousarray(env, dtype=np.float32)
    h, w = env.shape[:2]
    chain = np.empty((chain_texels(w, h), 4), dtype=np.float32)
    lib().oracle_build_chain(_fp(env), w, h, _fp(chain))
    return chain


def chain_level(chain: np.ndarray, w: int, h: int, level: int) -> np.ndarray:
    lw, lh = max(w >> level, 1), max(h >> level, 1)
    off = level_offset(w, h, level)
    return chain[off:off + lw * lh].reshape(lh, lw, 4)


def _xy_all(ow, oh):
    ys, xs = np.mgrid[0:oh, 0:ow]
    return np.stack([xs.ravel(), ys.ravel()], axis=1).astype(np.int32)


def prefilter(chain, w, h, ow, oh, roughness, samples, generator=GEN_REF_HASH,
              xy=None, nthreads=0):
    """Returns (n, 4) for listed texels, or (oh, ow, 4) for the whole image."""
    if xy is None:
        out = np.empty((oh, ow, 4), dtype=np.float32)
        lib().oracle_prefilter_image(_fp(chain), w, h, ow, oh, ctypes.c_float(roughness),
                                     samples, generator, _fp(out), nthreads)
        return out
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.empty((len(xy), 4), dtype=np.float32)
    lib().oracle_prefilter_texels(_fp(chain), w, h, ow, oh, ctypes.c_float(roughness),
                                  samples, generator, _ip(xy), len(xy), _fp(out), nthreads)
    return out


def irradiance(chain, w, h, ow, oh, xy=None, nthreads=0):
    if xy is None:
        out = np.empty((oh, ow, 4), dtype=np.float32)
        lib().oracle_irradiance_image(_fp(chain), w, h, ow, oh, _fp(out), nthreads)
        return out
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.empty((len(xy), 4), dtype=np.float32)
    lib().oracle_irradiance_texels(_fp(chain), w, h, ow, oh, _ip(xy), len(xy), _fp(out), nthreads)
    return out


def brdf_lut_f32(n, samples, orientation=LUT_ASSET, nthreads=0):
    out = np.empty((n, n, 2), dtype=np.float32)
    lib().oracle_brdf_lut_f32(n, samples, orientation, _fp(out), nthreads)
    return out


def brdf_lut_f64(n, samples, orientation=LUT_ASSET, nthreads=0):
    out = np.empty((n, n, 2), dtype=np.float64)
    lib().oracle_brdf_lut_f64(n, samples, orientation, _dp(out), nthreads)
    return out


def quad_prefilter(level0, ow, oh, roughness, xy, nthreads=0):
    level0 = np.ascontiguousarray(level0, dtype=np.float32)
    h, w = level0.shape[:2]
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.empty((len(xy), 4), dtype=np.float64)
    lib().oracle_quad_prefilter_texels(_fp(level0), w, h, ow, oh, ctypes.c_double(roughness),
                                       _ip(xy), len(xy), _dp(out), nthreads)
    return out


def quad_irradiance(level0, ow, oh, xy, nthreads=0):
    level0 = np.ascontiguousarray(level0, dtype=np.float32)
    h, w = level0.shape[:2]
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.empty((len(xy), 4), dtype=np.float64)
    lib().oracle_quad_irradiance_texels(_fp(level0), w, h, ow, oh, _ip(xy), len(xy), _dp(out),
                                        nthreads)
    return out


def builtin(fn: str, a, b=None):
    """Evaluates a portable GLSL built-in (sin, cos, atan, atan2, log2)."""
    code = {"sin": 0, "cos": 1, "atan": 2, "atan2": 3, "log2": 4}[fn]
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(a if b is None else b, dtype=np.float32)
    out = np.empty_like(a)
    lib().oracle_builtin_eval(code, _fp(a), _fp(b), _fp(out), len(a))
    return out


def rng_stream(sx, sy, count):
    out = np.empty(count, dtype=np.float32)
    lib().oracle_rng_stream(ctypes.c_uint32(sx), ctypes.c_uint32(sy), count, _fp(out))
    return out


# ---- the reference shaders compiled as C++ (oracle/_ref) --------------------

def ref_build_chain(env):
    env = np.ascontiguousarray(env, dtype=np.float32)
    h, w = env.shape[:2]
    chain = np.empty((chain_texels(w, h), 4), dtype=np.float32)
    ref_lib().ref_build_chain(_fp(env), w, h, _fp(chain))
    return chain


def ref_prefilter(chain, w, h, ow, oh, roughness, samples, generator=GEN_REF_HASH, xy=None,
                  nthreads=0):
    """Runs PreFilterEnvMap.comp's main for the listed texels (default: all).
    Returns the full (oh, ow, 4) image; unlisted texels are NaN."""
    R = ref_lib()
    fn = R.ref_prefilter_hash if generator == GEN_REF_HASH else R.ref_prefilter_hammersley
    if xy is None:
        xy = _xy_all(ow, oh)
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.full((oh, ow, 4), np.nan, dtype=np.float32)
    levels = level_count(w, h)
    fn(_fp(chain), w, h, levels, _fp(out), ow, oh, ctypes.c_float(roughness), samples,
       _ip(xy), len(xy), nthreads)
    return out


def ref_irradiance_envsize(chain, w, h, xy, nthreads=0):
    """Runs GenIrradianceMap.comp's main (output = env size, as the reference
    dispatches it) for the listed env-size texels."""
    xy = np.ascontiguousarray(xy, dtype=np.int32)
    out = np.full((h, w, 4), np.nan, dtype=np.float32)
    ref_lib().ref_irradiance_raw(_fp(chain), w, h, level_count(w, h), _fp(out), w, h, _ip(xy),
                                 len(xy), nthreads)
    return out


def ref_ssr_convolve(level0_half, mips, nthreads=0):
    """SSRGlossyConvolve.comp (the reference shader compiled as C++) dispatched
    the way ReflectionBuffer::convolveReflectionBuffer does it
    (Src/ReflectionBuffer.cpp:224-268): for level l = 1..mips-1, push constants
    width/height = level l's size, direction (0,1) for odd l and (1,0) for even
    l, roughness l/4, source = level l-1.  Returns the packed chain (flat
    float16, level 0 first) like ssr_convolve."""
    R = ref_lib()
    U16 = ctypes.POINTER(ctypes.c_uint16)
    R.ref_ssr_dispatch.restype = None
    R.ref_ssr_dispatch.argtypes = [U16, ctypes.c_int, ctypes.c_int, U16, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_float, ctypes.c_int]
    h, w = level0_half.shape[:2]
    dims = [(max(1, w >> l), max(1, h >> l)) for l in range(mips)]
    levels = [np.ascontiguousarray(level0_half, dtype=np.float16).view(np.uint16).copy()]
    for l in range(1, mips):
        (sw, sh), (dw, dh) = dims[l - 1], dims[l]
        dst = np.zeros((dh, dw, 4), dtype=np.uint16)
        dx, dy = (0.0, 1.0) if l & 1 else (1.0, 0.0)
        R.ref_ssr_dispatch(levels[-1].ctypes.data_as(U16), sw, sh, dst.ctypes.data_as(U16), dw,
                           dh, dw, dh, dx, dy, l / 4.0, nthreads)
        levels.append(dst)
    return np.concatenate([a.ravel() for a in levels]).view(np.float16)


# ---- reflection-buffer glossy convolution (ssr_oracle.c) --------------------------

def ssr_level_offset(w: int, h: int, level: int) -> int:
    L = lib()
    L.oracle_ssr_level_offset.restype = ctypes.c_size_t
    L.oracle_ssr_level_offset.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    return int(L.oracle_ssr_level_offset(w, h, level))


def ssr_convolve(level0_half: np.ndarray, mips: int) -> np.ndarray:
    """level0_half: (H, W, 4) float16.  Returns every level packed back to back
    as a flat float16 array (level 0 first), levels 1..mips-1 convolved."""
    h, w = level0_half.shape[:2]
    total = ssr_level_offset(w, h, mips)
    chain = np.zeros(total * 4, dtype=np.uint16)
    chain[:w * h * 4] = np.ascontiguousarray(level0_half, dtype=np.float16).view(np.uint16).ravel()
    L = lib()
    L.oracle_ssr_convolve.restype = None
    L.oracle_ssr_convolve.argtypes = [ctypes.POINTER(ctypes.c_uint16), ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int]
    L.oracle_ssr_convolve(chain.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16)), w, h, mips)
    return chain.view(np.float16)


def float_to_half_bits(x: np.ndarray) -> np.ndarray:
    L = lib()
    L.oracle_float_to_half.restype = ctypes.c_uint16
    L.oracle_float_to_half.argtypes = [ctypes.c_float]
    return np.array([L.oracle_float_to_half(float(v)) for v in np.asarray(x, np.float32).ravel()],
                    dtype=np.uint16)
