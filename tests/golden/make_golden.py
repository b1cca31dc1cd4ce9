"""Generate the golden fixtures in tests/golden/ (run in a checkout that has the
reference next to it; the fixtures themselves travel, the reference does not).

* ``ref_shaders_64x32.npz`` -- outputs of the reference's own compute shaders
  (Shaders/IBL_Precompute/*.comp, mechanically rewritten to C++ by
  oracle/make_ref.py and compiled into oracle/_ref/libref_ibl.so) on a seeded
  64x32 map: the whole 5-mip prefilter chain for both sample generators at
  N = 1024, two mips at the reference's N = 10000, and irradiance at env size
  (the reference's dispatch) on every texel.
* ``brdf_lut_png.npz`` -- the reference's baked LUT asset
  Content/PrecomputedMaps/brdf_lut.png (450x450, 8-bit palette), decoded here
  with a from-spec PNG reader, red/green channels subsampled every 5th texel.
* ``prefiltered_hdr_headers.npz`` -- width/height/format of the reference's
  shipped Content/PrecomputedMaps/*/Prefiltered{2..5}.hdr (RGBE).
* ``ref_LuxuryRoom_Prefiltered5.hdr`` -- one of those files, copied as is
  (25 KB), for the run-length RGBE reader.
* ``ref_ssr.npz`` -- the reference's Shaders/SSRGlossyConvolve.comp (rewritten
  to C++ by oracle/make_ref.py), dispatched level by level as
  Src/ReflectionBuffer.cpp:224-268 does, on seeded RGBA16F level-0 images of
  several shapes (odd, 16:9, tall, collapsing to 1x1, binary16 edge values).

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import struct
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from althea_gb300 import synth  # noqa: E402

REF = os.environ.get("ALTHEA_REFERENCE_ROOT", "/root/reference")


def ref_shader_fixture():
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref_ibl.so missing: run python oracle/make_ref.py")
    w, h = 64, 32
    env = synth.make_tinted_env(w, h, seed=11)
    chain = oracle.ref_build_chain(env)
    out = {"env": env, "chain": chain}
    for gen, tag in ((oracle.GEN_REF_HASH, "hash"), (oracle.GEN_HAMMERSLEY, "hammersley")):
        for m in range(5):
            ow, oh = w >> (m + 1), h >> (m + 1)
            out[f"prefilter_{tag}_n1024_m{m}"] = oracle.ref_prefilter(chain, w, h, ow, oh, m / 4.0,
                                                                     1024, gen)
    for m in (1, 3):
        ow, oh = w >> (m + 1), h >> (m + 1)
        out[f"prefilter_hash_n10000_m{m}"] = oracle.ref_prefilter(chain, w, h, ow, oh, m / 4.0,
                                                                 10000, oracle.GEN_REF_HASH)
    ys, xs = np.mgrid[0:h, 0:w]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    out["irradiance_envsize"] = oracle.ref_irradiance_envsize(chain, w, h, xy)
    out["rng_seed00_first8"] = oracle.rng_stream(0, 0, 8)
    np.savez_compressed(os.path.join(HERE, "ref_shaders_64x32.npz"), **out)


SSR_CASES = [(61, 37, 5, False), (96, 54, 5, False), (5, 3, 5, False), (33, 200, 5, False),
             (40, 24, 5, True), (128, 72, 7, True)]


def ref_ssr_fixture():
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libref_ibl.so missing: run python oracle/make_ref.py")
    out = {}
    for k, (w, h, mips, ext) in enumerate(SSR_CASES):
        l0 = synth.make_reflection(w, h, seed=40 + k, extremes=ext)
        out[f"in{k}"] = l0.view(np.uint16)
        out[f"out{k}"] = oracle.ref_ssr_convolve(l0, mips).view(np.uint16)
        out[f"shape{k}"] = np.array([w, h, mips])
    np.savez_compressed(os.path.join(HERE, "ref_ssr.npz"), **out)


def decode_png(path):
    """Minimal PNG reader (PNG spec, ISO/IEC 15948): 8-bit palette or RGB(A)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, plte, trns = 8, b"", None, None
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if typ == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif typ == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif typ == b"tRNS":
            trns = np.frombuffer(body, dtype=np.uint8)
        elif typ == b"IDAT":
            idat += body
    assert depth == 8 and interlace == 0
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = w * chans
    img = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    p = 0
    for y in range(h):
        ft = raw[p]
        line = np.frombuffer(raw[p + 1:p + 1 + stride], dtype=np.uint8).astype(np.int32)
        p += 1 + stride
        cur = np.zeros(stride, dtype=np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 255
        else:
            for i in range(stride):
                a = cur[i - chans] if i >= chans else 0
                b = prev[i]
                c = prev[i - chans] if i >= chans else 0
                if ft == 1:
                    v = a
                elif ft == 3:
                    v = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    v = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[i] = (line[i] + v) & 255
        img[y] = cur
        prev = cur
    img = img.reshape(h, w, chans)
    if ctype == 3:
        img = plte[img[..., 0]]
    return img


def lut_fixture():
    img = decode_png(os.path.join(REF, "Content", "PrecomputedMaps", "brdf_lut.png"))
    h, w = img.shape[:2]
    sub = img[2::5, 2::5, :2].copy()
    np.savez_compressed(os.path.join(HERE, "brdf_lut_png.npz"), rg=sub,
                        rows=np.arange(2, h, 5), cols=np.arange(2, w, 5), size=np.array([w, h]))


def hdr_header(path):
    with open(path, "rb") as f:
        head = f.read(4096)
    lines = head.split(b"\n")
    fmt = b""
    for i, ln in enumerate(lines):
        if ln.startswith(b"FORMAT="):
            fmt = ln[7:]
        if ln.startswith(b"-Y ") or ln.startswith(b"+Y "):
            parts = ln.split()
            return int(parts[3]), int(parts[1]), fmt.decode(), lines[0].decode()
    raise ValueError(path)


def hdr_fixture():
    rows = []
    base = os.path.join(REF, "Content", "PrecomputedMaps")
    for env in sorted(os.listdir(base)):
        d = os.path.join(base, env)
        if not os.path.isdir(d):
            continue
        for k in range(2, 6):
            p = os.path.join(d, f"Prefiltered{k}.hdr")
            if os.path.exists(p):
                w, h, fmt, magic = hdr_header(p)
                rows.append((env, k, w, h, fmt, magic))
    np.savez_compressed(os.path.join(HERE, "prefiltered_hdr_headers.npz"),
                        env=np.array([r[0] for r in rows]), mip=np.array([r[1] for r in rows]),
                        width=np.array([r[2] for r in rows]),
                        height=np.array([r[3] for r in rows]),
                        fmt=np.array([r[4] for r in rows]), magic=np.array([r[5] for r in rows]))


def hdr_file_fixture():
    """One shipped reference output (128x64, run-length RGBE) for the reader."""
    import shutil
    src = os.path.join(REF, "Content", "PrecomputedMaps", "LuxuryRoom", "Prefiltered5.hdr")
    shutil.copyfile(src, os.path.join(HERE, "ref_LuxuryRoom_Prefiltered5.hdr"))


if __name__ == "__main__":
    ref_shader_fixture()
    lut_fixture()
    hdr_fixture()
    hdr_file_fixture()
    ref_ssr_fixture()
    print("fixtures written to", HERE)
