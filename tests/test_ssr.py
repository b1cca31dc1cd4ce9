"""CPU tests of the reflection-buffer convolution's oracle and host logic.

The oracle (oracle/ssr_oracle.c) is pinned bit for bit to the reference's own
Shaders/SSRGlossyConvolve.comp, compiled as C++ and dispatched level by level
as Src/ReflectionBuffer.cpp:224-268 does (tests/golden/ref_ssr.npz, made by
tests/golden/make_golden.py)."""
import ctypes
import os

import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ssr.npz")


@pytest.fixture(scope="module")
def ssr_golden():
    return dict(np.load(GOLD))


def test_oracle_bit_identical_to_reference_shader(ssr_golden):
    k = 0
    while f"in{k}" in ssr_golden:
        w, h, mips = (int(v) for v in ssr_golden[f"shape{k}"])
        got = oracle.ssr_convolve(ssr_golden[f"in{k}"].view(np.float16), mips)
        assert np.array_equal(got.view(np.uint16), ssr_golden[f"out{k}"]), (w, h, mips)
        k += 1
    assert k == 6


def test_golden_covers_edge_cases(ssr_golden):
    shapes = [tuple(int(v) for v in ssr_golden[f"shape{k}"]) for k in range(6)]
    assert any(w % 2 and h % 2 for w, h, _ in shapes)              # odd both ways
    assert any(max(w, h) >> (m - 1) == 0 for w, h, m in shapes)    # levels collapse to 1x1
    assert any(h > 4 * w for w, h, _ in shapes)                     # tall
    planted = ssr_golden["in4"].ravel()
    assert (planted == 0x0001).any() and (planted == 0x7bff).any() and (planted == 0x8000).any()


def test_half_to_float_all_patterns():
    L = oracle.lib()
    L.oracle_half_to_float.restype = ctypes.c_float
    L.oracle_half_to_float.argtypes = [ctypes.c_uint16]
    bits = np.arange(65536, dtype=np.uint32).astype(np.uint16)
    ref = bits.view(np.float16).astype(np.float32)
    got = np.array([L.oracle_half_to_float(int(b)) for b in bits], dtype=np.float32)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))


def test_float_to_half_rounds_to_nearest_even():
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(30000) * 10.0 ** rng.integers(-9, 6, 30000)).astype(np.float32)
    # ties: the exact midpoints between neighbouring halfs, normal and subnormal
    h = np.arange(0, 0x7bff, 7, dtype=np.uint16)
    lo = h.view(np.float16).astype(np.float64)
    hi = (h + 1).view(np.float16).astype(np.float64)
    mids = ((lo + hi) / 2).astype(np.float32)
    edge = np.array([65504, 65519.996, 65520, 2.0 ** -24, 2.0 ** -25, 3 * 2.0 ** -25, 1e-30,
                     -0.0, np.inf, -np.inf], dtype=np.float32)
    x = np.concatenate([x, mids, -mids, edge])
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16)
    assert np.array_equal(oracle.float_to_half_bits(x), ref)


def test_level_offsets_agree_with_library():
    for w, h in [(3840, 2160), (61, 37), (1, 1), (5, 3)]:
        for l in range(8):
            assert ibl.ssr_level_offset(w, h, l) == oracle.ssr_level_offset(w, h, l)
    assert ibl.ssr_level_offset(3840, 2160, 1) == 3840 * 2160


def test_constant_buffer_stays_constant():
    l0 = np.ones((24, 40, 4), dtype=np.float16)
    out = oracle.ssr_convolve(l0, 5).astype(np.float32)
    assert np.abs(out - 1.0).max() <= 2.0 ** -10  # one half ulp at 1.0


def test_scaling_by_two_commutes():
    """Products and sums of the filter scale exactly by a power of two, and so
    does binary16 rounding of normal numbers: conv(2x) == 2 conv(x)."""
    l0 = synth.make_reflection(80, 48, seed=5)
    l0 = np.where(np.abs(l0) < 2.0 ** -13, np.float16(0), l0).astype(np.float16)
    a = oracle.ssr_convolve(l0, 5).astype(np.float32)
    b = oracle.ssr_convolve((l0.astype(np.float32) * 2).astype(np.float16), 5).astype(np.float32)
    small = np.abs(a) < 2.0 ** -13
    assert np.array_equal(b[~small], 2 * a[~small])


def test_python_binding_rejects_bad_arguments_without_gpu():
    with pytest.raises(ibl.IBLError):
        ibl.ssr_convolve(np.zeros(16, dtype=np.float16), 2, 2, 2)
    with pytest.raises(ibl.IBLError):
        ibl.ssr_convolve_levels([])


def test_c_abi_rejects_bad_arguments_without_gpu():
    L = ibl.load()
    assert L.althea_ssr_convolve(None, 16, 16, 5, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ssr_convolve(None, 16, 16, 0, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ssr_convolve(None, 16, 16, 17, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ssr_convolve(None, 0, 16, 5, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ssr_convolve_levels(None, None, 16, 16, 5, None) == ibl.ERR_INVALID_ARGUMENT
    ptrs = (ctypes.c_void_p * 2)(8, 16)
    pitch = (ctypes.c_size_t * 2)(12, 64)  # 12 bytes: not a whole texel
    assert L.althea_ssr_convolve_levels(ptrs, pitch, 1, 1, 2, None) == ibl.ERR_INVALID_ARGUMENT


@pytest.mark.skipif(oracle.ref_lib() is None, reason="oracle/_ref not built on this machine")
def test_ref_shader_agrees_on_random_case():
    """The reference shader compiled as C++ here and the C restatement agree on
    a fresh random case (beyond the committed fixtures)."""
    rng = np.random.default_rng(77)
    for w, h in [(50, 29), (128, 64), (3, 97)]:
        l0 = (rng.lognormal(0.0, 2.0, (h, w, 4)) * rng.choice([-1.0, 1.0], (h, w, 4)))
        l0 = l0.astype(np.float16)
        a = oracle.ssr_convolve(l0, 6)
        b = oracle.ref_ssr_convolve(l0, 6)
        assert np.array_equal(a.view(np.uint16), b.view(np.uint16)), (w, h)
