"""CPU checks of the algebra the tensor-core path runs, in numpy float64.

On an equirect map the weight of output texel (i, x) for source texel (j, y)
depends only on (i, j) and the column offset d = (y - s x) mod ws, with
s = ws / wo.  The contraction kernel turns each output into GEMMs: with a
phase count g and a column step m (8 g = s m), source row j splits into g
phase rows P_ph[u] = L_j[g u + ph], and for the column residue x0 in [0, m)

    out[i, x0 + m n] = sum_{j, ph, k} A[i, (j, ph, k)] B[(j, ph, k), n]
    A = W_ij[g ((k - (s / g) x0) mod krow) + ph],   krow = ws / g
    B[(j, ph, k), n] = P_ph[(k + 8 n) mod krow]      (a Hankel matrix: rows 8 apart)

These tests build A and B exactly as written, for every branch of (g, m),
and check them against the direct sum and against the FP64 quadrature oracle
over the same source level.  They also emulate the BF16 hi/lo split
(hi = bf16(x), lo = bf16(x - hi); products hi.hi + hi.lo + lo.hi) and bound
its error.  The GPU tests check the kernels themselves against the oracle."""
import numpy as np
import pytest

import oracle


def phase_and_step(s):
    """(g, m) with 8 g = s m: the three cases of the planner."""
    if 8 % s == 0:
        return 1, 8 // s
    if s % 8 == 0:
        return s // 8, 1
    return s, 8


def weight_table(ws, hs, wo, ho, roughness, ggx=True):
    """W[i, j, d]: the weight of output row i (at column 0) for source texel
    (j, d).  Output directions are texel corners, source directions texel
    centres, solid angles the pitch bands of each source row."""
    yaw = np.pi * (2.0 * (np.arange(ws) + 0.5) / ws - 1.0)
    pit = np.pi * ((np.arange(hs) + 0.5) / hs - 0.5)
    edges = np.pi * (np.arange(hs + 1) / hs - 0.5)
    omega = (2.0 * np.pi / ws) * np.diff(np.sin(edges))
    src = np.stack([np.cos(pit)[:, None] * np.cos(yaw)[None, :],
                    np.broadcast_to(np.sin(pit)[:, None], (hs, ws)),
                    np.cos(pit)[:, None] * np.sin(yaw)[None, :]], -1)
    po = np.pi * (np.arange(ho) / ho - 0.5)
    n = np.stack([np.cos(po) * np.cos(-np.pi), np.sin(po), np.cos(po) * np.sin(-np.pi)], -1)
    c = np.einsum("ic,jdc->ijd", n, src)
    a2 = roughness * roughness
    if ggx:
        nh2 = 0.5 * (1.0 + c)
        w = a2 / (np.pi * (nh2 * (a2 - 1.0) + 1.0) ** 2) * c
    else:
        w = c / np.pi
    return np.where(c > 0.0, w * omega[None, :, None], 0.0)


def direct(W, L, s):
    ho, hs, ws = W.shape
    wo = ws // s
    out = np.empty((ho, wo, L.shape[-1]))
    for x in range(wo):
        idx = (np.arange(ws) - s * x) % ws
        out[:, x] = np.einsum("ijd,jdc->ic", W[:, :, idx], L)
    return out


def contraction(W, L, s, split=None):
    """The GEMM form; `split` maps an array to its (hi, lo) parts."""
    ho, hs, ws = W.shape
    wo = ws // s
    g, m = phase_and_step(s)
    krow = ws // g
    k = np.arange(krow)
    out = np.empty((ho, wo, L.shape[-1]))
    for x0 in range(m):
        # A[i, j, ph, k] = W[i, j, g ((k - (s/g) x0) mod krow) + ph]
        cols = g * ((k[None, :] - (s // g) * x0) % krow) + np.arange(g)[:, None]  # [ph, k]
        A = W[:, :, cols].reshape(ho, -1)
        nn = np.arange(wo // m)
        # B[j, ph, k, n] = L[j, g ((k + 8 n) mod krow) + ph]
        rows = g * ((k[:, None] + 8 * nn[None, :]) % krow)                      # [k, n]
        src = rows[None, :, :] + np.arange(g)[:, None, None]                    # [ph, k, n]
        B = L[:, src].reshape(-1, len(nn), L.shape[-1])
        if split is None:
            res = np.einsum("ik,knc->inc", A, B)
        else:
            ah, al = split(A)
            bh, bl = split(B)
            res = (np.einsum("ik,knc->inc", ah, bh) + np.einsum("ik,knc->inc", ah, bl) +
                   np.einsum("ik,knc->inc", al, bh))
        out[:, x0 + m * nn] = res
    return out


def bf16(x):
    """float32 -> nearest BF16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    b = (b + (((b >> 16) & 1) + 0x7FFF)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def hi_lo(x):
    x = np.asarray(x, dtype=np.float32)
    hi = bf16(x)
    lo = bf16(x - hi)
    return hi.astype(np.float64), lo.astype(np.float64)


def _level(ws, hs, seed):
    rng = np.random.default_rng(seed)
    L = np.exp(rng.normal(0.0, 1.0, size=(hs, ws, 3)))
    L[rng.integers(hs), rng.integers(ws)] = 1e6  # a sun
    return L


@pytest.mark.parametrize("s", [1, 2, 3, 4, 6, 8, 16, 24])
def test_gemm_form_equals_direct_sum_and_quadrature(s):
    wo, ho = 16, 8
    ws, hs = s * wo, s * wo // 2
    L = _level(ws, hs, s)
    lvl = np.concatenate([L, np.ones((hs, ws, 1))], -1).astype(np.float32)
    L = lvl[..., :3].astype(np.float64)  # the radiance the kernels read (float32)
    xy = np.stack(np.meshgrid(np.arange(wo), np.arange(ho)), -1).reshape(-1, 2).astype(np.int32)
    for r in (0.3, 1.0):
        W = weight_table(ws, hs, wo, ho, r)
        ref = direct(W, L, s) / W.sum(axis=(1, 2))[:, None, None]
        got = contraction(W, L, s) / W.sum(axis=(1, 2))[:, None, None]
        assert np.allclose(got, ref, rtol=1e-12, atol=0), (s, r)
        q = oracle.quad_prefilter(lvl, wo, ho, r, xy)[:, :3].reshape(ho, wo, 3)
        assert np.allclose(ref, q, rtol=1e-9, atol=0), (s, r, np.abs(ref / q - 1).max())
    Wi = weight_table(ws, hs, wo, ho, 0.0, ggx=False)
    qi = oracle.quad_irradiance(lvl, wo, ho, xy)[:, :3].reshape(ho, wo, 3)
    assert np.allclose(contraction(Wi, L, s), qi, rtol=1e-9, atol=1e-12 * qi.max())


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, 3.0 + 2 ** -7],
                 dtype=np.float32)
    got = bf16(x)
    assert list(got) == [1.0, 1.0, 1.0 + 2 ** -6, 1.0, 3.0]
    # hi + lo carries 16 significant bits
    v = np.float32(np.pi)
    hi, lo = hi_lo(v)
    assert abs(hi + lo - float(v)) <= 2 ** -16 * float(v)


@pytest.mark.parametrize("s", [2, 3, 8])
def test_hi_lo_split_stays_within_1e4(s):
    """Three BF16 products per term, summed exactly: every term is
    non-negative, so the relative error of a sum is at most the worst term's
    (about 3 * 2^-16).  The kernel accumulates in FP32 on top of this."""
    wo, ho = 16, 8
    ws, hs = s * wo, s * wo // 2
    L = _level(ws, hs, 100 + s).astype(np.float32).astype(np.float64)
    for r in (0.25, 0.75):
        W = weight_table(ws, hs, wo, ho, r)
        exact = contraction(W, L, s)
        split = contraction(W, L, s, split=hi_lo)
        rel = np.abs(split - exact) / exact
        assert rel.max() <= 3 * 2.0 ** -16, rel.max()
        # a single BF16 product would not do: its error is about 2^-8
        single = contraction(W, L, s, split=lambda a: (bf16(a).astype(np.float64),
                                                        np.zeros_like(a, dtype=np.float64)))
        assert (np.abs(single - exact) / exact).max() > 1e-3
