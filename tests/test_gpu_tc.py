"""GPU tests of the precision path (tcgen05 BF16 hi/lo contraction).

1. The kernel computes the planned quadrature: against the FP64 oracle summed
   over the same source level, within SAME_LEVEL_TOL = 3e-4 relative (BF16
   hi/lo products are good to ~2^-17; the rest is the FP32 tensor-core
   accumulation, whose error grows with the MMAs summed into one accumulator:
   up to 1,500-2,000 of them for K = 32768, measured at up to 2.3e-4).  An
   indexing or weight error shows as far more than 1e-3.
2. The plan keeps the result within 1e-3 of the FP64 quadrature over level 0
   (the contract of the precision path).
"""
import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _rel(got, ref):
    return np.abs(got - ref) / np.abs(ref)


SAME_LEVEL_TOL = 3e-4

# (env w, h, mip sizes, roughness, source levels, irradiance size, irradiance level).
# The source/output width ratios s cover every decomposition of the kernel:
# s = 1, 2, 4 (column residues), s = 8, s = 16, 32 (phase rows), s = 3 (both),
# output heights above one 128-row tile (ragged), and tiny outputs.
SAME_LEVEL_CASES = [
    (512, 256, [(128, 64), (64, 32), (16, 8), (256, 128)], [0.25, 0.5, 1.0, 0.125],
     [1, 1, 2, 1], (32, 16), 2),
    (384, 192, [(128, 64), (24, 12), (12, 6), (96, 48), (384, 192), (4, 2)],
     [0.3, 0.6, 0.9, 0.2, 0.15, 1.0], [0, 0, 0, 1, 0, 1], (24, 12), 0),
]


@pytest.mark.parametrize("case", range(len(SAME_LEVEL_CASES)))
def test_contraction_matches_fp64_quadrature_at_same_source_level(case):
    w, h, sizes, rough, levels, (iw, ih), ilv = SAME_LEVEL_CASES[case]
    env = synth.make_env(w, h, seed=8 + case, sun_max=1e6)
    chain = oracle.build_chain(env)
    chain_d = torch.from_numpy(chain).cuda()
    outs = [torch.empty((mh, mw, 4), dtype=torch.float32, device="cuda") for mw, mh in sizes]
    irr = torch.empty((ih, iw, 4), dtype=torch.float32, device="cuda")
    ibl.bake_tc(chain_d, w, h, outs, rough, irradiance=irr, levels=levels, irradiance_level=ilv)
    torch.cuda.synchronize()
    rng = np.random.default_rng(case)
    for (mw, mh), r, lv, o in zip(sizes, rough, levels, outs):
        src = oracle.chain_level(chain, w, h, lv)
        n = min(mw * mh, 256)
        idx = rng.choice(mw * mh, size=n, replace=False)
        xy = np.stack([idx % mw, idx // mw], 1).astype(np.int32)
        ref = oracle.quad_prefilter(src, mw, mh, r, xy)[:, :3]
        got = o.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        assert _rel(got, ref).max() <= SAME_LEVEL_TOL, (mw, r, _rel(got, ref).max())
    src = oracle.chain_level(chain, w, h, ilv)
    ys, xs = np.mgrid[0:ih, 0:iw]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    ref = oracle.quad_irradiance(src, iw, ih, xy)[:, :3]
    got = irr.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
    assert _rel(got, ref).max() <= SAME_LEVEL_TOL, _rel(got, ref).max()


def test_plan_meets_1e3_against_level0_quadrature():
    w, h = 1024, 512
    env = synth.make_env(w, h, seed=2, sun_max=1e6)
    chain = oracle.build_chain(env)
    chain_d = torch.from_numpy(chain).cuda()
    sizes = [(512 >> m, 256 >> m) for m in range(7)]
    rough = [m / 6 for m in range(7)]
    outs = [torch.empty((mh, mw, 4), dtype=torch.float32, device="cuda") for mw, mh in sizes]
    irr = torch.empty((32, 64, 4), dtype=torch.float32, device="cuda")
    ibl.bake_tc(chain_d, w, h, outs, rough, irradiance=irr)
    torch.cuda.synchronize()
    rng = np.random.default_rng(1)
    lvl0 = oracle.chain_level(chain, w, h, 0)
    for (mw, mh), r, o in zip(sizes[1:], rough[1:], outs[1:]):
        n = min(mw * mh, 48)
        idx = rng.choice(mw * mh, size=n, replace=False)
        xy = np.stack([idx % mw, idx // mw], 1).astype(np.int32)
        ref = oracle.quad_prefilter(lvl0, mw, mh, r, xy)[:, :3]
        got = o.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        assert _rel(got, ref).max() <= 1e-3, (mw, r, _rel(got, ref).max())
    # roughness 0 is a delta: the reflected sample itself, which the reference
    # estimator reaches after summing 1024 identical samples in FP32
    ref0 = oracle.prefilter(chain, w, h, 512, 256, 0.0, 1024, oracle.GEN_HAMMERSLEY)
    assert _rel(outs[0].cpu().numpy()[..., :3], ref0[..., :3]).max() <= 1e-4
    idx = rng.choice(64 * 32, size=48, replace=False)
    xy = np.stack([idx % 64, idx // 64], 1).astype(np.int32)
    ref = oracle.quad_irradiance(lvl0, 64, 32, xy)[:, :3]
    got = irr.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
    assert _rel(got, ref).max() <= 1e-3, _rel(got, ref).max()


@pytest.mark.parametrize("sun_max", [1e4, 1e6])
def test_small_probe_every_texel_against_fp64(sun_max):
    """The 512x256 probe (5 mips of roughness m/4 from 256x128, 32x16
    irradiance) through the default plan, every output texel against the FP64
    quadrature over level 0 (the CPU oracle sums all 131072 source texels)."""
    w, h = 512, 256
    env = synth.make_env(w, h, seed=0, sun_max=sun_max)
    chain = oracle.build_chain(env)
    sizes = [(256 >> m, 128 >> m) for m in range(5)]
    rough = [m / 4 for m in range(5)]
    outs = [torch.full((mh, mw, 4), float("nan"), device="cuda") for mw, mh in sizes]
    irr = torch.full((16, 32, 4), float("nan"), device="cuda")
    ibl.bake_tc(torch.from_numpy(chain).cuda(), w, h, outs, rough, irradiance=irr)
    torch.cuda.synchronize()
    lvl0 = oracle.chain_level(chain, w, h, 0)
    for (mw, mh), r, o in zip(sizes[1:], rough[1:], outs[1:]):
        ys, xs = np.mgrid[0:mh, 0:mw]
        xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
        ref = oracle.quad_prefilter(lvl0, mw, mh, r, xy)[:, :3]
        got = o.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        assert np.isfinite(got).all()
        assert _rel(got, ref).max() <= 1e-3, (mw, r, _rel(got, ref).max())
    ref0 = oracle.prefilter(chain, w, h, 256, 128, 0.0, 1024, oracle.GEN_HAMMERSLEY)
    assert _rel(outs[0].cpu().numpy()[..., :3], ref0[..., :3]).max() <= 1e-4
    ys, xs = np.mgrid[0:16, 0:32]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    ref = oracle.quad_irradiance(lvl0, 32, 16, xy)[:, :3]
    got = irr.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
    assert np.isfinite(got).all() and _rel(got, ref).max() <= 1e-3, _rel(got, ref).max()


def test_half_outputs_are_the_float_outputs_rounded():
    w, h = 256, 128
    env = synth.make_env(w, h, seed=12, sun_max=1e6)
    chain = ibl.build_env_chain(torch.from_numpy(env).cuda())
    sizes = [(128, 64), (64, 32), (16, 8)]
    rough = [0.0, 0.4, 1.0]
    f32 = [torch.empty((mh, mw, 4), dtype=torch.float32, device="cuda") for mw, mh in sizes]
    f16 = [torch.empty((mh, mw, 4), dtype=torch.float16, device="cuda") for mw, mh in sizes]
    irr32 = torch.empty((16, 32, 4), dtype=torch.float32, device="cuda")
    irr16 = torch.empty((16, 32, 4), dtype=torch.float16, device="cuda")
    ibl.bake_tc(chain, w, h, f32, rough, irradiance=irr32)
    ibl.bake_tc(chain, w, h, f16, rough, irradiance=irr16)
    torch.cuda.synchronize()
    for a, b in zip(f32, f16):
        assert torch.equal(a.half(), b)
    assert torch.equal(irr32.half(), irr16)
    with pytest.raises(ibl.IBLError):  # mixed output types
        ibl.bake_tc(chain, w, h, [f32[0], f16[1]], rough[:2])


def test_single_bright_texel_gives_the_ggx_lobe():
    """Known answer through the tensor-core contraction: an env that is 0 but
    for one texel prefilters to L w(n, t0) / sum_t w(n, t) (the normalised GGX
    weight, written in numpy in tests/test_oracle.py)."""
    from test_oracle import single_texel_lobe
    w, h, L = 256, 128, 1000.0
    x0, y0 = 85, 51
    env = np.zeros((h, w, 4), dtype=np.float32)
    env[y0, x0, :3] = L
    env[..., 3] = 1.0
    chain = ibl.build_env_chain(torch.from_numpy(env).cuda())
    sizes, rough = [(64, 32), (32, 16)], [0.3, 0.8]
    outs = [torch.empty((mh, mw, 4), dtype=torch.float32, device="cuda") for mw, mh in sizes]
    ibl.bake_tc(chain, w, h, outs, rough, levels=[0, 0])
    torch.cuda.synchronize()
    for (mw, mh), r, o in zip(sizes, rough, outs):
        ys, xs = np.mgrid[0:mh, 0:mw]
        xy = np.stack([xs.ravel(), ys.ravel()], 1)
        ref = L * single_texel_lobe(w, h, mw, mh, r, x0, y0, xy)
        got = o.cpu().numpy()[..., 0].ravel()
        assert np.allclose(got, ref, rtol=1e-4, atol=1e-6 * L), (r, np.abs(got - ref).max())
        assert ref.max() > 1e-4 * L  # one texel of 32768 carries a visible share


def test_narrow_outputs_on_wide_source_levels():
    """Outputs of <= 128 texels are summed on the CUDA cores; check them (and a
    narrow irradiance) against the FP64 quadrature over a 2048-wide source."""
    w, h = 2048, 1024
    env = synth.make_env(w, h, seed=21, sun_max=1e6)
    chain_np = oracle.build_chain(env)
    chain = torch.from_numpy(chain_np).cuda()
    sizes, rough = [(32, 16), (16, 8), (8, 4), (4, 2)], [0.75, 0.875, 1.0, 0.6]
    outs = [torch.full((mh, mw, 4), float("nan"), device="cuda") for mw, mh in sizes]
    irr = torch.full((4, 8, 4), float("nan"), device="cuda")
    ibl.bake_tc(chain, w, h, outs, rough, irradiance=irr, levels=[0, 0, 0, 0],
                irradiance_level=0)
    torch.cuda.synchronize()
    lvl0 = oracle.chain_level(chain_np, w, h, 0)
    for (mw, mh), r, o in zip(sizes, rough, outs):
        ys, xs = np.mgrid[0:mh, 0:mw]
        xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
        ref = oracle.quad_prefilter(lvl0, mw, mh, r, xy)[:, :3]
        got = o.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        assert np.isfinite(got).all()
        # FP32 weights on the CUDA cores (<= 128 texels); BF16 hi/lo beyond
        tol = 1e-5 if mw * mh <= 128 else SAME_LEVEL_TOL
        assert _rel(got, ref).max() <= tol, (mw, _rel(got, ref).max())
    ys, xs = np.mgrid[0:4, 0:8]
    xy = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    ref = oracle.quad_irradiance(lvl0, 8, 4, xy)[:, :3]
    got = irr.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
    assert np.isfinite(got).all() and _rel(got, ref).max() <= 1e-5
    # the CUDA-core outputs alone: a bake with no contraction job (no queue
    # launch) writes the same texels
    only = [torch.full((mh, mw, 4), float("nan"), device="cuda") for mw, mh in sizes[1:]]
    irr2 = torch.full((4, 8, 4), float("nan"), device="cuda")
    ibl.bake_tc(chain, w, h, only, rough[1:], irradiance=irr2, levels=[0, 0, 0],
                irradiance_level=0)
    torch.cuda.synchronize()
    for a, b in zip(only, outs[1:]):
        assert torch.equal(a, b)
    assert torch.equal(irr2, irr)


def test_bounded_wait_gives_up_and_reports():
    """Failure detection without a fault: the kernel's mbarrier wait on a
    barrier that nothing completes gives up after its limit, raises the abort
    flag and returns; the context stays usable for a normal bake after it."""
    waited = ibl.tc_wait_selftest(limit_ms=20.0)
    assert 20 <= waited < 1000
    test_half_outputs_are_the_float_outputs_rounded()



@pytest.mark.parametrize("fmt", [ibl.FORMAT_RGBA32F, ibl.FORMAT_RGBA16F])
def test_context_precision_bake_equals_stateless_bake(fmt):
    """The createResources mirror on the precision path: the bake context plans
    the contraction and holds its workspace itself, and writes what the
    stateless bake_tc writes with the planner's levels, bit for bit, in either
    output format (RGBA16F = the RGBA32F result rounded)."""
    w, h = 1024, 512
    env = synth.make_env(w, h, seed=4, sun_max=1e6)
    env_d = torch.from_numpy(env).cuda()
    cfg = ibl.make_config(w, h, irradiance_size=(32, 16), mip_count=7, lut_size=64,
                          lut_samples=64, path=ibl.PATH_PRECISION, out_format=fmt)
    ctx = ibl.BakeContext(cfg)
    assert ctx.device_bytes() > ibl.chain_texels(w, h) * 16
    ctx.upload_env(env_d)
    irr, mips, lut = ctx.allocate_outputs()
    want = torch.float16 if fmt == ibl.FORMAT_RGBA16F else torch.float32
    assert irr.dtype == want and all(m.dtype == want for m in mips)
    ctx.bake(irr, mips, lut, check=True)
    rough = [ctx.mip_info(m)[2] for m in range(7)]
    chain = ibl.build_env_chain(env_d)
    ref_mips = [torch.empty(m.shape, dtype=torch.float32, device="cuda") for m in mips]
    ref_irr = torch.empty(irr.shape, dtype=torch.float32, device="cuda")
    ibl.bake_tc(chain, w, h, ref_mips, rough, irradiance=ref_irr)
    torch.cuda.synchronize()
    assert torch.equal(ctx.chain(), chain)
    for a, b in zip(mips, ref_mips):
        assert torch.equal(a, b.to(want))
    assert torch.equal(irr, ref_irr.to(want))
    assert torch.equal(lut, ibl.brdf_lut(64, 64, ibl.LUT_ASSET))
    with pytest.raises(ibl.IBLError):  # the other format is refused
        other = torch.float32 if want == torch.float16 else torch.float16
        ctx.bake(irr.to(other), [m.to(other) for m in mips], lut)
    ctx.close()
    res = ibl.ImageBasedLighting.createResources(env_d, cfg)
    assert torch.equal(res.prefilteredMap[3], ref_mips[3].to(want))
    assert torch.equal(res.irradianceMap, ref_irr.to(want))


def test_queue_launch_with_the_most_contraction_jobs():
    """The largest plan the C ABI admits: 16 mips and the irradiance, each a
    contraction of its own (128 rows: no pairs, no K interleave), so the
    bake's queue launch holds 17 jobs (136 work items).  Every output matches
    the FP64 quadrature over level 0 within the same-level bound."""
    w, h = 512, 256
    env = synth.make_env(w, h, seed=12, sun_max=1e6)
    chain_d = torch.from_numpy(oracle.build_chain(env)).cuda()
    n = 16
    rough = [0.2 + 0.05 * k for k in range(n)]
    outs = [torch.empty((128, 256, 4), dtype=torch.float32, device="cuda") for _ in range(n)]
    irr = torch.empty((128, 256, 4), dtype=torch.float32, device="cuda")
    ibl.bake_tc(chain_d, w, h, outs, rough, irradiance=irr, levels=[0] * n, irradiance_level=0)
    torch.cuda.synchronize()
    rng = np.random.default_rng(12)
    idx = rng.choice(256 * 128, size=32, replace=False)
    xy = np.stack([idx % 256, idx // 256], 1).astype(np.int32)
    for r, o in zip(rough, outs):
        ref = oracle.quad_prefilter(env, 256, 128, r, xy)[:, :3]
        got = o.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
        assert _rel(got, ref).max() <= SAME_LEVEL_TOL, (r, _rel(got, ref).max())
    ref = oracle.quad_irradiance(env, 256, 128, xy)[:, :3]
    got = irr.cpu().numpy()[xy[:, 1], xy[:, 0], :3]
    assert _rel(got, ref).max() <= SAME_LEVEL_TOL, _rel(got, ref).max()


def test_context_rebake_with_another_map_equals_stateless_bake():
    """A context re-baked with a different map (its queue counter, error word
    and tables reused from the first bake) writes the second map's stateless
    bake bit for bit, not the first map's."""
    w, h = 512, 256
    cfg = ibl.make_config(w, h, irradiance_size=(32, 16), mip_count=6, path=ibl.PATH_PRECISION)
    ctx = ibl.BakeContext(cfg)
    irr, mips, _ = ctx.allocate_outputs()
    envs = [torch.from_numpy(synth.make_env(w, h, seed=20 + k, sun_max=1e6)).cuda()
            for k in range(2)]
    rough = [ctx.mip_info(m)[2] for m in range(6)]
    for env_d in envs:
        ctx.upload_env(env_d)
        ctx.bake(irr, mips, None, check=True)
        ref_mips = [torch.empty_like(m) for m in mips]
        ref_irr = torch.empty_like(irr)
        ibl.bake_tc(ibl.build_env_chain(env_d), w, h, ref_mips, rough, irradiance=ref_irr)
        torch.cuda.synchronize()
        assert all(torch.equal(a, b) for a, b in zip(mips, ref_mips))
        assert torch.equal(irr, ref_irr)
    ctx.close()


def test_context_times_its_contraction_launch():
    """A precision context records CUDA events around its contraction launch
    (one queue launch per bake): one positive device time per bake, oldest
    first, the last TIMED_BAKES kept, each below the bake's own time; a
    plain-path context has none to give."""
    w, h = 512, 256
    env_d = torch.from_numpy(synth.make_env(w, h, seed=6, sun_max=1e6)).cuda()
    ctx = ibl.BakeContext(ibl.make_config(w, h, irradiance_size=(32, 16), mip_count=6,
                                          path=ibl.PATH_PRECISION))
    ctx.upload_env(env_d)
    irr, mips, lut = ctx.allocate_outputs()
    assert ctx.contraction_times() == []
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(3):
        ctx.bake(irr, mips, lut)
    e.record()
    t = ctx.contraction_times()
    assert len(t) == 3 and all(0 < x for x in t)
    assert sum(t) < s.elapsed_time(e)
    for _ in range(ibl.TIMED_BAKES):
        ctx.bake(irr, mips, lut)
    assert len(ctx.contraction_times()) == ibl.TIMED_BAKES
    ctx.status()
    ctx.close()
    plain = ibl.BakeContext(ibl.make_config(w, h, irradiance_size=(32, 16), mip_count=6))
    with pytest.raises(ibl.IBLError):
        plain.contraction_times()
    plain.close()


def test_two_product_split_on_low_roughness_planned_mips():
    """With planner-chosen levels, GGX mips of roughness <= 0.25 take the
    two-product split (BF16 hi weights, normalised by the sum of the rounded
    weights); the same levels named by the caller take three products.  On a
    2048x1024 probe with 1e6 suns: mip 1 (roughness 1/7) differs between the
    two by the weight rounding only, both stay within 1e-3 of the FP64
    quadrature over level 0, and every other output is bit-identical."""
    spec = ibl.spec_for(2048, 1024)
    w, h = 2048, 1024
    env = synth.make_env(w, h, seed=3, sun_max=1e6)
    chain = ibl.build_env_chain(torch.from_numpy(env).cuda())
    levels, il = ibl.tc_plan(w, h, spec.mip_sizes, spec.roughness, 32)

    def bake(lv, ilv):
        outs = [torch.empty((mh, mw, 4), dtype=torch.float32, device="cuda")
                for mw, mh in spec.mip_sizes]
        irr = torch.empty((16, 32, 4), dtype=torch.float32, device="cuda")
        ibl.bake_tc(chain, w, h, outs, spec.roughness, irradiance=irr, levels=lv,
                    irradiance_level=ilv)
        torch.cuda.synchronize()
        return [o.cpu().numpy() for o in outs], irr.cpu().numpy()

    two, irr_a = bake(None, -1)
    three, irr_b = bake(levels, il)
    assert np.array_equal(irr_a, irr_b)
    rng = np.random.default_rng(5)
    for m, r in enumerate(spec.roughness):
        if r == 0.0 or r > 0.25:
            assert np.array_equal(two[m], three[m]), m
            continue
        assert not np.array_equal(two[m], three[m])
        d = np.abs(two[m][..., :3] - three[m][..., :3]) / np.abs(three[m][..., :3])
        assert d.max() <= 1e-3, d.max()
        mw, mh = spec.mip_sizes[m]
        idx = rng.choice(mw * mh, size=192, replace=False)
        xy = np.stack([idx % mw, idx // mw], 1).astype(np.int32)
        ref = oracle.quad_prefilter(env, mw, mh, r, xy)[:, :3]
        for img in (two[m], three[m]):
            assert _rel(img[xy[:, 1], xy[:, 0], :3], ref).max() <= 1e-3
