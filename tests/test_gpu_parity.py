"""GPU parity: every CUDA kernel against the CPU oracle through the C ABI.

Tolerance: 1e-4 relative per texel and channel (|gpu - ref| / max(|ref|,
1e-6 * max|ref|)), the bar of the plain path.  The prefilter, the env chain
and the LUT are expected to be bit-identical (the kernels evaluate the same
IEEE operations in the same order as the oracle); the irradiance sum is split
across threads, so it differs from the serial sum by float rounding only.
"""
import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    floor = 1e-6 * np.max(np.abs(ref))
    return np.abs(got - ref) / np.maximum(np.abs(ref), floor)


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def run_prefilter(chain_d, w, h, sizes, rough, samples, gen):
    outs = [torch.empty((oh, ow, 4), dtype=torch.float32, device="cuda") for ow, oh in sizes]
    ibl.prefilter(chain_d, w, h, outs, rough, samples, gen)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("w,h", [(512, 256), (64, 32), (37, 19), (1, 1), (256, 1), (3, 100)])
def test_env_chain_bit_exact(w, h):
    env = synth.make_tinted_env(w, h, seed=w * 7 + h)
    ref = oracle.build_chain(env)
    got = ibl.build_env_chain(to_dev(env))
    torch.cuda.synchronize()
    assert got.shape[0] == ref.shape[0] == oracle.chain_texels(w, h)
    assert np.array_equal(got.cpu().numpy(), ref)


@pytest.mark.parametrize("gen,tag", [(ibl.GEN_REF_HASH, "hash"), (ibl.GEN_HAMMERSLEY, "hammersley")])
def test_prefilter_matches_reference_shader_golden(golden, gen, tag):
    env = golden["env"]
    h, w = env.shape[:2]
    chain_d = ibl.build_env_chain(to_dev(env))
    sizes = [(w >> (m + 1), h >> (m + 1)) for m in range(5)]
    outs = run_prefilter(chain_d, w, h, sizes, [m / 4.0 for m in range(5)], 1024, gen)
    for m, got in enumerate(outs):
        ref = golden[f"prefilter_{tag}_n1024_m{m}"]
        assert rel_err(got, ref).max() <= TOL, (m, rel_err(got, ref).max())
        assert np.array_equal(got, ref), f"mip {m} not bit-identical"


def test_prefilter_reference_sample_count_golden(golden):
    env = golden["env"]
    h, w = env.shape[:2]
    chain_d = ibl.build_env_chain(to_dev(env))
    for m in (1, 3):
        got = run_prefilter(chain_d, w, h, [(w >> (m + 1), h >> (m + 1))], [m / 4.0], 10000,
                            ibl.GEN_REF_HASH)[0]
        ref = golden[f"prefilter_hash_n10000_m{m}"]
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("gen", [ibl.GEN_REF_HASH, ibl.GEN_HAMMERSLEY])
def test_prefilter_small_config_all_texels(gen):
    # 512x256 map, 5 mips 256x128 .. 16x8, roughness i/4, N = 1024.
    w, h = 512, 256
    env = synth.make_env(w, h, seed=0, sun_max=1e4)
    chain = oracle.build_chain(env)
    chain_d = to_dev(chain)
    sizes = [(w >> (m + 1), h >> (m + 1)) for m in range(5)]
    rough = [m / 4.0 for m in range(5)]
    outs = run_prefilter(chain_d, w, h, sizes, rough, 1024, gen)
    for m, ((ow, oh), r) in enumerate(zip(sizes, rough)):
        ref = oracle.prefilter(chain, w, h, ow, oh, r, 1024, gen)
        err = rel_err(outs[m], ref)
        assert err.max() <= TOL, (m, err.max())
        assert np.isfinite(outs[m]).all()


def test_irradiance_small_config_all_texels():
    w, h = 512, 256
    env = synth.make_env(w, h, seed=0, sun_max=1e4)
    chain = oracle.build_chain(env)
    out = torch.empty((16, 32, 4), dtype=torch.float32, device="cuda")
    ibl.irradiance(to_dev(chain), w, h, out)
    torch.cuda.synchronize()
    ref = oracle.irradiance(chain, w, h, 32, 16)
    err = rel_err(out.cpu().numpy(), ref)
    assert err.max() <= TOL, err.max()


def test_irradiance_env_size_golden(golden):
    # The reference dispatches irradiance at env size (Src/ImageBasedLighting.cpp:208-221).
    env = golden["env"]
    h, w = env.shape[:2]
    chain_d = ibl.build_env_chain(to_dev(env))
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    ibl.irradiance(chain_d, w, h, out)
    torch.cuda.synchronize()
    err = rel_err(out.cpu().numpy(), golden["irradiance_envsize"])
    assert err.max() <= TOL, err.max()


@pytest.mark.parametrize("orientation", [ibl.LUT_ASSET, ibl.LUT_CORRECTED])
def test_brdf_lut_bit_exact(orientation):
    got = ibl.brdf_lut(256, 1024, orientation)
    torch.cuda.synchronize()
    ref = oracle.brdf_lut_f32(256, 1024, orientation)
    assert np.array_equal(got.cpu().numpy(), ref)


def test_context_bake_equals_stateless():
    w, h = 512, 256
    env = synth.make_env(w, h, seed=5)
    cfg = ibl.make_config(w, h, irradiance_size=(32, 16), mip_count=5, samples=1024,
                          lut_size=64, lut_samples=256)
    ctx = ibl.BakeContext(cfg)
    ctx.upload_env(torch.from_numpy(env))  # host source
    irr, mips, lut = ctx.allocate_outputs()
    ctx.bake(irr, mips, lut)
    torch.cuda.synchronize()
    chain = oracle.build_chain(env)
    assert np.array_equal(ctx.chain().cpu().numpy(), chain)
    for m in range(5):
        mw, mh, r = ctx.mip_info(m)
        assert (mw, mh, r) == (w >> (m + 1), h >> (m + 1), m / 4.0)
        ref = oracle.prefilter(chain, w, h, mw, mh, r, 1024, oracle.GEN_REF_HASH)
        assert np.array_equal(mips[m].cpu().numpy(), ref)
    ref_irr = oracle.irradiance(chain, w, h, 32, 16)
    assert rel_err(irr.cpu().numpy(), ref_irr).max() <= TOL
    assert np.array_equal(lut.cpu().numpy(), oracle.brdf_lut_f32(64, 256, oracle.LUT_ASSET))
    ctx.close()


def test_create_resources_interface():
    w, h = 128, 64
    env = synth.make_env(w, h, seed=2)
    cfg = ibl.make_config(w, h, samples=256, lut_size=32, lut_samples=64)
    res = ibl.ImageBasedLighting.createResources(torch.from_numpy(env), cfg)
    assert tuple(res.irradianceMap.shape) == (h, w, 4)  # reference: env-sized irradiance
    assert [tuple(m.shape) for m in res.prefilteredMap] == [
        (h >> (m + 1), w >> (m + 1), 4) for m in range(5)]
    assert np.array_equal(res.environmentMap.cpu().numpy(), env)
    bound = res.bind([])
    assert len(bound) == 4 and bound[0] is res.environmentMap and bound[3] is res.brdfLut
    heap = []
    res.registerToHeap(heap)
    assert res.getHandles() == (0, 1, 2, 3)


@pytest.mark.parametrize("gen", [ibl.GEN_REF_HASH, ibl.GEN_HAMMERSLEY])
def test_production_size_sampled_texels(gen):
    # 4096x2048 map, 9 mips from 2048x1024 (roughness m/8), 128x64 irradiance,
    # N = 1024: sampled texels against the oracle (every texel is too slow for
    # the oracle), plus seam, pole rows and corners; bit-identical.  The
    # Hammersley generator takes its own code path in the kernel (the sample
    # half-vectors tabulated once per block in shared memory).
    w, h = 4096, 2048
    env = synth.make_env(w, h, seed=0, sun_max=1e4)
    chain = oracle.build_chain(env)
    chain_d = to_dev(chain)
    got_chain = ibl.build_env_chain(to_dev(env))
    torch.cuda.synchronize()
    assert torch.equal(got_chain, chain_d)
    sizes = [(2048 >> m, 1024 >> m) for m in range(9)]
    rough = [m / 8.0 for m in range(9)]
    outs = run_prefilter(chain_d, w, h, sizes, rough, 1024, gen)
    rng = np.random.default_rng(1 + gen)
    for m, ((ow, oh), r) in enumerate(zip(sizes, rough)):
        n = 160
        xs = rng.integers(0, ow, n)
        ys = rng.integers(0, oh, n)
        extra = np.array([[0, 0], [ow - 1, oh - 1], [0, oh - 1], [ow - 1, 0], [ow // 2, 0],
                          [0, oh // 2], [ow // 2, oh // 2]])
        xy = np.concatenate([np.stack([xs, ys], 1), extra]).astype(np.int32)
        ref = oracle.prefilter(chain, w, h, ow, oh, r, 1024, gen, xy=xy)
        got = outs[m][xy[:, 1], xy[:, 0]]
        err = rel_err(got, ref)
        assert err.max() <= TOL, (m, err.max())
        assert np.array_equal(got, ref), f"mip {m} not bit-identical"
        assert np.isfinite(outs[m]).all() and (outs[m][..., :3] > 0).all()
    irr = torch.empty((64, 128, 4), dtype=torch.float32, device="cuda")
    ibl.irradiance(chain_d, w, h, irr)
    irr2 = torch.empty_like(irr)
    ibl.irradiance(chain_d, w, h, irr2)
    torch.cuda.synchronize()
    assert torch.equal(irr, irr2)  # deterministic split reduction
    xy = np.array([[0, 0], [127, 63], [64, 32], [5, 60], [100, 3], [31, 17]], dtype=np.int32)
    ref = oracle.irradiance(chain, w, h, 128, 64, xy=xy)
    got = irr.cpu().numpy()[xy[:, 1], xy[:, 0]]
    assert rel_err(got, ref).max() <= TOL


def test_invalid_arguments_rejected():
    L = ibl.load()
    buf = torch.empty((8, 8, 4), dtype=torch.float32, device="cuda")
    arr = (ibl.MipTarget * 1)()
    arr[0] = ibl.MipTarget(buf.data_ptr(), 8 * 16, 8, 8, 1.5)  # roughness > 1
    assert L.althea_ibl_prefilter(buf.data_ptr(), 8, 8, arr, 1, 64, 0, None) == ibl.ERR_INVALID_ARGUMENT
    assert b"roughness" in L.althea_ibl_last_error()
    arr[0] = ibl.MipTarget(buf.data_ptr(), 8, 8, 8, 0.5)  # pitch too small
    assert L.althea_ibl_prefilter(buf.data_ptr(), 8, 8, arr, 1, 64, 0, None) == ibl.ERR_INVALID_ARGUMENT
    # irradiance grid int(300*H/W) = 0 for a 1000x1 map
    assert L.althea_ibl_irradiance(buf.data_ptr(), 1000, 1, buf.data_ptr(), 8, 8, 128,
                                   buf.data_ptr(), 1 << 20, None) == ibl.ERR_UNSUPPORTED
    cfg = ibl.make_config(64, 32, samples=16)
    ctx = ibl.BakeContext(cfg)
    irr, mips, lut = ctx.allocate_outputs()
    with pytest.raises(ibl.IBLError) as e:
        ctx.bake(irr, mips, lut)
    assert e.value.status == ibl.ERR_NOT_READY
    ctx.close()
