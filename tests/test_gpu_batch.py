"""GPU tests of batched bakes (many probes of uneven size in one graph launch):
every output equals baking that probe alone through the stateless calls."""
import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _solo(spec, env_d, samples, generator):
    chain = ibl.build_env_chain(env_d)
    mips = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for w, h in spec.mip_sizes]
    ibl.prefilter(chain, spec.env_width, spec.env_height, mips, spec.roughness, samples, generator)
    irr = None
    if spec.irradiance_size is not None:
        iw, ih = spec.irradiance_size
        irr = torch.empty((ih, iw, 4), dtype=torch.float32, device="cuda")
        ibl.irradiance(chain, spec.env_width, spec.env_height, irr)
    return chain, mips, irr


@pytest.mark.parametrize("graph,autotune", [(True, True), (False, False)])
@pytest.mark.parametrize("generator", [ibl.GEN_HAMMERSLEY, ibl.GEN_REF_HASH])
def test_batch_equals_probes_alone(graph, autotune, generator):
    sizes = [(256, 128), (64, 32), (128, 64), (256, 128), (32, 16), (128, 64), (512, 256)]
    specs = [ibl.spec_for(w, h) for w, h in sizes]
    specs[4] = ibl.spec_for(32, 16, mip_count=3, irradiance_size=(8, 4))
    specs[5].irradiance_size = None  # a probe without irradiance
    envs = [torch.from_numpy(synth.make_env(w, h, seed=40 + i)).cuda()
            for i, (w, h) in enumerate(sizes)]
    stream = torch.cuda.Stream()
    batch = ibl.ProbeBatch(specs, envs, samples=256, generator=generator, lut_size=64,
                           lut_samples=128, autotune=autotune, graph=graph, stream=stream)
    for _ in range(2):  # second run replays the graph
        batch.run(stream)
    stream.synchronize()
    info = batch.info()
    assert info.probes == len(specs)
    assert info.graph == (1 if graph else 0)
    assert info.tuned == (1 if autotune else 0) or autotune is False
    for i, (s, env) in enumerate(zip(specs, envs)):
        chain, mips, irr = _solo(s, env, 256, generator)
        torch.cuda.synchronize()
        assert torch.equal(batch.chains[i], chain), i
        for m in range(len(mips)):
            assert torch.equal(batch.mips[i][m], mips[m]), (i, m)
        if irr is not None:
            assert torch.equal(batch.irradiance[i], irr), i
    ref_lut = oracle.brdf_lut_f32(64, 128, oracle.LUT_ASSET)
    assert np.array_equal(batch.lut.cpu().numpy(), ref_lut)
    batch.close()


def test_batch_matches_oracle_on_one_probe():
    w, h = 128, 64
    spec = ibl.spec_for(w, h)
    env = synth.make_env(w, h, seed=77)
    batch = ibl.ProbeBatch([spec], [torch.from_numpy(env).cuda()], samples=128, autotune=False)
    batch.run()
    torch.cuda.synchronize()
    chain = oracle.build_chain(env)
    for m, ((mw, mh), r) in enumerate(zip(spec.mip_sizes, spec.roughness)):
        ref = oracle.prefilter(chain, w, h, mw, mh, r, 128, oracle.GEN_HAMMERSLEY)
        assert np.array_equal(batch.mips[0][m].cpu().numpy(), ref)
    batch.close()


def test_autotune_choice_is_cached_per_shape():
    specs = [ibl.spec_for(64, 32), ibl.spec_for(128, 64)]
    envs = [torch.from_numpy(synth.make_env(s.env_width, s.env_height, seed=3)).cuda()
            for s in specs]
    a = ibl.ProbeBatch(specs, envs, samples=64, autotune=True, graph=False)
    b = ibl.ProbeBatch(specs[::-1], envs[::-1], samples=64, autotune=True, graph=False)
    ia, ib = a.info(), b.info()
    assert ia.tuned == 1 and ib.tuned == 1
    assert (ia.tile_x, ia.tile_y, ia.irradiance_target_blocks) == \
        (ib.tile_x, ib.tile_y, ib.irradiance_target_blocks)
    a.close()
    b.close()


@pytest.mark.parametrize("half", [False, True])
def test_precision_batch_equals_probes_alone(half):
    """The precision path in a batch (one graph: the split passes of every
    probe, one persistent contraction kernel over the work items of every
    probe, every probe's finish) gives every probe exactly its solo
    tensor-core bake (whose contractions are one queue launch of the same
    work items); RGBA16F outputs are the RGBA32F results rounded to half.
    The graph is replayed, then run again on new maps written into the same
    input buffers: the queue counter and error word restart each run."""
    sizes = [(256, 128), (64, 32), (256, 128), (128, 64), (512, 256)]
    specs = [ibl.spec_for(w, h) for w, h in sizes]
    specs[3].irradiance_size = None
    envs = [torch.from_numpy(synth.make_env(w, h, seed=60 + i, sun_max=1e6)).cuda()
            for i, (w, h) in enumerate(sizes)]
    stream = torch.cuda.Stream()
    batch = ibl.ProbeBatch(specs, envs, lut_size=64, lut_samples=128, graph=True, stream=stream,
                           precision=True, half=half)
    for _ in range(2):  # the second run replays the graph
        batch.run(stream)
    batch.status(stream)  # synchronises; no bounded wait gave up
    info = batch.info()
    assert info.graph == 1
    assert info.contraction_items > 0
    _check_precision_batch(batch, specs, envs, half)
    for i, (w, h) in enumerate(sizes):  # new maps in the same buffers
        envs[i].copy_(torch.from_numpy(synth.make_env(w, h, seed=70 + i, sun_max=1e6)))
    torch.cuda.synchronize()
    batch.run(stream)
    batch.status(stream)
    _check_precision_batch(batch, specs, envs, half)
    batch.close()


def _check_precision_batch(batch, specs, envs, half):
    for i, (s, env) in enumerate(zip(specs, envs)):
        chain = ibl.build_env_chain(env)
        mips = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
                for w, h in s.mip_sizes]
        irr = None
        if s.irradiance_size is not None:
            iw, ih = s.irradiance_size
            irr = torch.empty((ih, iw, 4), dtype=torch.float32, device="cuda")
        ibl.bake_tc(chain, s.env_width, s.env_height, mips, s.roughness, irradiance=irr)
        torch.cuda.synchronize()
        assert torch.equal(batch.chains[i], chain), i
        for m in range(len(mips)):
            want = mips[m].half() if half else mips[m]
            assert batch.mips[i][m].dtype == want.dtype
            assert torch.equal(batch.mips[i][m], want), (i, m)
        if irr is not None:
            assert torch.equal(batch.irradiance[i], irr.half() if half else irr), i


def test_precision_batch_of_the_batching_configuration_equals_solo_bakes():
    """Probes of the batching configuration's widths (2048 down to 256, log2(W)-3
    mips, 32x16 irradiance): their plans hold every kind of work item of the
    persistent contraction -- two-product row tiles (mip 1), three-product row
    tiles, column tiles (128x64 outputs), paired and K-interleaved outputs --
    and CUDA-core narrow outputs.  Every output equals the probe's solo bake."""
    sizes = [(2048, 1024), (1024, 512), (512, 256), (256, 128)]
    specs = [ibl.spec_for(w, h) for w, h in sizes]
    envs = [torch.from_numpy(synth.make_env(w, h, seed=80 + i, sun_max=1e6)).cuda()
            for i, (w, h) in enumerate(sizes)]
    stream = torch.cuda.Stream()
    batch = ibl.ProbeBatch(specs, envs, graph=True, stream=stream, precision=True)
    batch.run(stream)
    batch.status(stream)
    assert batch.info().contraction_items > 0
    for i, (s, env) in enumerate(zip(specs, envs)):
        chain = ibl.build_env_chain(env)
        mips = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
                for w, h in s.mip_sizes]
        iw, ih = s.irradiance_size
        irr = torch.empty((ih, iw, 4), dtype=torch.float32, device="cuda")
        ibl.bake_tc(chain, s.env_width, s.env_height, mips, s.roughness, irradiance=irr)
        torch.cuda.synchronize()
        for m in range(len(mips)):
            assert torch.equal(batch.mips[i][m], mips[m]), (s.env_width, m)
        assert torch.equal(batch.irradiance[i], irr), s.env_width
    batch.close()


def test_half_outputs_need_the_precision_path():
    spec = ibl.spec_for(64, 32)
    env = torch.from_numpy(synth.make_env(64, 32, seed=3)).cuda()
    with pytest.raises(ibl.IBLError):
        ibl.ProbeBatch([spec], [env], half=True)
