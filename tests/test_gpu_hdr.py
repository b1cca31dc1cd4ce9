"""GPU: the on-disk bake cache.  The first createResources bakes and writes the
RGBE files, the second loads them without baking; both hand back the
RGBE-quantised bake of the env file's own (decoded) pixels."""
import os

import numpy as np
import pytest

from althea_gb300 import hdr, ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_bake_cache_bakes_once_then_loads(tmp_path):
    root = str(tmp_path)
    name = "SynthRoom"
    w, h = 64, 32
    cache = hdr.BakeCache(root)
    with pytest.raises(ibl.IBLError):
        cache.create_resources(name)
    os.makedirs(os.path.dirname(cache.env_path(name)))
    hdr.write_hdr(cache.env_path(name), synth.make_tinted_env(w, h, seed=5))
    cfg = ibl.make_config(w, h, samples=512, generator=ibl.GEN_HAMMERSLEY)

    res, baked = cache.create_resources(name, cfg)
    assert baked and cache.complete(name)
    assert [tuple(m.shape) for m in res.prefilteredMap] == [(h >> (i + 1), w >> (i + 1), 4)
                                                           for i in range(5)]

    # the same bake done directly, then quantised through an RGBE file
    env = hdr.read_hdr(cache.env_path(name))
    ctx = ibl.BakeContext(ibl.make_config(w, h, samples=512, generator=ibl.GEN_HAMMERSLEY))
    ctx.upload_env(torch.from_numpy(env))
    irr, mips, _ = ctx.allocate_outputs()
    ctx.bake(irr, mips)
    torch.cuda.synchronize()
    ctx.close()
    q = str(tmp_path / "q.hdr")
    for got, ref in zip(res.prefilteredMap + [res.irradianceMap], mips + [irr]):
        hdr.write_hdr(q, ref.cpu().numpy())
        assert np.array_equal(got.cpu().numpy(), hdr.read_hdr(q))
    assert np.array_equal(res.environmentMap.cpu().numpy(), env)

    stamp = os.path.getmtime(cache.irradiance_path(name))
    res2, baked2 = cache.create_resources(name, cfg)
    assert not baked2 and os.path.getmtime(cache.irradiance_path(name)) == stamp
    for a, b in zip(res.prefilteredMap + [res.irradianceMap], res2.prefilteredMap + [res2.irradianceMap]):
        assert torch.equal(a, b)
