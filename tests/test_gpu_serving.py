"""GPU tests of the serving loop: admission by slot and HBM budget, overlap,
and the same result for a request alone and in the mix."""
import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, serving, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pool(server, sizes, seed0):
    bufs = []
    for i, w in enumerate(sizes):
        env = synth.make_env(w, w // 2, seed=seed0 + i)
        bufs.append(server.buffers(env, max(1, w.bit_length() - 1 - 3)))
    return bufs


def test_alone_equals_mixed():
    sizes = [256, 128, 512, 256, 64, 128, 256, 512]
    alone = serving.ProbeServer(budget_bytes=1 << 30, max_inflight=1, samples=128)
    mixed = serving.ProbeServer(budget_bytes=1 << 30, max_inflight=8, samples=128)
    pa = _pool(alone, sizes, 100)
    pm = _pool(mixed, sizes, 100)
    for i, b in enumerate(pa):  # one at a time, drained between requests
        alone.submit(i, b)
        alone.drain()
    for i, b in enumerate(pm):  # all at once, overlapping on the device
        mixed.submit(i, b)
    comps = mixed.drain()
    assert sorted(c.tag for c in comps) == list(range(len(sizes)))
    assert all(c.status == ibl.OK for c in comps)
    assert mixed.stats().peak_bytes_in_use > alone.stats().peak_bytes_in_use  # they overlapped
    for a, m in zip(pa, pm):
        assert torch.equal(a.mips, m.mips)
        assert torch.equal(a.irradiance, m.irradiance)
    # and the first request against the oracle
    env = synth.make_env(256, 128, seed=100)
    chain = oracle.build_chain(env)
    off = 0
    for k, (w, h) in enumerate(pa[0].mip_sizes):
        n = w * h * 4
        got = pa[0].mips[off:off + n].numpy().reshape(h, w, 4)
        r = k / (len(pa[0].mip_sizes) - 1)
        assert np.array_equal(got, oracle.prefilter(chain, 256, 128, w, h, r, 128,
                                                    oracle.GEN_HAMMERSLEY))
        off += n
    alone.close()
    mixed.close()


def test_budget_limits_concurrency_and_rejects_oversize():
    probe = serving.ProbeServer(budget_bytes=1 << 30, max_inflight=1, samples=64)
    need = probe.request_bytes(512, 256, 6)
    probe.close()
    server = serving.ProbeServer(budget_bytes=int(need * 2.5), max_inflight=8, samples=64)
    bufs = _pool(server, [512] * 6, 7)
    for i, b in enumerate(bufs):
        server.submit(i, b)
    st = server.stats()
    assert st.inflight <= 2 and st.queued >= 4 - 0  # only two fit the budget
    comps = server.drain()
    assert len(comps) == 6 and all(c.status == ibl.OK for c in comps)
    assert server.stats().peak_bytes_in_use <= int(need * 2.5)
    big = server.buffers(synth.make_env(2048, 1024, seed=1), 8)
    with pytest.raises(ibl.IBLError) as e:
        server.submit(99, big)
    assert e.value.status == ibl.ERR_BUDGET
    server.close()


def test_poisson_run_reports_latency():
    server = serving.ProbeServer(budget_bytes=2 << 30, max_inflight=8, samples=256)
    pool = _pool(server, [256, 512, 256, 128] * 4, 11)
    r = serving.run_poisson(server, pool, rate=500.0, n_requests=64, seed=3)
    assert r["ok"] == 64 and r["p99_ms"] >= r["p50_ms"] > 0
    server.close()


def test_precision_server_alone_equals_mixed_and_solo_bake():
    """Requests on the precision path: the same alone, in the mix, and as the
    stateless tensor-core bake of the same map."""
    sizes = [256, 128, 512, 256, 64]
    alone = serving.ProbeServer(budget_bytes=1 << 31, max_inflight=1, path=ibl.PATH_PRECISION)
    mixed = serving.ProbeServer(budget_bytes=1 << 31, max_inflight=8, path=ibl.PATH_PRECISION)
    pa = _pool(alone, sizes, 300)
    pm = _pool(mixed, sizes, 300)
    for i, b in enumerate(pa):
        alone.submit(i, b)
        alone.drain()
    for i, b in enumerate(pm):
        mixed.submit(i, b)
    comps = mixed.drain()
    assert sorted(c.tag for c in comps) == list(range(len(sizes)))
    assert all(c.status == ibl.OK for c in comps)
    for a, m in zip(pa, pm):
        assert torch.equal(a.mips, m.mips)
        assert torch.equal(a.irradiance, m.irradiance)
    # the first request against the stateless precision bake
    env = synth.make_env(256, 128, seed=300)
    chain = ibl.build_env_chain(torch.from_numpy(env).cuda())
    sizes0 = pa[0].mip_sizes
    mips = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for w, h in sizes0]
    rough = [k / (len(sizes0) - 1) for k in range(len(sizes0))]
    irr = torch.empty((16, 32, 4), dtype=torch.float32, device="cuda")
    ibl.bake_tc(chain, 256, 128, mips, rough, irradiance=irr)
    torch.cuda.synchronize()
    flat = torch.cat([t.reshape(-1) for t in mips]).cpu()
    assert torch.equal(pa[0].mips, flat)
    assert torch.equal(pa[0].irradiance, irr.cpu())
    alone.close()
    mixed.close()


def _sky(w, seed):
    """A sky map without suns (the resident part of a re-bake request)."""
    return synth.make_env(w, w // 2, seed=seed, with_suns=False)


@pytest.mark.parametrize("path", [ibl.PATH_PLAIN, ibl.PATH_PRECISION])
def test_resident_maps_with_per_request_suns(path):
    """Maps registered once stay on the device; requests name a map and the
    sun lobes to add to it.  Each result equals, bit for bit, the same request
    run alone and the stateless bake of apply_suns(map, suns); unregister is
    refused while a request holds the map; resident bytes count against the
    budget."""
    sizes = [256, 512, 128]
    kw = dict(samples=128, path=path)
    alone = serving.ProbeServer(budget_bytes=1 << 31, max_inflight=1, **kw)
    mixed = serving.ProbeServer(budget_bytes=1 << 31, max_inflight=8, **kw)
    skies = [_sky(w, 40 + i) for i, w in enumerate(sizes)]
    ids_a = [alone.register_env(e) for e in skies]
    ids_m = [mixed.register_env(torch.from_numpy(e).cuda()) for e in skies]  # device source
    assert mixed.stats().resident_maps == 3
    assert mixed.stats().bytes_resident == sum(w * (w // 2) * 16 for w in sizes)
    reqs = []  # (map index, suns) -- each map twice with different suns
    for k in range(6):
        i = k % 3
        reqs.append((i, synth.sun_params(sizes[i], sizes[i] // 2, seed=900 + k, sun_max=1e5)))
    mips = [max(1, sizes[i].bit_length() - 1 - 3) for i, _ in reqs]
    ba = [alone.output_buffers(ids_a[i], m) for (i, _), m in zip(reqs, mips)]
    bm = [mixed.output_buffers(ids_m[i], m) for (i, _), m in zip(reqs, mips)]
    for k, ((i, suns), b) in enumerate(zip(reqs, ba)):
        alone.submit(k, b, suns)
        alone.drain()
    for k, ((i, suns), b) in enumerate(zip(reqs, bm)):
        mixed.submit(k, b, suns)
    comps = mixed.drain()
    assert sorted(c.tag for c in comps) == list(range(6)) and all(c.status == ibl.OK
                                                                for c in comps)
    for a, m in zip(ba, bm):
        assert torch.equal(a.mips, m.mips) and torch.equal(a.irradiance, m.irradiance)
    # request 4 (map 1 with its suns) against the stateless bake of the same map
    i, suns = reqs[4]
    w, h = sizes[i], sizes[i] // 2
    env = ibl.apply_suns(torch.from_numpy(skies[i]).cuda(), suns)
    chain = ibl.build_env_chain(env)
    sz = bm[4].mip_sizes
    outs = [torch.empty((mh, mw, 4), dtype=torch.float32, device="cuda") for mw, mh in sz]
    rough = [k / (len(sz) - 1) for k in range(len(sz))]
    irr = torch.empty((16, 32, 4), dtype=torch.float32, device="cuda")
    if path == ibl.PATH_PRECISION:
        ibl.bake_tc(chain, w, h, outs, rough, irradiance=irr)
    else:
        ibl.prefilter(chain, w, h, outs, rough, 128, ibl.GEN_HAMMERSLEY)
        ibl.irradiance(chain, w, h, irr)
    torch.cuda.synchronize()
    assert torch.equal(bm[4].mips, torch.cat([t.reshape(-1) for t in outs]).cpu())
    assert torch.equal(bm[4].irradiance, irr.cpu())
    for j in ids_m:
        mixed.unregister_env(j)
    assert mixed.stats().resident_maps == 0 and mixed.stats().bytes_resident == 0
    alone.close()
    mixed.close()


def test_apply_suns_matches_the_synthetic_generator():
    """The device sun lobes (FP32, chord-angle form) against the FP64 numpy
    generator that makes the benchmark maps: sky + the same 8 suns.  In a
    lobe's tail the FP32 angle (about 1e-7 rad) is amplified by the exponent
    (theta^2 / 2 sigma^2 up to ~15 where the lobe still dominates the sky):
    up to ~4e-5 relative, hence 1e-4."""
    w, h = 512, 256
    suns = synth.sun_params(w, h, seed=5, sun_max=1e6)
    sky = torch.from_numpy(synth.make_env(w, h, seed=5, with_suns=False)).cuda()
    got = ibl.apply_suns(sky, suns).cpu().numpy()
    ref = synth.make_env(w, h, seed=5, sun_max=1e6)
    rel = np.abs(got[..., :3] - ref[..., :3]) / np.abs(ref[..., :3])
    assert rel.max() <= 1e-4, rel.max()
    assert np.array_equal(got[..., 3], ref[..., 3])
    # in place, and refusals
    ibl.apply_suns(sky, suns, out=sky)
    assert torch.equal(sky.cpu(), torch.from_numpy(got))
    with pytest.raises(ibl.IBLError):
        ibl.apply_suns(sky, [((0.0, 0.0, 0.0), 0.02, 1.0)])  # no direction
    with pytest.raises(ibl.IBLError):
        ibl.apply_suns(sky, [((0.0, 1.0, 0.0), 0.02, 1.0)] * 17)  # too many


def test_unregister_refused_while_a_request_holds_the_map():
    """A resident map named by a queued request cannot be unregistered; once
    the request has completed it can.  One slot: the small map's request
    waits behind a 2048x1024 bake (milliseconds; the refusal takes
    microseconds)."""
    server = serving.ProbeServer(budget_bytes=1 << 31, max_inflight=1, samples=256)
    big = server.register_env(_sky(2048, 60))
    small = server.register_env(_sky(256, 61))
    b_big = server.output_buffers(big, 8)
    b_small = server.output_buffers(small, 5)
    server.submit(0, b_big, synth.draw_suns(1, 1e4))
    server.submit(1, b_small, synth.draw_suns(2, 1e4))
    with pytest.raises(ibl.IBLError) as e:
        server.unregister_env(small)
    assert e.value.status == ibl.ERR_NOT_READY
    comps = server.drain()
    assert sorted(c.tag for c in comps) == [0, 1] and all(c.status == ibl.OK for c in comps)
    server.unregister_env(small)
    server.unregister_env(big)
    with pytest.raises(ibl.IBLError) as e:  # gone
        server.submit(2, b_small)
    assert e.value.status == ibl.ERR_INVALID_ARGUMENT
    assert server.stats().resident_maps == 0
    server.close()
