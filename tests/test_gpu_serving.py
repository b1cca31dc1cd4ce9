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
