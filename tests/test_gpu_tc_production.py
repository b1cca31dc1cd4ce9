"""Accuracy of the precision path at production size, against the FP64
quadrature over level 0 (the oracle's quad_prefilter / quad_irradiance).

The benchmark map: 4096x2048, suns log-uniform up to 1e6 (seed 0), 9 mips
from 2048x1024 (roughness m/8) and a 128x64 irradiance, baked by the tensor-core
path with the planner's source levels -- the configuration the headline
throughput is quoted on -- and probes of every width of the batch
configuration (2048 down to 256 wide: log2(W) - 3 mips from W/2, 32x16
irradiance).  Checked texels, per output with
roughness > 0 and for the irradiance:

  * a seeded random sample;
  * every output texel whose direction lies within 5 degrees of one of the 8
    suns (a seeded subsample when there are more than the cap);
  * the u = 0 seam (columns 0 and W - 1) and the pole rows (rows 0 and H - 1).

Error per channel: |x - ref| / max(|ref|, 1e-6 max|ref|) <= 1e-3, and every
output texel finite.  The oracle runs on every host core (about 25 s for the
4096 map on 16 cores).  Each case prints one line (shown with ``-s``): the
checked texels and the worst and mean error per output.
"""
import json
import os

import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BAR = 1e-3
SUN_MAX = 1e6


def probe_config(env_w):
    """4096: the benchmark map; other widths: a batch-configuration probe
    (log2(W) - 3 mips from W/2, 32x16 irradiance)."""
    if env_w == 4096:
        mips, irr = [(2048 >> m, 1024 >> m) for m in range(9)], (128, 64)
    else:
        n = env_w.bit_length() - 1 - 3
        mips, irr = [((env_w // 2) >> m, (env_w // 4) >> m) for m in range(n)], (32, 16)
    rough = [m / (len(mips) - 1) for m in range(len(mips))]
    return env_w, env_w // 2, mips, rough, irr


def out_dirs(ow, oh):
    """Output texel directions at the reference's texel corners."""
    ys, xs = np.mgrid[0:oh, 0:ow]
    yaw = np.pi * (2.0 * xs / ow - 1.0)
    pit = np.pi * (ys / oh - 0.5)
    return np.stack([np.cos(pit) * np.cos(yaw), np.sin(pit), np.cos(pit) * np.sin(yaw)], -1)


def texel_set(ow, oh, suns, rng, per, sun_deg, cap):
    idx = set(rng.choice(ow * oh, size=min(per, ow * oh), replace=False).tolist())
    d = out_dirs(ow, oh).reshape(-1, 3)
    near = np.zeros(ow * oh, dtype=bool)
    for sd, _, _ in suns:
        near |= d @ sd >= np.cos(np.deg2rad(sun_deg))
    near_idx = np.nonzero(near)[0]
    if near_idx.size > cap:
        near_idx = rng.choice(near_idx, size=cap, replace=False)
    idx |= set(near_idx.tolist())
    idx |= {y * ow for y in range(oh)} | {y * ow + ow - 1 for y in range(oh)}
    idx |= set(range(ow)) | {(oh - 1) * ow + x for x in range(ow)}
    idx = np.array(sorted(idx))
    return np.stack([idx % ow, idx // ow], 1).astype(np.int32), int(near.sum())


def rel_errors(got, ref):
    scale = 1e-6 * np.abs(ref).max()
    e = np.abs(got.astype(np.float64) - ref) / np.maximum(np.abs(ref), scale)
    return np.where(np.isfinite(got), e, np.inf)  # a missing output is a failure


# (map width, random texels per output, cap on near-sun texels, map seed): seed 1
# of the 2048-wide probe holds the closest approach to the bar measured (8.2e-4,
# its two-product mip 1)
@pytest.mark.parametrize("env_w,per,cap,seed", [(4096, 1024, 4096, 0), (2048, 1024, 2048, 0),
                                                (2048, 1024, 2048, 1), (1024, 1024, 1024, 0),
                                                (1024, 1024, 1024, 2), (512, 1024, 1024, 0),
                                                (256, 1024, 512, 0)])
def test_precision_path_within_1e3_of_fp64_at_production_size(env_w, per, cap, seed):
    w, h, sizes, rough, (iw, ih) = probe_config(env_w)
    env = synth.make_env(w, h, seed=seed, sun_max=SUN_MAX)
    suns = synth.sun_params(w, h, seed=seed, sun_max=SUN_MAX)
    chain = ibl.build_env_chain(torch.from_numpy(env).cuda())
    outs = [torch.full((mh, mw, 4), float("nan"), dtype=torch.float32, device="cuda")
            for mw, mh in sizes]
    irr = torch.full((ih, iw, 4), float("nan"), dtype=torch.float32, device="cuda")
    levels, irr_level = ibl.tc_plan(w, h, sizes, rough, iw)
    ibl.bake_tc(chain, w, h, outs, rough, irradiance=irr)  # planner levels, error flag checked
    torch.cuda.synchronize()
    outs = [o.cpu().numpy() for o in outs]
    irr = irr.cpu().numpy()
    for o in outs + [irr]:
        assert np.isfinite(o).all()
    rng = np.random.default_rng(2024 + seed)
    nt = os.cpu_count() or 0
    worst, report = {}, {}
    targets = [(f"mip{m}", mw, mh, r, outs[m]) for m, ((mw, mh), r) in
               enumerate(zip(sizes, rough)) if r > 0.0]
    targets.append(("irradiance", iw, ih, None, irr))
    for name, ow, oh, r, img in targets:
        xy, _ = texel_set(ow, oh, suns, rng, per, 5.0, cap)
        if r is None:
            ref = oracle.quad_irradiance(env, ow, oh, xy, nthreads=nt)[:, :3]
        else:
            ref = oracle.quad_prefilter(env, ow, oh, r, xy, nthreads=nt)[:, :3]
        e = rel_errors(img[xy[:, 1], xy[:, 0], :3], ref)
        worst[name] = float(e.max())
        report[name] = {"texels": int(len(xy)), "max": float(e.max()), "mean": float(e.mean())}
    print(json.dumps({"map": [w, h], "seed": seed, "levels": levels, "irradiance_level": irr_level,
                      "outputs": report}))
    assert max(worst.values()) <= BAR, (levels, irr_level, worst)
