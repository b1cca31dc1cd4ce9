"""Accuracy report of the precision path (tcgen05 BF16 hi/lo contraction) on
the 4096x2048 benchmark map with suns up to 1e6, against the FP64 quadrature
over level 0 (oracle O2).  Not a pytest module: it bakes on cuda:0, then
evaluates the oracle on every host core for a few minutes.

Texels checked, per prefilter mip with roughness > 0 and for the irradiance:
  * a seeded random sample (--per-mip, default 1024);
  * every output texel whose direction lies within --sun-deg (5) degrees of a
    sun (a seeded subsample when more than --cap);
  * the u = 0 seam (columns 0 and W-1) and the pole rows (rows 0 and H-1).
Error per channel: |x - ref| / max(|ref|, 1e-6 max|ref|); the table gives
max, mean and the 99.99th percentile per output.

Usage: python tests/precision_report.py [--per-mip N] [--sun-deg D] [--cap C]
                                       [--env-width 4096|2048|1024|512|256]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from althea_gb300 import ibl, synth  # noqa: E402

SUN_MAX = 1e6


def config(env_w):
    """The benchmark map (4096 wide: 9 mips from W/2, 128x64 irradiance) or a
    batch-configuration probe (log2(W) - 3 mips from W/2, 32x16 irradiance)."""
    if env_w == 4096:
        mips, irr = [(2048 >> m, 1024 >> m) for m in range(9)], (128, 64)
    else:
        n = env_w.bit_length() - 1 - 3
        mips, irr = [((env_w // 2) >> m, (env_w // 4) >> m) for m in range(n)], (32, 16)
    rough = [m / (len(mips) - 1) for m in range(len(mips))]
    return env_w, env_w // 2, mips, rough, irr


def out_dirs(ow, oh):
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


def errors(got, ref):
    scale = 1e-6 * np.abs(ref).max()
    e = np.abs(got - ref) / np.maximum(np.abs(ref), scale)
    e = np.where(np.isfinite(got), e, np.inf)  # a missing output is a failure
    return {"max": float(e.max()), "mean": float(e.mean()),
            "p99.99": float(np.percentile(e, 99.99))}


def main():
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--per-mip", type=int, default=1024)
    ap.add_argument("--sun-deg", type=float, default=5.0)
    ap.add_argument("--cap", type=int, default=4096)
    ap.add_argument("--env-width", type=int, default=4096,
                    help="4096: the benchmark map; 256..2048: a batch-configuration probe")
    ap.add_argument("--seed", type=int, default=0, help="map seed (the benchmark uses 0)")
    args = ap.parse_args()
    SEED = args.seed
    ENV_W, ENV_H, MIPS, ROUGH, IRR = config(args.env_width)
    env = synth.make_env(ENV_W, ENV_H, seed=SEED, sun_max=SUN_MAX)
    suns = synth.sun_params(ENV_W, ENV_H, seed=SEED, sun_max=SUN_MAX)
    chain = ibl.build_env_chain(torch.from_numpy(env).cuda())
    outs = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for w, h in MIPS]
    irr = torch.empty((IRR[1], IRR[0], 4), dtype=torch.float32, device="cuda")
    levels, irr_level = ibl.tc_plan(ENV_W, ENV_H, MIPS, ROUGH, IRR[0])
    ibl.bake_tc(chain, ENV_W, ENV_H, outs, ROUGH, irradiance=irr)
    torch.cuda.synchronize()
    outs = [o.cpu().numpy() for o in outs]
    irr = irr.cpu().numpy()
    rng = np.random.default_rng(2024)
    rows, t0, checked = [], time.time(), 0
    targets = [(f"mip{m}", w, h, r, outs[m], lv) for m, ((w, h), r, lv) in
               enumerate(zip(MIPS, ROUGH, levels)) if r > 0.0]
    targets.append(("irradiance", IRR[0], IRR[1], None, irr, irr_level))
    for name, w, h, r, img, lv in targets:
        xy, near = texel_set(w, h, suns, rng, args.per_mip, args.sun_deg, args.cap)
        if r is None:
            ref = oracle.quad_irradiance(env, w, h, xy)[:, :3]
        else:
            ref = oracle.quad_prefilter(env, w, h, r, xy)[:, :3]
        got = img[xy[:, 1], xy[:, 0], :3]
        row = {"output": name, "size": f"{w}x{h}", "source_level": lv, "texels": int(len(xy)),
               "near_sun": near, **errors(got, ref)}
        rows.append(row)
        checked += len(xy)
    worst = max(r["max"] for r in rows)
    print("| output | size | source level | texels checked | max | mean | p99.99 |")
    print("|---|---|---|---|---|---|---|")
    for r in rows:
        print(f"| {r['output']} | {r['size']} | {r['source_level']} | {r['texels']} | "
              f"{r['max']:.2e} | {r['mean']:.2e} | {r['p99.99']:.2e} |")
    print(json.dumps({"worst_max": worst, "texels": checked, "cores": os.cpu_count(),
                      "oracle_seconds": time.time() - t0, "rows": rows}))
    return 0 if worst <= 1e-3 else 1


if __name__ == "__main__":
    sys.exit(main())
