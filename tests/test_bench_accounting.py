"""CPU checks of the numerators bench.py reports its rooflines against, for
the 4096x2048 workloads, recomputed here from their definitions:

* plain path: algorithmic gathered bytes, 128 B per sample (two levels x four
  RGBA32F taps) for mips of roughness > 0, one 64 B bilinear tap per texel at
  roughness 0, plus 16 B written per output texel;
* precision path: 2 flops x 4 channels per (output texel, source texel) pair
  of every contraction the planner emits, and the launches of one bake."""
import bench
from althea_gb300 import ibl


def _plan():
    return ibl.tc_plan(bench.ENV_W, bench.ENV_H, bench.mip_sizes(), bench.roughness(),
                       bench.IRR_W)


def test_workload_shape():
    assert (bench.ENV_W, bench.ENV_H) == (4096, 2048)
    assert bench.mip_sizes() == [(2048 >> m, 1024 >> m) for m in range(9)]
    assert bench.roughness() == [m / 8 for m in range(9)]
    assert (bench.IRR_W, bench.IRR_H) == (128, 64)


def test_plain_algorithmic_bytes():
    texels = [w * h for w, h in bench.mip_sizes()]
    gathers = texels[0] * 64 + sum(texels[1:]) * bench.SAMPLES * 128
    assert bench.prefilter_algorithmic_bytes() == gathers + 16 * sum(texels)
    assert round(bench.prefilter_algorithmic_bytes() / 1e9, 2) == 91.80


def test_precision_flops_and_jobs():
    levels, irr_level = _plan()
    assert levels == [-1, 2, 2, 2, 1, 1, 1, 1, 1] and irr_level == 1
    pairs = executed_pairs = 0
    for m, ((w, h), lv) in enumerate(list(zip(bench.mip_sizes(), levels)) +
                                     [((128, 64), irr_level)]):
        # mip 8 (8x4, roughness 1, level 1 like the irradiance) is the
        # irradiance's normalised sum: no pairs of its own
        if lv >= 0 and m != 8:
            p = w * h * (4096 >> lv) * (2048 >> lv)
            pairs += p
            # mips 1 and 2 (roughness 1/8 and 1/4) take two BF16 products per
            # channel, the rest three
            executed_pairs += p * (2 if m in (1, 2) else 3)
    alg, executed = bench.tc_flops(levels, irr_level)
    assert alg == 8 * pairs and executed == 6 * executed_pairs
    assert round(alg / 1e12, 2) == 3.21
    # the library's own account: the same pairs (tensor + CUDA cores), the
    # visible part of them smaller, and at least the flops of the visible
    # pairs at two products per channel issued on the tensor cores
    work = bench.tc_work()
    assert work["dense_pairs"] + work["cuda_core_pairs"] == pairs
    assert 0.5 * work["dense_pairs"] < work["visible_pairs"] < work["dense_pairs"]
    assert work["tensor_flops_issued"] >= 2 * 3 * 2 * work["visible_pairs"]
    assert work["tensor_launches"] == 1  # one queue launch
    # phase counts: s = source / output width; g = 1, s / 8 or s
    for w, h, ws, hs, lv, g in bench.tc_jobs(levels, irr_level):
        s = ws // w
        assert ws % w == 0 and 8 * g == s * (8 // s if 8 % s == 0 else (1 if s % 8 == 0 else 8))


def test_precision_launches_per_bake():
    """12 chain blits, 2 split passes (levels 1 and 2), 1 tables pass,
    1 queue launch for every contraction (mips 1-6 and the irradiance), 1
    finish, 2 for the 16x8 mip on the CUDA cores (the 8x4 roughness-1 mip
    comes out of the irradiance's finish), 1 delta mip, 1 LUT: 21."""
    levels, irr_level = _plan()
    assert bench.tc_launches(levels, irr_level) == 12 + 2 + 1 + 1 + 1 + 2 + 1 + 1 == 21


def test_cpu_strata_cover_every_texel_once():
    """The CPU baseline and the reference arm bake a probe in row strata: over
    S consecutive strata every texel of every output is baked exactly once
    (outputs with fewer rows than S are done in their first strata)."""
    import numpy as np
    for strata in (1, 3, 8):
        for ow, oh in bench.mip_sizes() + [(bench.IRR_W, bench.IRR_H), (5, 3)]:
            seen = np.zeros((oh, ow), dtype=np.int32)
            for k in range(strata):
                xy = bench.CpuProbe.rows_xy(ow, oh, k, strata)
                if xy is None:
                    continue
                np.add.at(seen, (xy[:, 1], xy[:, 0]), 1)
            assert (seen == 1).all(), (strata, ow, oh)
