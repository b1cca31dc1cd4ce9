"""GPU parity of the reflection-buffer glossy convolution (C ABI,
althea_ssr_convolve / althea_ssr_convolve_levels): bit-identical to the
reference shader's outputs (golden fixtures) and to the oracle at full frame
sizes, plus properties that hold at any size."""
import os

import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ssr.npz")


def _gpu_convolve(l0, mips):
    h, w = l0.shape[:2]
    chain = torch.zeros(4 * ibl.ssr_level_offset(w, h, mips), dtype=torch.float16, device="cuda")
    chain[:l0.size] = torch.from_numpy(np.ascontiguousarray(l0).reshape(-1)).cuda()
    ibl.ssr_convolve(chain, w, h, mips)
    torch.cuda.synchronize()
    return chain.cpu().numpy()


def test_bit_identical_to_reference_shader_golden():
    g = dict(np.load(GOLD))
    for k in range(6):
        w, h, mips = (int(v) for v in g[f"shape{k}"])
        got = _gpu_convolve(g[f"in{k}"].view(np.float16), mips)
        assert np.array_equal(got.view(np.uint16), g[f"out{k}"]), (w, h, mips)


@pytest.mark.parametrize("w,h,mips", [(3840, 2160, 5), (1920, 1080, 5), (2561, 1439, 5),
                                      (1, 1, 5), (2, 1, 3), (1, 3, 3), (777, 5, 12),
                                      (64, 64, 1)])
def test_bit_identical_to_oracle(w, h, mips):
    l0 = synth.make_reflection(w, h, seed=w * 7 + h, extremes=True)
    ref = oracle.ssr_convolve(l0, mips)
    got = _gpu_convolve(l0, mips)
    assert np.array_equal(got.view(np.uint16), ref.view(np.uint16))


def test_pitched_levels_equal_packed_chain():
    w, h, mips = 1000, 562, 5
    l0 = synth.make_reflection(w, h, seed=3)
    packed = _gpu_convolve(l0, mips)
    levels = []
    for l in range(mips):
        lw, lh = max(1, w >> l), max(1, h >> l)
        big = torch.full((lh, lw + 13, 4), float("nan"), dtype=torch.float16, device="cuda")
        levels.append(big[:, :lw])  # padded rows: pitch (lw + 13) texels
    levels[0].copy_(torch.from_numpy(l0).cuda())
    ibl.ssr_convolve_levels(levels)
    torch.cuda.synchronize()
    flat = np.concatenate([t.cpu().numpy().reshape(-1) for t in levels])
    assert np.array_equal(flat.view(np.uint16), packed.view(np.uint16))


def test_full_frame_scaling_by_two_commutes():
    w, h = 3840, 2160
    l0 = synth.make_reflection(w, h, seed=9)
    l0 = np.where(np.abs(l0) < 2.0 ** -13, np.float16(0), l0).astype(np.float16)
    a = _gpu_convolve(l0, 5).astype(np.float32)
    b = _gpu_convolve((l0.astype(np.float32) * 2).astype(np.float16), 5).astype(np.float32)
    small = np.abs(a) < 2.0 ** -13
    assert np.array_equal(b[~small], 2 * a[~small])


def test_reflection_buffer_class_and_graph_capture():
    rb = ibl.ReflectionBuffer(640, 360)
    l0 = synth.make_reflection(640, 360, seed=4)
    rb.level(0).copy_(torch.from_numpy(l0).cuda())
    ref = oracle.ssr_convolve(l0, 5)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        rb.convolveReflectionBuffer(stream=s)  # warm-up outside capture
    torch.cuda.synchronize()
    assert np.array_equal(rb.chain.cpu().numpy().view(np.uint16), ref.view(np.uint16))
    g = torch.cuda.CUDAGraph()
    rb.chain[4 * 640 * 360:].zero_()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        rb.convolveReflectionBuffer(stream=s)
    g.replay()
    torch.cuda.synchronize()
    assert np.array_equal(rb.chain.cpu().numpy().view(np.uint16), ref.view(np.uint16))


def test_errors_leave_outputs_untouched():
    rb = ibl.ReflectionBuffer(64, 32)
    before = rb.chain.clone()
    with pytest.raises(ibl.IBLError):
        ibl.ssr_convolve(rb.chain, 64, 32, 17)
    with pytest.raises(ibl.IBLError):
        ibl.ssr_convolve(rb.chain[:10], 64, 32, 5)
    torch.cuda.synchronize()
    assert torch.equal(before, rb.chain)
