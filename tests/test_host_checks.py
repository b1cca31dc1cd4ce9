"""CPU tests of the Python mirror's extent checks.

The C calls take chains and outputs as bare pointers and pitches, so the
mirror checks every tensor against the extents the kernels will read or
write before any call reaches the library.  The checks look only at tensor
metadata, so they run here on CPU tensors: a tensor of the right extent gets
as far as the device check ("must be a CUDA tensor"), a wrong one is refused
before it."""
import pytest

from althea_gb300 import ibl

torch = pytest.importorskip("torch")


def _status_and_text(fn):
    with pytest.raises(ibl.IBLError) as e:
        fn()
    return e.value.status, str(e.value)


def _chain(w, h, extra=0, dtype=None):
    return torch.zeros((ibl.chain_texels(w, h) + extra, 4), dtype=dtype or torch.float32)


def test_chain_extent_dtype_and_layout():
    w, h = 64, 32
    st, text = _status_and_text(lambda: ibl._require_chain(_chain(w, h, extra=-1), w, h))
    assert st == ibl.ERR_INVALID_ARGUMENT and "texels" in text
    st, text = _status_and_text(lambda: ibl._require_chain(_chain(w, h, dtype=torch.float64), w, h))
    assert "float32" in text
    strided = torch.zeros((ibl.chain_texels(w, h), 8))[:, :4]
    st, text = _status_and_text(lambda: ibl._require_chain(strided, w, h))
    assert "contiguous" in text
    # the right extent (or more) passes every metadata check and stops at the device
    for extra in (0, 5):
        st, text = _status_and_text(lambda: ibl._require_chain(_chain(w, h, extra), w, h))
        assert "CUDA" in text


def test_prefilter_and_irradiance_refuse_short_chains():
    w, h = 128, 64
    outs = [torch.zeros((32, 64, 4))]
    st, text = _status_and_text(
        lambda: ibl.prefilter(_chain(w, h, extra=-8), w, h, outs, [0.5], 64))
    assert st == ibl.ERR_INVALID_ARGUMENT and "texels" in text
    st, text = _status_and_text(
        lambda: ibl.irradiance(_chain(w, h, extra=-1), w, h, torch.zeros((16, 32, 4))))
    assert "texels" in text
    # a chain for a smaller env is short for a larger one
    st, text = _status_and_text(
        lambda: ibl.prefilter(_chain(64, 32), w, h, outs, [0.5], 64))
    assert "texels" in text


def test_counts_of_outputs_roughness_and_levels():
    w, h = 128, 64
    chain = _chain(w, h)
    outs = [torch.zeros((32, 64, 4)), torch.zeros((16, 32, 4))]
    st, text = _status_and_text(lambda: ibl.prefilter(chain, w, h, outs, [0.5], 64))
    assert "roughness" in text
    st, text = _status_and_text(lambda: ibl.bake_tc(chain, w, h, outs, [0.5]))
    assert "roughness" in text
    st, text = _status_and_text(lambda: ibl.bake_tc(chain, w, h, outs, [0.5, 1.0], levels=[0]))
    assert "source levels" in text
    many = [torch.zeros((1, 1, 4))] * (ibl.MAX_MIPS + 1)
    st, text = _status_and_text(
        lambda: ibl.prefilter(chain, w, h, many, [0.5] * len(many), 64))
    assert "at most" in text


class _FakeContext(ibl.BakeContext):
    """BakeContext's extent checks without a device: sizes come from the
    config the way the library derives them (mips from the first-mip size,
    halved per mip; irradiance at the configured size)."""

    def __init__(self, cfg):
        self.cfg = cfg
        self._ctx = None

    def irradiance_size(self):
        return self.cfg.irradiance_width, self.cfg.irradiance_height

    def mip_info(self, m):
        return (max(self.cfg.first_mip_width >> m, 1), max(self.cfg.first_mip_height >> m, 1),
                m / max(self.cfg.mip_count - 1, 1))

    def close(self):
        pass


def _outputs(ctx):
    iw, ih = ctx.irradiance_size()
    mips = [torch.zeros((ctx.mip_info(m)[1], ctx.mip_info(m)[0], 4))
            for m in range(ctx.cfg.mip_count)]
    n = ctx.cfg.lut_size
    return torch.zeros((ih, iw, 4)), mips, (torch.zeros((n, n, 2)) if n else None)


def test_context_bake_holds_outputs_to_its_sizes():
    cfg = ibl.make_config(256, 128, irradiance_size=(32, 16), mip_count=4, lut_size=16)
    ctx = _FakeContext(cfg)
    irr, mips, lut = _outputs(ctx)
    # every extent right: the call gets as far as the device check
    st, text = _status_and_text(lambda: ctx.bake(irr, mips, lut))
    assert "CUDA" in text
    cases = [
        (torch.zeros((16, 31, 4)), mips, lut, "irradiance"),
        (irr, mips[:-1], lut, "mip tensors"),
        (irr, mips + [torch.zeros((8, 16, 4))], lut, "mip tensors"),
        (irr, [mips[0], torch.zeros((16, 32, 4))] + mips[2:], lut, "mip 1"),
        (irr, mips, None, "LUT"),
        (irr, mips, torch.zeros((16, 8, 2)), "lut"),
    ]
    for i, m, l, what in cases:
        st, text = _status_and_text(lambda: ctx.bake(i, m, l))
        assert st == ibl.ERR_INVALID_ARGUMENT and what in text, (what, text)


def test_context_without_lut_ignores_a_passed_lut():
    cfg = ibl.make_config(64, 32, irradiance_size=(16, 8), mip_count=2)
    ctx = _FakeContext(cfg)
    irr, mips, _ = _outputs(ctx)
    st, text = _status_and_text(lambda: ctx.bake(irr, mips, torch.zeros((3, 3, 2))))
    assert "CUDA" in text
