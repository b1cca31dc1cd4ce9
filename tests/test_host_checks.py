"""CPU tests of the Python mirror's extent checks.

The C calls take chains and outputs as bare pointers and pitches, so the
mirror checks every tensor against the extents the kernels will read or
write before any call reaches the library.  The checks look only at tensor
metadata, so they run here on CPU tensors: a tensor of the right extent gets
as far as the device check ("must be a CUDA tensor"), a wrong one is refused
before it.  With tensors that report themselves as CUDA tensors and a library
that records its computing calls, valid calls are followed through to the C
call and its arguments."""
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
    wide = _chain(w, h, dtype=torch.float64)
    st, text = _status_and_text(lambda: ibl._require_chain(wide, w, h))
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


# ---- valid calls reach the library -------------------------------------------
# CPU tensors that report themselves as CUDA tensors, and a library whose
# computing calls are recorded instead of run (its host-only calls, such as
# chain_texels and the workspace sizes, are the real ones).

class _AsCuda(torch.Tensor):
    @property
    def is_cuda(self):
        return True


def _dev(*shape, dtype=None):
    return torch.zeros(shape, dtype=dtype or torch.float32).as_subclass(_AsCuda)


class _Stream:
    cuda_stream = 0


class _Recorder:
    def __init__(self, real):
        self.real = real
        self.calls = []

    def __getattr__(self, name):
        if name.startswith("althea_") and name in self.RECORDED:
            def rec(*args):
                self.calls.append((name, args))
                return ibl.OK
            return rec
        return getattr(self.real, name)

    RECORDED = {"althea_ibl_prefilter", "althea_ibl_irradiance", "althea_ibl_bake_tc_ex",
                "althea_ibl_tc_error", "althea_ibl_build_env_chain", "althea_ibl_bake"}


@pytest.fixture
def recorder(monkeypatch):
    rec = _Recorder(ibl.load())
    monkeypatch.setattr(ibl, "load", lambda *a, **k: rec)
    return rec


def test_valid_calls_reach_the_library(recorder):
    w, h = 256, 128
    chain = _dev(ibl.chain_texels(w, h), 4)
    env = _dev(h, w, 4)
    sizes, rough = [(128, 64), (64, 32), (8, 4)], [0.0, 0.5, 1.0]
    mips = [_dev(mh, mw, 4) for mw, mh in sizes]
    irr = _dev(16, 32, 4)
    s = _Stream()
    ibl.build_env_chain_into(env, chain, s)
    ibl.prefilter(chain, w, h, mips, rough, 64, ibl.GEN_HAMMERSLEY, s)
    ibl.irradiance(chain, w, h, irr, stream=s)
    ibl.bake_tc(chain, w, h, mips, rough, irradiance=irr, stream=s)
    half = [_dev(mh, mw, 4, dtype=torch.float16) for mw, mh in sizes]
    ibl.bake_tc(chain, w, h, half, rough, irradiance=_dev(16, 32, 4, dtype=torch.float16),
                stream=s)
    names = [n for n, _ in recorder.calls]
    assert names == ["althea_ibl_build_env_chain", "althea_ibl_prefilter",
                     "althea_ibl_irradiance", "althea_ibl_bake_tc_ex", "althea_ibl_tc_error",
                     "althea_ibl_bake_tc_ex", "althea_ibl_tc_error"]
    args = dict(recorder.calls[1:2])["althea_ibl_prefilter"]
    arr, n = args[3], args[4]
    assert n == 3
    assert [(arr[k].width, arr[k].height, arr[k].pitch_bytes) for k in range(n)] == \
        [(mw, mh, mw * 16) for mw, mh in sizes]
    irr_args = recorder.calls[2][1]
    assert irr_args[4:7] == (32, 16, 32 * 16)
    assert irr_args[8] >= ibl.load().althea_ibl_irradiance_workspace_size(w, h, 32, 16) > 0
    tc32, tc16 = recorder.calls[3][1], recorder.calls[5][1]
    assert tc32[-2] == ibl.FORMAT_RGBA32F and tc16[-2] == ibl.FORMAT_RGBA16F
    assert tc16[3][1].pitch_bytes == 64 * 8  # RGBA16F rows


def test_context_bake_passes_every_output(recorder):
    cfg = ibl.make_config(256, 128, irradiance_size=(32, 16), mip_count=3, lut_size=16)
    ctx = _FakeContext(cfg)
    irr = _dev(16, 32, 4)
    mips = [_dev(ctx.mip_info(m)[1], ctx.mip_info(m)[0], 4) for m in range(3)]
    lut = _dev(16, 16, 2)
    ctx.bake(irr, mips, lut, _Stream())
    (name, args), = recorder.calls
    assert name == "althea_ibl_bake"
    o = args[1]._obj
    assert o.irradiance_pitch_bytes == 32 * 16
    assert [o.mip_pitch_bytes[m] for m in range(3)] == [128 * 16, 64 * 16, 32 * 16]
    assert o.mip_dev[3] is None and o.lut_pitch_bytes == 16 * 8
