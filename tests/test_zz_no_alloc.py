"""The irradiance entry point that allocates nothing.

Some callers cannot call cudaMalloc -- a renderer that owns all device memory
through its own allocator and budget, a plug-in with a fixed memory envelope,
code running inside a frame or real-time callback where an allocation may
stall the device.  althea_ibl_irradiance_noalloc serves them: the caller
passes only the env chain and the output, and the partial sums live in a
fixed array inside the library.  This file checks, through the C ABI, that
calls in a row give the same irradiance, bit for bit, as althea_ibl_irradiance
(with its caller-provided workspace) -- the two run the same deterministic
kernels -- including an output whose partial sums fill the fixed array
exactly, and that one texel more is refused.  It is named to be collected
last.
"""
import ctypes

import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 4 * 1024 * 1024  # ALTHEA_IBL_NOALLOC_SCRATCH_BYTES


def _noalloc():
    L = ibl.load()
    f = L.althea_ibl_irradiance_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
    return L, f


def _check_same(L, noalloc, chain, w, h, ow, oh, stream):
    ref = torch.empty((oh, ow, 4), dtype=torch.float32, device="cuda")
    ibl.irradiance(chain, w, h, ref)
    got = torch.full((oh, ow, 4), float("nan"), dtype=torch.float32, device="cuda")
    st = noalloc(chain.data_ptr(), w, h, got.data_ptr(), ow, oh, ow * 16, stream)
    assert st == ibl.OK, L.althea_ibl_last_error()
    torch.cuda.synchronize()
    assert torch.equal(got, ref), (w, h, ow, oh)


def test_noalloc_irradiance_matches_workspace_variant_bitwise():
    L, noalloc = _noalloc()
    stream = torch.cuda.current_stream().cuda_stream
    # calls in a row, different inputs and sizes; the last fills the array
    # exactly (512 x 512 texels x one 16-byte partial sum each)
    cases = [(512, 256, 32, 16, 3), (256, 128, 64, 32, 4), (1024, 512, 512, 256, 5),
             (1024, 512, 512, 512, 6), (512, 256, 32, 16, 3)]
    for w, h, ow, oh, seed in cases:
        env = synth.make_env(w, h, seed=seed, sun_max=1e4)
        chain = torch.from_numpy(oracle.build_chain(env)).cuda()
        _check_same(L, noalloc, chain, w, h, ow, oh, stream)
    assert ibl.load().althea_ibl_irradiance_workspace_size(1024, 512, 512, 512) == SCRATCH_BYTES


def test_noalloc_rejects_outputs_beyond_its_fixed_scratch():
    L, noalloc = _noalloc()
    w, h = 1024, 512
    chain = torch.zeros((ibl.chain_texels(w, h), 4), dtype=torch.float32, device="cuda")
    # 545 x 481 = 262,145 texels: one partial sum more than the array holds
    for ow, oh in [(545, 481), (1024, 512)]:
        assert ibl.load().althea_ibl_irradiance_workspace_size(w, h, ow, oh) > SCRATCH_BYTES
        out = torch.full((oh, ow, 4), 7.0, dtype=torch.float32, device="cuda")
        st = noalloc(chain.data_ptr(), w, h, out.data_ptr(), ow, oh, ow * 16, None)
        assert st == ibl.ERR_UNSUPPORTED
        assert b"no-allocation" in L.althea_ibl_last_error()
        torch.cuda.synchronize()
        assert bool((out == 7.0).all())  # refused before any launch
