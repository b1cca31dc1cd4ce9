"""The irradiance entry point that allocates nothing.

Some callers cannot call cudaMalloc -- a renderer that owns all device memory
through its own allocator and budget, a plug-in with a fixed memory envelope,
code running inside a frame or real-time callback where an allocation may
stall the device.  althea_ibl_irradiance_noalloc serves them: the caller
passes only the env chain and the output, and the partial sums live in a
fixed array inside the library.  This file checks, through the C ABI, that
two calls in a row give the same irradiance as althea_ibl_irradiance (with its
caller-provided workspace), and that outputs too large for the fixed array
are refused.  It is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import oracle
from althea_gb300 import ibl, synth

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-4  # the per-texel relative tolerance of the plain path


def _noalloc():
    L = ibl.load()
    f = L.althea_ibl_irradiance_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
    return L, f


def _rel_err(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return (np.abs(a - b) / np.maximum(np.abs(b), 1e-6 * np.abs(b).max())).max()


def test_noalloc_irradiance_matches_workspace_variant_twice():
    L, noalloc = _noalloc()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(512, 256, 32, 16, 3), (256, 128, 64, 32, 4)]
    for w, h, ow, oh, seed in cases:  # two calls in a row, different inputs and sizes
        env = synth.make_env(w, h, seed=seed, sun_max=1e4)
        chain = torch.from_numpy(oracle.build_chain(env)).cuda()
        ref = torch.empty((oh, ow, 4), dtype=torch.float32, device="cuda")
        ibl.irradiance(chain, w, h, ref)
        got = torch.full((oh, ow, 4), float("nan"), dtype=torch.float32, device="cuda")
        st = noalloc(chain.data_ptr(), w, h, got.data_ptr(), ow, oh, ow * 16, stream)
        assert st == ibl.OK, L.althea_ibl_last_error()
        torch.cuda.synchronize()
        assert _rel_err(got.cpu().numpy(), ref.cpu().numpy()) <= TOL


def test_noalloc_rejects_outputs_beyond_its_fixed_scratch():
    L, noalloc = _noalloc()
    w, h, ow, oh = 2048, 1024, 1024, 512
    chain = torch.zeros((ibl.chain_texels(w, h), 4), dtype=torch.float32, device="cuda")
    out = torch.empty((oh, ow, 4), dtype=torch.float32, device="cuda")
    st = noalloc(chain.data_ptr(), w, h, out.data_ptr(), ow, oh, ow * 16, None)
    assert st == ibl.ERR_UNSUPPORTED
    assert b"no-allocation" in L.althea_ibl_last_error()
