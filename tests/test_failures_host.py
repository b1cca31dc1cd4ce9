"""Failures injected on the host, without a GPU: with no usable CUDA device
every call that needs device memory, a stream or a launch fails cleanly --
an althea_ibl_status, a message naming the failed step, no handle handed
out -- and the Python layer turns each into an IBLError.  Nothing here
touches a GPU; on a machine that has one these tests are skipped (the GPU
tests cover the same paths succeeding)."""
import ctypes

import pytest

from althea_gb300 import ibl, serving

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.skipif(torch.cuda.is_available(),
                                reason="checks the failure paths of a machine without a GPU")


def _expect_cuda_error(status, handle, words):
    assert status == ibl.ERR_CUDA
    assert not handle.value
    msg = ibl.load().althea_ibl_last_error().decode()
    assert any(w in msg for w in words), msg


def test_context_creation_reports_the_device_failure():
    ctx = ctypes.c_void_p()
    cfg = ibl.make_config(64, 32)
    st = ibl.load().althea_ibl_create(ctypes.byref(cfg), ctypes.byref(ctx))
    _expect_cuda_error(st, ctx, ("cudaGetDevice", "allocation"))
    with pytest.raises(ibl.IBLError) as e:
        ibl.BakeContext(cfg)
    assert e.value.status == ibl.ERR_CUDA


def test_server_creation_reports_the_stream_failure():
    s = ctypes.c_void_p()
    cfg = ibl.ServerConfig(1 << 30, 4, 64, ibl.GEN_HAMMERSLEY, 32, 16, ibl.PATH_PLAIN)
    st = ibl.load().althea_ibl_server_create(ctypes.byref(cfg), ctypes.byref(s))
    _expect_cuda_error(st, s, ("stream",))
    with pytest.raises(ibl.IBLError) as e:
        serving.ProbeServer(budget_bytes=1 << 30)
    assert e.value.status == ibl.ERR_CUDA


def test_batch_creation_reports_the_allocation_failure():
    b = ctypes.c_void_p()
    params = ibl.BatchParams()
    params.samples, params.generator = 64, ibl.GEN_HAMMERSLEY
    st = ibl.load().althea_ibl_batch_create(None, 0, ctypes.byref(params), None, ctypes.byref(b))
    _expect_cuda_error(st, b, ("batch tables",))


def test_launches_report_instead_of_running():
    L = ibl.load()
    waited = ctypes.c_int(-1)
    assert L.althea_ibl_tc_wait_selftest(1_000_000, ctypes.byref(waited), None) == ibl.ERR_CUDA
    assert b"wait self-test" in L.althea_ibl_last_error()
    assert L.althea_ibl_tc_error(None, None) == ibl.ERR_INVALID_ARGUMENT
