"""Failure detection on the GPU without a fault: the tensor-core kernels' bounded mbarrier wait,
run by a test hook on a barrier that nothing completes, gives up, records the device error, and
ngp_device_status() reports it once; the context stays usable (a kernel run afterwards gives the
right results)."""
import ctypes
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports():
    from jaxngp_gb300 import _lib as L
    lib = L.lib()
    lib.ngp_selftest_bounded_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint]
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.ngp_device_status() == 0   # nothing pending
    t = time.perf_counter()
    assert lib.ngp_selftest_bounded_wait(stream, 4096) == 0
    st = lib.ngp_device_status()   # synchronises: the wait has run out by now
    waited = time.perf_counter() - t
    assert st == 4, (st, lib.ngp_last_status_message())   # NGP_ERR_DEVICE
    assert b"gave up" in lib.ngp_last_status_message()
    assert lib.ngp_device_status() == 0   # reported once, then cleared
    assert waited < 10.0
    # the context is intact: a kernel afterwards computes the right Morton codes
    from jaxngp_gb300 import volrendjax as vr
    from oracle import volrend as V
    xyz = np.random.default_rng(0).integers(0, 1024, size=(4096, 3)).astype(np.uint32)
    got = vr.morton3d(torch.from_numpy(xyz.astype(np.int32)).cuda()).cpu().numpy().astype(np.uint32)
    assert np.array_equal(got, V.morton3d(xyz))
    # out-of-contract poll counts are refused before any launch
    assert lib.ngp_selftest_bounded_wait(stream, 0) == 2
    assert lib.ngp_selftest_bounded_wait(stream, (1 << 20) + 1) == 2
