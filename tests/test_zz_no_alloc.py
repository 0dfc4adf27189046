"""fw_apsp_i32_noalloc: the entry point for callers that cannot allocate
device memory (their pool owns the GPU's free memory, or they must avoid the
synchronisation a cudaMalloc brings). It must give exactly what fw_apsp_i32
gives, call after call, while taking its workspace from the library's fixed
device array (8 MiB + 256 bytes) instead of allocating one. This file is collected last so
that a run stopping at its first failure has already run every other test."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(fw):
    L = fw.lib()
    f = L.fw_apsp_i32_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


@pytest.mark.parametrize("n,variant,kappa", [(1000, 2, 4), (8192, 2, 4), (8192, 2, 8), (777, 1, 4), (300, 0, 4)])
def test_noalloc_matches_allocating_entry_point_twice(fw, cuda, n, variant, kappa):
    f = _noalloc(fw)
    W = fw.generate_graph(n, 0.3, 4242 + n, 1, 100)
    ref = cuda.from_numpy(W).cuda()
    fw.apsp_i32(ref, n, 32, kappa, variant, None)
    cuda.cuda.synchronize()
    expected = ref.cpu().numpy()
    for call in range(2):  # the second call sees the scratch the first one left behind
        d = cuda.from_numpy(W).cuda()
        rc = f(d.data_ptr(), n, 32, kappa, variant, None)
        assert rc == fw.FW_OK, fw.lib().fw_last_error_string()
        cuda.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), expected), (n, variant, call)


def test_noalloc_rejects_graphs_beyond_its_scratch(fw, cuda):
    f = _noalloc(fw)
    d = cuda.zeros(16, dtype=cuda.int32, device="cuda")
    rc = f(d.data_ptr(), 8193, 32, 4, 2, None)
    assert rc == fw.FW_ERR_INVALID_ARGUMENT
    assert b"8192" in fw.lib().fw_last_error_string()


@pytest.mark.parametrize("n,variant", [(8192, 2), (1024, 0)])
def test_noalloc_allocates_no_device_memory(fw, cuda, n, variant):
    """The defining property: once the library is loaded (the first call looks
    up the array, which loads the module that holds it), a call on a stream
    the library has never seen leaves the device's free memory unchanged. At
    n = 1024 the allocating entry point would replay the per-pivot sweep from
    a captured CUDA graph; this one must launch directly."""
    f = _noalloc(fw)
    W = fw.generate_graph(n, 0.3, 77, 1, 100)
    d = cuda.from_numpy(W).cuda()
    warm = cuda.from_numpy(W).cuda()
    assert f(warm.data_ptr(), n, 32, 4, variant, None) == fw.FW_OK
    cuda.cuda.synchronize()
    s = cuda.cuda.Stream()
    free_before, _ = cuda.cuda.mem_get_info()
    rc = f(d.data_ptr(), n, 32, 4, variant, s.cuda_stream)
    assert rc == fw.FW_OK, fw.lib().fw_last_error_string()
    s.synchronize()
    free_after, _ = cuda.cuda.mem_get_info()
    assert free_after == free_before
    assert np.array_equal(d.cpu().numpy(), warm.cpu().numpy())
    fw.check_faults(s)  # its status word lives in the fixed array too


def test_noalloc_auto_runs_int32_and_drops_the_auto_report(fw, cuda):
    f = _noalloc(fw)
    n = 2100  # above 2048, where the allocating entry point's AUTO takes the packed path
    W = fw.generate_graph(n, 0.5, 78, 1, 100)
    s = cuda.cuda.Stream()
    d = cuda.from_numpy(W).cuda()
    fw.apsp_i32(d, n, 32, 8, fw.VARIANT_AUTO, s)
    assert fw.auto_used_packed(s)
    expected = d.cpu().numpy()
    d = cuda.from_numpy(W).cuda()
    assert f(d.data_ptr(), n, 32, 8, fw.VARIANT_AUTO, s.cuda_stream) == fw.FW_OK
    s.synchronize()
    assert np.array_equal(d.cpu().numpy(), expected)
    with pytest.raises(fw.FwError) as e:
        fw.auto_used_packed(s)
    assert e.value.status == fw.FW_ERR_INVALID_ARGUMENT
