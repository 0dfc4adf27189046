"""fw_apsp_i32_noalloc: the entry point for callers that cannot allocate
device memory (their pool owns the GPU's free memory, or they must avoid the
synchronisation a cudaMalloc brings). It must give exactly what fw_apsp_i32
gives, call after call, while taking its workspace from the library's fixed
8 MiB device array instead of allocating one. This file is collected last so
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
