"""CPU-side checks of the C ABI: the library loads, exports every symbol the
public header declares, and rejects bad arguments before touching a device
(no compute call is made here)."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, sha, load_json


def declared_symbols() -> set[str]:
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        # C declarations at file scope: "<type> fw_name(" (not typedef / macros)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(fw_[a-z0-9_]+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declarations_are_exported(fw):
    names = declared_symbols()
    assert "fw_apsp_i32" in names and "fw_last_error_string" in names
    L = fw.lib()
    for name in sorted(names):
        assert hasattr(L, name), f"{name} declared in include/ but not exported"
    assert set(fw.EXPORTED_SYMBOLS) <= names


def test_version(fw):
    assert "sm_103a" in fw.version()


def test_bad_arguments_fail_before_any_device_work(fw):
    L = fw.lib()
    # NULL matrix
    assert L.fw_apsp_i32_ws(None, 16, 0, 0, 1, None, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"NULL" in L.fw_last_error_string()
    fake = 0x7F0000000000  # never dereferenced: every check below fails first
    assert L.fw_apsp_i32_ws(fake, 0, 0, 0, 1, None, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_apsp_i32_ws(fake, -5, 0, 0, 1, None, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_apsp_i32_ws(fake, 16, 0, 0, 7, None, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"variant" in L.fw_last_error_string()
    assert L.fw_apsp_i32_ws(fake + 4, 16, 0, 0, 1, None, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"aligned" in L.fw_last_error_string()
    # workspace missing / too small / misaligned
    need = L.fw_workspace_bytes_i32(1000, 32, 4, 2)
    assert need > 0
    assert L.fw_apsp_i32_ws(fake, 1000, 32, 4, 2, None, need, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_apsp_i32_ws(fake, 1000, 32, 4, 2, fake, 4096, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"workspace" in L.fw_last_error_string()
    assert L.fw_apsp_i32_ws(fake, 1000, 32, 4, 2, fake + 16, need, None) == fw.FW_ERR_INVALID_ARGUMENT
    # the per-pivot sweep puts one row per grid row
    assert L.fw_apsp_i32_ws(fake, 70000, 0, 0, 0, fake, 1 << 40, None) == fw.FW_ERR_INVALID_ARGUMENT


def test_host_solve_arguments(fw):
    L = fw.lib()
    fake = 0x7F0000000000  # never dereferenced: every check below fails first
    assert L.fw_apsp_i32_host(None, 16, 0, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"NULL" in L.fw_last_error_string()
    assert L.fw_apsp_i32_host(fake, 0, 0, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_apsp_i32_host(fake, 3_000_000, 0, 0, None) == fw.FW_ERR_INVALID_ARGUMENT
    for bad_w in (-128, 100, 64):
        assert L.fw_apsp_i32_host(fake, 1000, bad_w, 128, None) == fw.FW_ERR_INVALID_ARGUMENT
        assert b"pass_width" in L.fw_last_error_string()
    for bad_h in (-128, 200):
        assert L.fw_apsp_i32_host(fake, 1000, 256, bad_h, None) == fw.FW_ERR_INVALID_ARGUMENT
        assert b"stripe_rows" in L.fw_last_error_string()
    with pytest.raises(ValueError):
        fw.apsp_i32_host(np.zeros((4, 4), dtype=np.int64), 4)
    # device bytes: four W x ldp panels, the n x W column stripe, Dg, two
    # padded copies of Dg*, three H x n stripes
    n, W, H = 1000, 256, 384
    ldp = 1024
    want = 4 * (4 * W * ldp + n * W + W * W + 2 * W * W + 3 * H * n)
    assert fw.host_solve_device_bytes(n, W, H) == want
    assert fw.host_solve_device_bytes(100, 0, 128) == 4 * (4 * 128 * 128 + 100 * 128 + 128 * 128 + 2 * 128 * 128
                                                           + 3 * 128 * 100)
    assert fw.host_solve_device_bytes(n, W, 0) == 0


def test_workspace_sizes(fw):
    # every workspace starts with a 256-byte status block (the call's missed
    # copy count); blocked: two buffers of two 128-row panels (look-ahead or
    # the two-block pass), leading dimension padded to 128
    status = 256
    assert fw.workspace_bytes_i32(1, variant=1) == status + 2 * 256 * 128 * 4
    assert fw.workspace_bytes_i32(32768, variant=2) == status + 2 * 256 * 32768 * 4
    assert fw.workspace_bytes_i32(32769, variant=2) == status + 2 * 256 * (32768 + 128) * 4
    assert fw.workspace_bytes_i32(32768, kappa=8, variant=1) == status + 2 * 256 * 32768 * 4
    # n <= 2048 (blocked variants and AUTO): at least the stripe sweep's
    # published pivot rows (8 * ceil(n / 8) rows of 128 * ceil(n / 128) ints)
    # and one flag per stripe, each part rounded up to 256 bytes
    assert fw.workspace_bytes_i32(1024, variant=1) == status + 128 * 8 * 1024 * 4 + 512
    assert fw.workspace_bytes_i32(1000, variant=2) == status + 125 * 8 * 1024 * 4 + 512
    assert fw.workspace_bytes_i32(2048, variant=2) == status + 256 * 8 * 2048 * 4 + 1024
    assert fw.workspace_bytes_i32(2049, variant=2) == status + 2 * 256 * 2176 * 4
    # per-pivot: two row and two column snapshots
    assert fw.workspace_bytes_i32(1001, variant=0) == status + 4 * 1004 * 4
    assert fw.workspace_bytes_i32(0, variant=1) == 0


def test_fault_hooks_reject_bad_arguments(fw):
    L = fw.lib()
    assert L.fw_debug_inject(4) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"unknown kind" in L.fw_last_error_string()
    assert L.fw_debug_inject(0) == fw.FW_OK
    for spins in (0, -1, (1 << 20) + 1):
        assert L.fw_debug_bounded_wait(spins, None) == fw.FW_ERR_INVALID_ARGUMENT
        assert b"spins" in L.fw_last_error_string()
    for limit in (0, -5, 1000001):
        assert L.fw_debug_flag_wait(limit, None) == fw.FW_ERR_INVALID_ARGUMENT
        assert b"limit_us" in L.fw_last_error_string()


def test_noalloc_rejects_before_device_work(fw):
    L = fw.lib()
    fake = 0x7F0000000000  # never dereferenced: the size check fails first
    assert L.fw_apsp_i32_noalloc(fake, 8193, 32, 4, 2, None) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"8192" in L.fw_last_error_string()
    assert L.fw_apsp_i32_noalloc(None, 100, 32, 4, 2, None) == fw.FW_ERR_INVALID_ARGUMENT


def test_generator_matches_reference_hashes(fw, oracle):
    for c in load_json("reference_cases.json")["cases"]:
        if c["n"] > 1024:
            continue
        a = fw.generate_graph(c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
        assert sha(a) == c["input_sha256"], c["id"]
    a = fw.generate_graph(77, 0.4, 5, 1, 100)
    assert np.array_equal(a, oracle.generate_graph(77, 0.4, 5, 1, 100))
    assert a.min() == 0 and a[a < fw.INF].max() <= 100
    assert np.all(np.diag(a) == 0)


def test_generator_rejects_bad_arguments(fw):
    L = fw.lib()
    buf = np.empty(16, dtype=np.int32)
    assert L.fw_generate_graph_i32(None, 4, 0.5, 1, 0, 10) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_generate_graph_i32(buf.ctypes.data, 4, 1.5, 1, 0, 10) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_generate_graph_i32(buf.ctypes.data, 4, 0.5, 1, 10, 0) == fw.FW_ERR_INVALID_ARGUMENT
    assert L.fw_generate_graph_i32(buf.ctypes.data, 0, 0.5, 1, 0, 10) == fw.FW_ERR_INVALID_ARGUMENT


def test_registry_mirrors_reference(fw):
    assert set(fw.GPU_ALGORITHMS) == {"baseline_gpu", "tiling_gpu", "multi_layer_tiling_gpu"}
    assert fw.is_gpu_algorithm("tiling_gpu") and not fw.is_gpu_algorithm("baseline_cpu")
    try:
        fw.get_gpu_algorithm_func("nope")
    except KeyError as e:
        assert "Unsupported GPU algorithm: nope" in str(e)
    else:
        raise AssertionError("expected KeyError")


def test_library_missing_fails_loudly(monkeypatch):
    import fw_cuda_gb300 as F

    monkeypatch.setattr(F, "_lib", None)
    monkeypatch.setattr(F, "library_path", lambda: "/nonexistent/libfw103.so")
    try:
        F.lib()
    except F.FwLibraryMissing as e:
        assert "not found" in str(e)
    else:
        raise AssertionError("expected FwLibraryMissing")
    assert ctypes is not None


class _FakeCudaTensor:
    """Stands in for a CUDA tensor: the Python view checks dtype and size before
    the C call, so none of these reaches the library."""

    is_cuda = True

    def __init__(self, dtype: str, numel: int):
        self.dtype, self._numel = dtype, numel

    def is_contiguous(self):
        return True

    def data_ptr(self):
        return 1 << 20

    def numel(self):
        return self._numel

    def element_size(self):
        return 4


def test_tensor_arguments_are_checked_before_the_call(fw):
    T = _FakeCudaTensor
    n = 10
    with pytest.raises(TypeError):
        fw.apsp_i32(T("torch.float32", n * n), n)
    with pytest.raises(ValueError):
        fw.apsp_i32(T("torch.int32", n * n - 1), n)
    with pytest.raises(ValueError):
        fw.generate_graph_device(T("torch.int32", 50), n, 0.5, 1)
    with pytest.raises(ValueError):
        fw.apsp_paths_i32(T("torch.int32", 3 * n * n), T("torch.int32", 3 * n * n - 1), n, 3)
    with pytest.raises(TypeError):
        fw.negative_cycle_flags(T("torch.int32", 2 * n * n), n, 2, T("torch.int64", 2))
    with pytest.raises(ValueError):
        fw.apsp_i32_ws(T("torch.int32", n * n), n, T("torch.int32", 8), 64)
    with pytest.raises(TypeError):
        fw.dense_from_csr(T("torch.int32", n + 1), None, None, n, T("torch.int32", n * n))
    with pytest.raises(ValueError):
        fw.apsp_i32_host(np.zeros(n * n - 1, dtype=np.int32), n)
