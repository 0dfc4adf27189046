"""The drop-in as the reference's users see it, on the GPU.

* The exported C++ symbols with the AlgorithmFuncGPU signature
  (include/algo_types.h:9): fwBaselineGPU, fwTilingGPU and
  fwMultiLayerTilingGPU of libfw103.so, called by their C++ names on the
  reference's known answers (src/tests.cpp:59-132) and on the reference's
  generated cases (fwBaselineCPU output hashes).
* The command-line tools: tests_runner's GPU suite (src/tests_gpu.cu:156-185)
  and one bench_runner run (src/bench_runner.cpp:24-103).
* Failure status: a missed tile copy is reported by fw_check_faults, by the
  Python registry (an exception) and by the C++ shims (print and exit 1, as
  the reference's checkCudaErrors does, include/cuda_utils.cuh:13-32). The
  misses are injected on the host (fw_debug_inject); the only device-side
  wait that runs out is fw_debug_bounded_wait's, on a copy that is never
  issued, after which the context is still used for a correct solve.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, load_json, sha

pytestmark = pytest.mark.gpu

SHIMS = {
    "baseline_gpu": "_Z13fwBaselineGPUPiiii",
    "tiling_gpu": "_Z11fwTilingGPUPiiii",
    "multi_layer_tiling_gpu": "_Z21fwMultiLayerTilingGPUPiiii",
}


def shim(fw, name):
    f = getattr(fw.lib(), SHIMS[name])
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    f.restype = None
    return f


@pytest.mark.parametrize("name", list(SHIMS))
def test_cpp_symbols_known_answers(fw, cuda, name):
    f = shim(fw, name)
    for case in load_json("known_answer.json")["cases"]:
        n = case["n"]
        d = cuda.tensor(case["input"], dtype=cuda.int32, device="cuda")
        f(d.data_ptr(), n, 32, 4)  # synchronises, like the reference's launchers
        assert d.cpu().tolist() == case["reference_output"], (name, case["name"])


@pytest.mark.parametrize("name,kappa", [("baseline_gpu", 0), ("tiling_gpu", 0), ("multi_layer_tiling_gpu", 4),
                                        ("multi_layer_tiling_gpu", 8)])
def test_cpp_symbols_reference_cases(fw, cuda, name, kappa):
    f = shim(fw, name)
    for c in load_json("reference_cases.json")["cases"]:
        if c["n"] > 1024 or (name == "baseline_gpu" and c["n"] > 512):
            continue
        a = fw.generate_graph(c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
        assert sha(a) == c["input_sha256"]
        d = cuda.from_numpy(a).cuda()
        f(d.data_ptr(), c["n"], 32, kappa)
        assert sha(d.cpu().numpy()) == c["output_sha256"], (name, kappa, c["id"])


@pytest.fixture(scope="module")
def tools(fw):
    from fw_cuda_gb300 import build

    if not os.path.exists(build.tool_path("tests_runner")):
        build.build()
    return build.tool_path("bench_runner"), build.tool_path("tests_runner")


@pytest.mark.parametrize("name", list(SHIMS))
def test_tests_runner_gpu_suite(tools, name):
    r = subprocess.run([tools[1], name, "32", "4"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"TESTING (GPU): {name} (tileSize=32, kappa=4)" in r.stdout
    assert r.stdout.count("[ PASSED ]") == 14
    assert "RESULTS: 14/14 passed" in r.stdout
    assert "[ FAILED ]" not in r.stdout + r.stderr


def test_bench_runner_gpu(tools):
    r = subprocess.run([tools[0], "multi_layer_tiling_gpu", "1024", "0.9", "42", "32", "4"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for line in ("BENCHMARK: multi_layer_tiling_gpu", "Graph size: 1024 vertices", "Algorithm type: GPU",
                 "Warming up GPU...", "Copying graph to GPU...", "Running multi_layer_tiling_gpu..."):
        assert line in r.stdout, line
    secs = [l for l in r.stdout.splitlines() if l.startswith("Execution time: ")]
    assert len(secs) == 1 and 0 < float(secs[0].split()[2]) < 10


# ------------------------------------------------------------------ failure status
def test_clean_call_has_no_faults(fw, cuda):
    W = fw.generate_graph(700, 0.4, 3, 1, 100)
    d = cuda.from_numpy(W).cuda()
    before = fw.copy_faults()
    fw.apsp_i32(d, 700, 32, 4, fw.VARIANT_MULTI_LAYER, None)
    fw.check_faults(None)  # no exception
    assert fw.copy_faults() == before == 0


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_injected_miss_is_reported_then_cleared(fw, cuda, oracle, variant):
    n = 500
    W = fw.generate_graph(n, 0.4, 11, 1, 100)
    d = cuda.from_numpy(W).cuda()
    fw.debug_inject(fw.INJECT_CALL_FAULT)
    fw.apsp_i32(d, n, 32, 8, variant, None)
    with pytest.raises(fw.FwError) as e:
        fw.check_faults(None)
    assert e.value.status == fw.FW_ERR_TIMEOUT
    assert "not valid" in str(e.value)
    # the next call resets its status word
    d = cuda.from_numpy(W).cuda()
    fw.apsp_i32(d, n, 32, 8, variant, None)
    fw.check_faults(None)
    assert np.array_equal(d.cpu().numpy(), oracle.fw_i32(W))


def test_injected_miss_python_registry_raises(fw, cuda):
    W = fw.generate_graph(300, 0.5, 12, 1, 100)
    d = cuda.from_numpy(W).cuda()
    fw.debug_inject(fw.INJECT_CALL_FAULT)
    with pytest.raises(fw.FwError) as e:
        fw.get_gpu_algorithm_func("tiling_gpu")(d, 300, 32, 4)
    assert e.value.status == fw.FW_ERR_TIMEOUT


_SHIM_CHILD = r"""
import ctypes, sys
import torch
sys.path.insert(0, {root!r})
import fw_cuda_gb300 as F
L = F.lib()
f = getattr(L, {sym!r})
f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
f.restype = None
d = torch.from_numpy(F.generate_graph(256, 0.5, 9, 1, 100)).cuda()
torch.cuda.synchronize()
if {inject}:
    F.debug_inject(F.INJECT_CALL_FAULT)
f(d.data_ptr(), 256, 32, 4)
print("returned")
"""


@pytest.mark.parametrize("name", list(SHIMS))
def test_cpp_shim_exits_on_injected_miss(fw, cuda, name):
    for inject in (False, True):
        code = _SHIM_CHILD.format(root=ROOT, sym=SHIMS[name], inject=inject)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
        if inject:
            assert r.returncode == 1, r.stdout + r.stderr
            assert "returned" not in r.stdout
            assert f"fw103 error in {name} (status 4)" in r.stderr
        else:
            assert r.returncode == 0 and "returned" in r.stdout, r.stdout + r.stderr


def test_injected_packed_miss_falls_back_to_int32(fw, cuda, oracle):
    n = 2200  # above 2048, where AUTO takes the packed path
    W = fw.generate_graph(n, 0.5, 21, 1, 100)
    ref = W.copy()
    oracle.fw_i32_pivots(ref, 0, n, threads=os.cpu_count() or 1)
    d = cuda.from_numpy(W).cuda()
    fw.apsp_i32(d, n, 32, 8, fw.VARIANT_AUTO, None)
    assert fw.auto_used_packed(None)
    assert np.array_equal(d.cpu().numpy(), ref)
    d = cuda.from_numpy(W).cuda()
    fw.debug_inject(fw.INJECT_PACKED_FAULT)
    fw.apsp_i32(d, n, 32, 8, fw.VARIANT_AUTO, None)
    assert not fw.auto_used_packed(None)  # the packed result was refused
    fw.check_faults(None)  # and the int32 sweep that ran missed nothing
    assert np.array_equal(d.cpu().numpy(), ref)


def test_injected_miss_next_hop_forward(fw, cuda):
    from fw_cuda_gb300 import autograd as A
    from fw_cuda_gb300 import workloads

    W = cuda.from_numpy(workloads.diff_graph(200, np.random.default_rng(3))).cuda()
    fw.debug_inject(fw.INJECT_CALL_FAULT)
    A.forward_with_next_hops(W, None)
    with pytest.raises(fw.FwError) as e:
        fw.check_faults(None)
    assert e.value.status == fw.FW_ERR_TIMEOUT
    A.forward_with_next_hops(W, None)
    fw.check_faults(None)


def test_injected_miss_out_of_core(fw, cuda, oracle):
    n = 600
    W = fw.generate_graph(n, 0.5, 31, 1, 100)
    h = W.copy()
    fw.debug_inject(fw.INJECT_CALL_FAULT)
    with pytest.raises(fw.FwError) as e:
        fw.apsp_i32_host(h, n, 256, 256)
    assert e.value.status == fw.FW_ERR_TIMEOUT
    h = W.copy()
    fw.apsp_i32_host(h, n, 256, 256)
    assert np.array_equal(h, oracle.fw_i32(W))


def test_bounded_wait_gives_up_and_context_stays_usable(fw, cuda, oracle):
    before = fw.copy_faults()
    assert fw.debug_bounded_wait(1000, None) == fw.FW_ERR_TIMEOUT
    assert b"gave up" in fw.lib().fw_last_error_string()
    # a wait whose copy never comes is not a copy fault of any sweep
    assert fw.copy_faults() == before
    W = fw.generate_graph(400, 0.5, 41, 1, 100)
    d = cuda.from_numpy(W).cuda()
    fw.apsp_i32(d, 400, 32, 4, fw.VARIANT_TILING, None)
    fw.check_faults(None)
    assert np.array_equal(d.cpu().numpy(), oracle.fw_i32(W))
