"""CPU checks of the drop-in's host side: the command-line tools keep the
reference's argv contract and usage text (src/bench_runner.cpp:7-103,
src/tests_main.cpp:6-50), their CPU algorithm runs end to end, and the
library's own `fwBaselineCPU` / `hasNegativeCycle` (the reference's C++
symbols, include/fw103_algorithms.h) give the reference's results. Nothing
here touches a GPU: only the "baseline_cpu" algorithm is run."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import load_json, sha

INF = 1_000_000_000


@pytest.fixture(scope="module")
def tools(fw):
    from fw_cuda_gb300 import build

    bench = build.tool_path("bench_runner")
    tests = build.tool_path("tests_runner")
    if not (os.path.exists(bench) and os.path.exists(tests)):
        build.build()
    return bench, tests


def run(args, timeout=300):
    return subprocess.run(args, capture_output=True, text=True, timeout=timeout)


# ------------------------------------------------------------------ bench_runner argv
BENCH_USAGE_LINES = [
    "<algorithm_name> <n_size> <density> [seed] [tile_size] [kappa]",
    "Arguments:",
    "  algorithm_name  Name of the algorithm to run",
    "  n_size          Graph size (number of vertices, 1 to 32769)",
    "  density         Edge density (0.0 to 1.0)",
    "  seed            Random seed (optional, 0 for random)",
    "  tile_size       Tile size for tiling/CUDA (optional)",
    "  kappa           Number of tile-layers to group (optional, used by multi_layer_tiling_gpu)",
    "Examples:",
    " baseline_cpu 1024 0.8",
    " baseline_gpu 2048 0.9 42 16",
    " multi_layer_tiling_gpu 4096 0.9 42 32 4",
]


@pytest.mark.parametrize("argv", [[], ["baseline_cpu"], ["baseline_cpu", "64"],
                                  ["baseline_cpu", "64", "0.5", "1", "32", "4", "extra"]])
def test_bench_runner_usage(tools, argv):
    r = run([tools[0], *argv])
    assert r.returncode == 1
    assert r.stderr.startswith("Usage: ")
    for line in BENCH_USAGE_LINES:
        assert line in r.stderr, line
    assert r.stdout == ""


@pytest.mark.parametrize("argv,message", [
    (["baseline_cpu", "0", "0.5"], "ERROR: Invalid graph size (0). Must be between 1 and 32769."),
    (["baseline_cpu", "40000", "0.5"], "ERROR: Invalid graph size (40000). Must be between 1 and 32769."),
    (["baseline_cpu", "abc", "0.5"], "ERROR: Invalid N_SIZE provided (abc). Must be an integer."),
    (["baseline_cpu", "64", "1.5"], "ERROR: Invalid density (1.5). Must be between 0.0 and 1.0."),
    (["baseline_cpu", "64", "-0.5"], "ERROR: Invalid density (-0.5). Must be between 0.0 and 1.0."),
    (["baseline_cpu", "64", "dense"], "ERROR: Invalid DENSITY provided (dense). Must be a floating point number."),
    (["baseline_cpu", "64", "0.5", "x"], "ERROR: Invalid SEED provided (x). Must be an unsigned integer."),
    (["baseline_cpu", "64", "0.5", "1", "65"], "ERROR: Invalid TILE_SIZE (65). Must be between 0 and 64."),
    (["baseline_cpu", "64", "0.5", "1", "-1"], "ERROR: Invalid TILE_SIZE (-1). Must be between 0 and 64."),
    (["baseline_cpu", "64", "0.5", "1", "t"], "ERROR: Invalid TILE_SIZE provided (t). Must be an integer."),
    (["baseline_cpu", "64", "0.5", "1", "32", "-2"], "ERROR: Invalid KAPPA (-2). Must be non-negative."),
    (["baseline_cpu", "64", "0.5", "1", "32", "k"], "ERROR: Invalid KAPPA provided (k). Must be an integer."),
])
def test_bench_runner_rejects_bad_arguments(tools, argv, message):
    r = run([tools[0], *argv])
    assert r.returncode == 1
    assert message in r.stderr


def test_bench_runner_unknown_algorithm(tools):
    r = run([tools[0], "nope", "16", "0.5", "1"])
    assert r.returncode == 1
    assert "RUNTIME ERROR: ERROR: Unsupported CPU algorithm: nope" in r.stderr


def test_bench_runner_baseline_cpu(tools):
    r = run([tools[0], "baseline_cpu", "256", "0.9", "42", "32", "4"])
    assert r.returncode == 0, r.stderr
    out = r.stdout
    for line in ("BENCHMARK: baseline_cpu", "Graph size: 256 vertices", "Edge density: 90.0%", "Tile size: 32",
                 "Kappa: 4", "Algorithm type: CPU", "Seed: 42 (Reproducible)", "Generating graph...",
                 "Running baseline_cpu...", "Results:"):
        assert line in out, line
    secs = [l for l in out.splitlines() if l.startswith("Execution time: ")]
    assert len(secs) == 1 and secs[0].endswith(" seconds")
    assert float(secs[0].split()[2]) > 0
    thr = [l for l in out.splitlines() if l.startswith("Throughput: ")]
    assert len(thr) == 1 and float(thr[0].split()[1]) > 0


# ------------------------------------------------------------------ tests_runner
def test_tests_runner_usage_and_errors(tools):
    r = run([tools[1]])
    assert r.returncode == 1 and r.stderr.startswith("Usage: ")
    for line in ("<algorithm_name> [tile_size] [kappa]", "  tile_size       Tile size (optional, default 0)",
                 " multi_layer_tiling_gpu 32 4"):
        assert line in r.stderr
    r = run([tools[1], "baseline_cpu", "x"])
    assert r.returncode == 1 and "ERROR: Invalid TILE_SIZE provided (x). Must be an integer." in r.stderr
    r = run([tools[1], "baseline_cpu", "32", "y"])
    assert r.returncode == 1 and "ERROR: Invalid KAPPA provided (y). Must be an integer." in r.stderr
    r = run([tools[1], "nope"])
    assert r.returncode == 1 and "ERROR: ERROR: Unsupported CPU algorithm: nope" in r.stderr


def test_tests_runner_baseline_cpu_suite(tools):
    r = run([tools[1], "baseline_cpu", "32"])
    assert r.returncode == 0, r.stderr
    assert "TESTING: baseline_cpu (tileSize=32)" in r.stdout
    assert r.stdout.count("[ PASSED ]") == 10
    assert "RESULTS: 10/10 passed" in r.stdout
    assert "[ FAILED ]" not in r.stdout + r.stderr


# ------------------------------------------------------------------ library C++ symbols
def _cpp(fw, mangled, argtypes, restype):
    f = getattr(fw.lib(), mangled)
    f.argtypes = argtypes
    f.restype = restype
    return f


def test_library_baseline_cpu_matches_reference(fw):
    """fwBaselineCPU of libfw103.so (the runners' baseline_cpu and the
    comparison reference of tests_runner) on the reference's known answers and
    on the reference-generated inputs, by their fwBaselineCPU output hashes."""
    cpu = _cpp(fw, "_Z13fwBaselineCPUPiii", [ctypes.c_void_p, ctypes.c_int, ctypes.c_int], None)
    neg = _cpp(fw, "_Z16hasNegativeCyclePKii", [ctypes.c_void_p, ctypes.c_int], ctypes.c_bool)
    data = load_json("known_answer.json")
    for case in data["cases"]:
        n = case["n"]
        a = np.array(case["input"], dtype=np.int32).reshape(n, n).copy()
        cpu(a.ctypes.data, n, 0)
        assert a.ravel().tolist() == case["reference_output"], case["name"]
        assert bool(neg(a.ctypes.data, n)) == case["reference_negative_cycle"], case["name"]
    for c in load_json("reference_cases.json")["cases"]:
        if c["n"] > 1024:
            continue
        a = fw.generate_graph(c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
        assert sha(a) == c["input_sha256"], c["id"]
        cpu(a.ctypes.data, c["n"], 32)
        assert sha(a) == c["output_sha256"], c["id"]
