"""ctypes view of the oracle libraries (test infrastructure only).

The oracle is the checker, never the product: only the test suite, the smoke
check and the benchmark's CPU-baseline / reference legs import this module.

* ``libfworacle.so`` (oracle/fw_oracle.cpp) — the CPU restatement of the
  reference's baseline_cpu sweep (src/fw_baseline_cpu.cpp:3-16), its graph
  generator (src/graph_generator.cpp:7-46) and the added checkers.
* ``libfwrefgpu.so`` (oracle/ref_gpu.cpp) + ``_ref/*.cubin`` — the reference's
  own GPU kernels, compiled from its sources, replayed with its launch loops.
* ``_ref/libfwref.so`` (oracle/ref_shim.cpp) — the reference's own CPU code;
  only exists where the reference checkout was present at build time.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")
INF = 1_000_000_000  # include/constants.h:3
MAX_N = 32769  # include/constants.h:5
MAX_EDGE_WEIGHT = 25_000  # include/constants.h:7

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i64 = ctypes.c_int64

_lib = None
_ref = None
_refgpu = None


def build() -> None:
    """Compile the oracle's own sources (and, where the reference checkout
    exists, the reference CPU library and kernel cubins)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    # The reference checkout: FW_REFERENCE_ROOT, else a directory named
    # `reference` beside this repository.
    ref_root = os.environ.get("FW_REFERENCE_ROOT",
                              os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
    if os.path.isdir(os.path.join(ref_root, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(BUILD, "libfworacle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_generate_graph.argtypes = [_i32p, _i64, ctypes.c_double, ctypes.c_uint32,
                                            ctypes.c_int32, ctypes.c_int32]
        L.oracle_generate_graph.restype = ctypes.c_int
        L.oracle_fw_i32.argtypes = [_i32p, _i64]
        L.oracle_fw_i32.restype = None
        L.oracle_fw_i32_pivots.argtypes = [_i32p, _i64, _i64, _i64, ctypes.c_int]
        L.oracle_fw_i32_pivots.restype = None
        L.oracle_has_negative_cycle.argtypes = [_i32p, _i64]
        L.oracle_has_negative_cycle.restype = ctypes.c_int
        L.oracle_sssp_dense.argtypes = [_i32p, _i64, _i64, _i32p]
        L.oracle_sssp_dense.restype = None
        L.oracle_fw_f64_nexthop.argtypes = [_f64p, _i32p, _i64]
        L.oracle_fw_f64_nexthop.restype = None
        L.oracle_fw_f32_nexthop.argtypes = [_f32p, _i32p, _i64]
        L.oracle_fw_f32_nexthop.restype = None
        L.oracle_fw_backward.argtypes = [_f64p, _i32p, _i64, _f64p]
        L.oracle_fw_backward.restype = _i64
        L.oracle_mt19937_outputs.argtypes = [ctypes.c_uint32, ctypes.c_uint64, _i64,
                                             np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")]
        L.oracle_mt19937_outputs.restype = None
        _lib = L
    return _lib


def generate_graph(n: int, density: float, seed: int, wmin: int = 0,
                   wmax: int = MAX_EDGE_WEIGHT) -> np.ndarray:
    out = np.empty((n, n), dtype=np.int32)
    rc = lib().oracle_generate_graph(out, n, float(density), seed, wmin, wmax)
    if rc:
        raise ValueError(f"bad generator arguments n={n} density={density}")
    return out


def fw_i32(D: np.ndarray) -> np.ndarray:
    """baseline_cpu (k-i-j sweep) on a copy of D."""
    out = np.ascontiguousarray(D, dtype=np.int32).copy()
    lib().oracle_fw_i32(out, out.shape[0])
    return out


def fw_i32_pivots(D: np.ndarray, k0: int, k1: int, threads: int = 1) -> None:
    """Pivots [k0, k1) of the sweep, in place."""
    assert D.dtype == np.int32 and D.flags.c_contiguous
    lib().oracle_fw_i32_pivots(D, D.shape[0], k0, k1, threads)


def mt19937_outputs(seed: int, skip: int, count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.uint32)
    lib().oracle_mt19937_outputs(seed, skip, count, out)
    return out


def has_negative_cycle(D: np.ndarray) -> bool:
    return bool(lib().oracle_has_negative_cycle(np.ascontiguousarray(D, dtype=np.int32), D.shape[0]))


def sssp_row(W: np.ndarray, src: int) -> np.ndarray:
    out = np.empty(W.shape[0], dtype=np.int32)
    lib().oracle_sssp_dense(np.ascontiguousarray(W, dtype=np.int32), W.shape[0], src, out)
    return out


def fw_f64_nexthop(W: np.ndarray):
    D = np.ascontiguousarray(W, dtype=np.float64).copy()
    nh = np.empty(D.shape, dtype=np.int32)
    lib().oracle_fw_f64_nexthop(D, nh, D.shape[0])
    return D, nh


def fw_f32_nexthop(W: np.ndarray):
    D = np.ascontiguousarray(W, dtype=np.float32).copy()
    nh = np.empty(D.shape, dtype=np.int32)
    lib().oracle_fw_f32_nexthop(D, nh, D.shape[0])
    return D, nh


def fw_backward(G: np.ndarray, nh: np.ndarray):
    """dL/dW (float64) and the number of walks that did not reach their end."""
    n = nh.shape[0]
    dW = np.empty((n, n), dtype=np.float64)
    bad = lib().oracle_fw_backward(np.ascontiguousarray(G, dtype=np.float64),
                                   np.ascontiguousarray(nh, dtype=np.int32), n, dW)
    return dW, int(bad)


# ---------------------------------------------------------------- reference CPU
def ref_available() -> bool:
    return os.path.exists(os.path.join(REFDIR, "libfwref.so"))


def ref():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(os.path.join(REFDIR, "libfwref.so"))
        R.ref_generate_graph.argtypes = [_i32p, ctypes.c_int, ctypes.c_double, ctypes.c_uint]
        R.ref_generate_graph.restype = ctypes.c_int
        R.ref_fw_baseline_cpu.argtypes = [_i32p, ctypes.c_int]
        R.ref_fw_baseline_cpu.restype = None
        R.ref_has_negative_cycle.argtypes = [_i32p, ctypes.c_int]
        R.ref_has_negative_cycle.restype = ctypes.c_int
        R.ref_run_tests_cpu.argtypes = []
        R.ref_run_tests_cpu.restype = None
        _ref = R
    return _ref


# ---------------------------------------------------------------- reference GPU
def refgpu_available() -> bool:
    return all(os.path.exists(os.path.join(REFDIR, f"ref_{k}.cubin"))
               for k in ("fw_baseline_gpu", "fw_tiling_gpu", "fw_multi_layer_tiling_gpu"))


def refgpu():
    """Load the reference kernels; raises if the cubins are missing."""
    global _refgpu
    if _refgpu is None:
        path = os.path.join(BUILD, "libfwrefgpu.so")
        if not os.path.exists(path):
            build()
        G = ctypes.CDLL(path)
        G.refgpu_load.argtypes = [ctypes.c_char_p]
        G.refgpu_load.restype = ctypes.c_int
        G.refgpu_last_error.restype = ctypes.c_char_p
        G.refgpu_baseline_gpu.argtypes = [ctypes.c_uint64, ctypes.c_int]
        G.refgpu_tiling_gpu.argtypes = [ctypes.c_uint64, ctypes.c_int]
        G.refgpu_multi_layer_tiling_gpu.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int]
        for f in (G.refgpu_baseline_gpu, G.refgpu_tiling_gpu, G.refgpu_multi_layer_tiling_gpu):
            f.restype = ctypes.c_int
        rc = G.refgpu_load(REFDIR.encode())
        if rc:
            raise RuntimeError("reference kernels: " + G.refgpu_last_error().decode())
        _refgpu = G
    return _refgpu


def refgpu_run(name: str, d_ptr: int, n: int, kappa: int = 0) -> None:
    G = refgpu()
    if name == "baseline_gpu":
        rc = G.refgpu_baseline_gpu(d_ptr, n)
    elif name == "tiling_gpu":
        rc = G.refgpu_tiling_gpu(d_ptr, n)
    elif name == "multi_layer_tiling_gpu":
        rc = G.refgpu_multi_layer_tiling_gpu(d_ptr, n, kappa)
    else:
        raise KeyError(name)
    if rc:
        raise RuntimeError(f"reference {name}: " + G.refgpu_last_error().decode())
