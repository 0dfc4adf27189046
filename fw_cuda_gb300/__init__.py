"""fw_cuda_gb300 — Python view of libfw103.so, the GB300 Floyd-Warshall engine.

The engine itself is CUDA + C++ behind the C ABI in include/fw103.h; this
module only loads that library with ctypes and mirrors the reference's
algorithm registry (src/cuda_utils.cu:7-23, include/algo_types.h:9) so that
Python callers and tests see the same names and argument meaning:

    fn = get_gpu_algorithm_func("multi_layer_tiling_gpu")
    fn(d_D, n, tile_size, kappa)     # d_D: int32 CUDA tensor (or device address), in place

There is no CPU fallback: if the library is missing, importing works but every
call raises FwLibraryMissing.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

INF = 1_000_000_000  # include/constants.h:3
MAX_N = 32769  # include/constants.h:5
MAX_EDGE_WEIGHT = 25_000  # include/constants.h:7

FW_OK = 0
FW_ERR_INVALID_ARGUMENT = 1
FW_ERR_CUDA = 2
FW_ERR_NO_MEMORY = 3
FW_ERR_TIMEOUT = 4
FW_ERR_NOT_BUILT = 5
FW_ERR_INTERNAL = 6

VARIANT_BASELINE = 0
VARIANT_TILING = 1
VARIANT_MULTI_LAYER = 2
VARIANT_AUTO = 3  # exact packed 16-bit sweep when provably identical, else the multi-layer int32 sweep

# Every symbol include/fw103.h declares (checked by the CPU tests).
EXPORTED_SYMBOLS = (
    "fw_apsp_i32",
    "fw_workspace_bytes_i32",
    "fw_apsp_i32_ws",
    "fw_generate_graph_i32",
    "fw_last_error_string",
    "fw_version",
    "fw_profile_begin",
    "fw_profile_end",
    "fw_measure_relax_peak",
    "fw_apsp_auto_report",
    "fw_measure_relax_peak_packed",
    "fw_apsp_paths_i32",
    "fw_path_length_i32",
    "fw_dense_from_csr_i32",
    "fw_negative_cycle_i32",
    "fw_apsp_i32_host",
    "fw_generate_graph_device_i32",
    "fw_mt19937_outputs",
    "fw_copy_faults",
    "fw_host_solve_device_bytes",
    "fw_batch_pack_offsets",
    "fw_batch_plan_create",
    "fw_batch_plan_autotune",
    "fw_apsp_batched_i32",
    "fw_batch_plan_describe",
    "fw_batch_plan_destroy",
    "fw_apsp_i32_noalloc",
    "fw_check_faults",
    "fw_debug_inject",
    "fw_debug_bounded_wait",
    "fw_measure_int32_rates",
    "fw_debug_flag_wait",
)

# Host-side fault injection kinds of fw_debug_inject (tests only).
INJECT_CALL_FAULT = 1
INJECT_PACKED_FAULT = 2


class FwError(RuntimeError):
    """A libfw103 call returned a nonzero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"fw103 status {status}: {msg}")
        self.status = status


class FwLibraryMissing(FwError):
    def __init__(self, path: str):
        super().__init__(FW_ERR_NOT_BUILT, f"{path} not found; run fw_cuda_gb300.build.build()")


class KernelStats(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int64), ("total_ms", ctypes.c_double),
                ("relaxations", ctypes.c_double)]


_lib = None


def library_path() -> str:
    return _build.library_path()


def lib():
    """The loaded libfw103.so (raises FwLibraryMissing if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise FwLibraryMissing(path)
    L = ctypes.CDLL(path)
    vp, i64, c_int = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    L.fw_apsp_i32.argtypes = [vp, i64, c_int, c_int, c_int, vp]
    L.fw_apsp_i32.restype = c_int
    L.fw_workspace_bytes_i32.argtypes = [i64, c_int, c_int, c_int]
    L.fw_workspace_bytes_i32.restype = ctypes.c_size_t
    L.fw_apsp_i32_ws.argtypes = [vp, i64, c_int, c_int, c_int, vp, ctypes.c_size_t, vp]
    L.fw_apsp_i32_ws.restype = c_int
    L.fw_generate_graph_i32.argtypes = [vp, i64, ctypes.c_double, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32]
    L.fw_generate_graph_i32.restype = c_int
    L.fw_last_error_string.argtypes = []
    L.fw_last_error_string.restype = ctypes.c_char_p
    L.fw_version.argtypes = []
    L.fw_version.restype = ctypes.c_char_p
    L.fw_profile_begin.argtypes = []
    L.fw_profile_begin.restype = c_int
    L.fw_profile_end.argtypes = [ctypes.POINTER(KernelStats), c_int, ctypes.POINTER(c_int)]
    L.fw_profile_end.restype = c_int
    L.fw_measure_relax_peak.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), vp]
    L.fw_measure_relax_peak.restype = c_int
    L.fw_apsp_paths_i32.argtypes = [vp, vp, i64, i64, vp]
    L.fw_apsp_paths_i32.restype = c_int
    L.fw_path_length_i32.argtypes = [vp, i64, i64, i64, vp, i64]
    L.fw_path_length_i32.restype = c_int
    L.fw_dense_from_csr_i32.argtypes = [vp, vp, vp, i64, vp, vp, vp]
    L.fw_dense_from_csr_i32.restype = c_int
    L.fw_negative_cycle_i32.argtypes = [vp, i64, i64, vp, vp]
    L.fw_negative_cycle_i32.restype = c_int
    L.fw_generate_graph_device_i32.argtypes = [vp, i64, ctypes.c_double, ctypes.c_uint32, ctypes.c_int32,
                                               ctypes.c_int32, vp]
    L.fw_generate_graph_device_i32.restype = c_int
    L.fw_mt19937_outputs.argtypes = [ctypes.c_uint32, ctypes.c_uint64, i64, vp]
    L.fw_mt19937_outputs.restype = c_int
    L.fw_copy_faults.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    L.fw_copy_faults.restype = c_int
    L.fw_apsp_i32_host.argtypes = [vp, i64, i64, i64, vp]
    L.fw_apsp_i32_host.restype = c_int
    L.fw_host_solve_device_bytes.argtypes = [i64, i64, i64]
    L.fw_host_solve_device_bytes.restype = ctypes.c_size_t
    L.fw_measure_relax_peak_packed.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), vp]
    L.fw_measure_relax_peak_packed.restype = c_int
    L.fw_apsp_auto_report.argtypes = [vp, ctypes.POINTER(c_int)]
    L.fw_apsp_auto_report.restype = c_int
    L.fw_batch_pack_offsets.argtypes = [vp, i64, vp, ctypes.POINTER(i64)]
    L.fw_batch_pack_offsets.restype = c_int
    L.fw_batch_plan_create.argtypes = [ctypes.POINTER(vp), vp, vp, i64]
    L.fw_batch_plan_create.restype = c_int
    L.fw_batch_plan_autotune.argtypes = [vp, vp, vp]
    L.fw_batch_plan_autotune.restype = c_int
    L.fw_apsp_batched_i32.argtypes = [vp, vp, vp]
    L.fw_apsp_batched_i32.restype = c_int
    L.fw_batch_plan_describe.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_double)]
    L.fw_batch_plan_describe.restype = c_int
    L.fw_batch_plan_destroy.argtypes = [vp]
    L.fw_batch_plan_destroy.restype = None
    L.fw_apsp_i32_noalloc.argtypes = [vp, i64, c_int, c_int, c_int, vp]
    L.fw_apsp_i32_noalloc.restype = c_int
    L.fw_check_faults.argtypes = [vp, ctypes.POINTER(ctypes.c_uint)]
    L.fw_check_faults.restype = c_int
    L.fw_debug_inject.argtypes = [c_int]
    L.fw_debug_inject.restype = c_int
    L.fw_debug_bounded_wait.argtypes = [c_int, vp]
    L.fw_debug_bounded_wait.restype = c_int
    L.fw_measure_int32_rates.argtypes = [ctypes.POINTER(ctypes.c_double), c_int, vp]
    L.fw_measure_int32_rates.restype = c_int
    L.fw_debug_flag_wait.argtypes = [i64, vp]
    L.fw_debug_flag_wait.restype = c_int
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != FW_OK:
        raise FwError(rc, lib().fw_last_error_string().decode())


def _ptr(x) -> int:
    """Device address of a torch CUDA tensor, or an int address as is."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("expected a CUDA tensor")
        if not x.is_contiguous():
            raise ValueError("expected a contiguous tensor")
        return x.data_ptr()
    raise TypeError(f"cannot take a device address of {type(x)!r}")


def _dev(x, count: int, dtypes: tuple[str, ...], what: str) -> int:
    """Device address of `x` after checking what the C-ABI call will touch: a
    contiguous CUDA tensor of one of `dtypes` (names such as "int32") with at
    least `count` elements. An int is a raw address and is passed unchecked."""
    if isinstance(x, int):
        return x
    p = _ptr(x)
    name = str(x.dtype).replace("torch.", "")
    if name not in dtypes:
        raise TypeError(f"{what}: expected dtype {' or '.join(dtypes)}, got {name}")
    if x.numel() < count:
        raise ValueError(f"{what}: needs at least {count} elements, got {x.numel()}")
    return p


def _sq(n: int, batch: int = 1) -> int:
    return max(int(n), 0) ** 2 * max(int(batch), 0)


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def apsp_i32(d_D, n: int, tile: int = 0, kappa: int = 0, variant: int = VARIANT_MULTI_LAYER, stream=None) -> None:
    """In-place APSP on the device (enqueued on `stream`; no synchronisation)."""
    _check(lib().fw_apsp_i32(_dev(d_D, _sq(n), ("int32",), "d_D"), n, tile, kappa, variant, _stream(stream)))


def auto_used_packed(stream=None) -> bool:
    """Whether the last VARIANT_AUTO call on `stream` used the packed path (synchronises)."""
    v = ctypes.c_int(0)
    _check(lib().fw_apsp_auto_report(_stream(stream), ctypes.byref(v)))
    return bool(v.value)


def workspace_bytes_i32(n: int, tile: int = 0, kappa: int = 0, variant: int = VARIANT_MULTI_LAYER) -> int:
    return int(lib().fw_workspace_bytes_i32(n, tile, kappa, variant))


def apsp_i32_ws(d_D, n: int, workspace, workspace_bytes: int, tile: int = 0, kappa: int = 0,
                variant: int = VARIANT_MULTI_LAYER, stream=None) -> None:
    if not isinstance(workspace, int) and workspace.numel() * workspace.element_size() < workspace_bytes:
        raise ValueError(f"workspace: holds {workspace.numel() * workspace.element_size()} bytes, "
                         f"workspace_bytes says {workspace_bytes}")
    _check(lib().fw_apsp_i32_ws(_dev(d_D, _sq(n), ("int32",), "d_D"), n, tile, kappa, variant, _ptr(workspace),
                                workspace_bytes, _stream(stream)))


def generate_graph(n: int, density: float, seed: int, wmin: int = 0, wmax: int = MAX_EDGE_WEIGHT,
                   out: np.ndarray | None = None) -> np.ndarray:
    """The reference's random digraph (src/graph_generator.cpp:7-46) with a weight range."""
    if out is None:
        out = np.empty((n, n), dtype=np.int32)
    assert out.dtype == np.int32 and out.flags.c_contiguous and out.size == n * n
    _check(lib().fw_generate_graph_i32(out.ctypes.data, n, float(density), seed, wmin, wmax))
    return out


def generate_graph_device(d_D, n: int, density: float, seed: int, wmin: int = 0, wmax: int = MAX_EDGE_WEIGHT,
                          stream=None) -> None:
    """generate_graph's matrix, value for value, generated on the device into d_D."""
    _check(lib().fw_generate_graph_device_i32(_dev(d_D, _sq(n), ("int32",), "d_D"), n, float(density), seed, wmin,
                                              wmax, _stream(stream)))


def mt19937_outputs(seed: int, skip: int, count: int) -> np.ndarray:
    """Host: `count` std::mt19937(seed) outputs after the first `skip`, by polynomial jump-ahead."""
    out = np.empty(count, dtype=np.uint32)
    _check(lib().fw_mt19937_outputs(seed, skip, count, out.ctypes.data))
    return out


def copy_faults() -> int:
    """Tile copies that missed their bounded wait since the library was loaded (0 when healthy)."""
    c = ctypes.c_uint(0)
    _check(lib().fw_copy_faults(ctypes.byref(c)))
    return int(c.value)


def check_faults(stream=None) -> None:
    """Synchronises `stream` and raises FwError(FW_ERR_TIMEOUT) when the last
    sweep call on it had a tile copy that missed its bounded wait (its result
    is then not valid)."""
    c = ctypes.c_uint(0)
    _check(lib().fw_check_faults(_stream(stream), ctypes.byref(c)))


def debug_inject(kinds: int) -> None:
    """Test hook: host-side fault injection for the next call on this thread
    (INJECT_CALL_FAULT, INJECT_PACKED_FAULT; 0 clears)."""
    _check(lib().fw_debug_inject(kinds))


def debug_bounded_wait(spins: int, stream=None) -> int:
    """Test hook: a bounded wait on a copy that is never issued; returns the
    status (FW_ERR_TIMEOUT when the wait gave up, as it should)."""
    return int(lib().fw_debug_bounded_wait(spins, _stream(stream)))


def debug_flag_wait(limit_us: int, stream=None) -> int:
    """Test hook: the stripe sweep's bounded flag wait on a flag nothing sets;
    returns the status (FW_ERR_TIMEOUT when the wait gave up, as it should)."""
    return int(lib().fw_debug_flag_wait(limit_us, _stream(stream)))


def version() -> str:
    return lib().fw_version().decode()


def profile_begin() -> None:
    _check(lib().fw_profile_begin())


def profile_end() -> dict:
    """{kernel name: {"launches", "total_ms", "relaxations"}} since profile_begin()."""
    cap = 16
    arr = (KernelStats * cap)()
    cnt = ctypes.c_int(0)
    _check(lib().fw_profile_end(arr, cap, ctypes.byref(cnt)))
    out = {}
    for i in range(min(cnt.value, cap)):
        s = arr[i]
        out[s.name.decode()] = {"launches": int(s.launches), "total_ms": float(s.total_ms),
                                "relaxations": float(s.relaxations)}
    return out


def measure_relax_peak(stream=None) -> tuple[float, float]:
    """(DPX-only, best mixed) relaxations/s of the register-only kernels."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    _check(lib().fw_measure_relax_peak(ctypes.byref(a), ctypes.byref(b), _stream(stream)))
    return a.value, b.value


INT32_RATE_NAMES = ("dpx_addmin", "imad", "dpx_min3", "add", "min", "dpx_addmin_imad_alternating",
                    "form_b_relax", "form_a_relax", "form_b_then_addmin_relax")


def measure_int32_rates(stream=None) -> dict:
    """Register-only int32 rates (fw_measure_int32_rates): lane operations/s of
    each instruction class and relaxations/s of each relaxation form."""
    r = (ctypes.c_double * len(INT32_RATE_NAMES))()
    _check(lib().fw_measure_int32_rates(r, len(INT32_RATE_NAMES), _stream(stream)))
    return dict(zip(INT32_RATE_NAMES, list(r)))


def measure_relax_peak_packed(stream=None) -> tuple[float, float]:
    """(DPX-only, best mixed) relaxations/s of the register-only packed 16-bit kernels."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    _check(lib().fw_measure_relax_peak_packed(ctypes.byref(a), ctypes.byref(b), _stream(stream)))
    return a.value, b.value


# ------------------------------------------------------ paths, graph I/O, checks
def apsp_paths_i32(d_D, d_nh, n: int, batch: int = 1, stream=None) -> None:
    """In-place int32 APSP that also writes next hops into d_nh (int32, same shape)."""
    _check(lib().fw_apsp_paths_i32(_dev(d_D, _sq(n, batch), ("int32",), "d_D"),
                                   _dev(d_nh, _sq(n, batch), ("int32",), "d_nh"), n, batch, _stream(stream)))


def path(nh: np.ndarray, i: int, j: int) -> list[int]:
    """Vertices of the recorded path i -> j ([] if unreachable), from a host next-hop matrix."""
    nh = np.ascontiguousarray(nh, dtype=np.int32)
    n = nh.shape[0]
    buf = np.empty(n + 1, dtype=np.int32)
    k = lib().fw_path_length_i32(nh.ctypes.data, n, i, j, buf.ctypes.data, n + 1)
    if k < 0:
        raise FwError(-k, lib().fw_last_error_string().decode())
    return buf[:k].tolist()


def dense_from_csr(d_rowptr, d_col, d_w, n: int, d_D, d_bad=None, stream=None) -> None:
    """Dense int32 matrix (INF / 0 diagonal / min of duplicates) from a device CSR graph."""
    _check(lib().fw_dense_from_csr_i32(_dev(d_rowptr, max(int(n), 0) + 1, ("int64",), "d_rowptr"),
                                       _dev(d_col, 0, ("int32",), "d_col") if d_col is not None else None,
                                       _dev(d_w, 0, ("int32",), "d_w") if d_w is not None else None, n,
                                       _dev(d_D, _sq(n), ("int32",), "d_D"),
                                       _dev(d_bad, 1, ("int32", "uint32"), "d_bad") if d_bad is not None else None,
                                       _stream(stream)))


def negative_cycle_flags(d_D, n: int, batch: int, d_flags, stream=None) -> None:
    """d_flags[b] = 1 if graph b has a negative diagonal entry (hasNegativeCycle)."""
    _check(lib().fw_negative_cycle_i32(_dev(d_D, _sq(n, batch), ("int32",), "d_D"), n, batch,
                                       _dev(d_flags, max(int(batch), 0), ("int32",), "d_flags"), _stream(stream)))


def apsp_i32_host(h_D, n: int, pass_width: int = 0, stripe_rows: int = 0, stream=None) -> None:
    """In-place APSP of an n x n int32 matrix held in HOST memory (a C-contiguous
    numpy array or CPU tensor), streamed through the device in row stripes;
    returns when h_D holds the result."""
    if hasattr(h_D, "data_ptr"):
        if h_D.is_cuda or not h_D.is_contiguous() or str(h_D.dtype) != "torch.int32":
            raise ValueError("expected a contiguous int32 CPU tensor")
        if h_D.numel() < _sq(n):
            raise ValueError(f"h_D: needs at least {_sq(n)} elements, got {h_D.numel()}")
        addr = h_D.data_ptr()
    elif isinstance(h_D, np.ndarray):
        if h_D.dtype != np.int32 or not h_D.flags.c_contiguous or not h_D.flags.writeable:
            raise ValueError("expected a writeable C-contiguous int32 array")
        if h_D.size < _sq(n):
            raise ValueError(f"h_D: needs at least {_sq(n)} elements, got {h_D.size}")
        addr = h_D.ctypes.data
    else:
        raise TypeError(f"cannot take a host address of {type(h_D)!r}")
    _check(lib().fw_apsp_i32_host(addr, n, pass_width, stripe_rows, _stream(stream)))


def host_solve_device_bytes(n: int, pass_width: int, stripe_rows: int) -> int:
    return int(lib().fw_host_solve_device_bytes(n, pass_width, stripe_rows))


# ----------------------------------------------------------------- batched APSP
def pack_offsets(sizes) -> tuple[np.ndarray, int]:
    """Element offsets of a dense packing (16-byte aligned starts) and its total size."""
    sizes = np.ascontiguousarray(sizes, dtype=np.int32)
    offs = np.empty(len(sizes), dtype=np.int64)
    total = ctypes.c_int64(0)
    _check(lib().fw_batch_pack_offsets(sizes.ctypes.data, len(sizes), offs.ctypes.data, ctypes.byref(total)))
    return offs, int(total.value)


class BatchPlan:
    """A planned batch of graphs (sizes + offsets into one packed int32 buffer)."""

    def __init__(self, sizes, offsets=None):
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int32)
        if offsets is None:
            offsets, self.total_elems = pack_offsets(self.sizes)
        else:
            offsets = np.ascontiguousarray(offsets, dtype=np.int64)
            self.total_elems = int(np.max(offsets + self.sizes.astype(np.int64) ** 2))
        self.offsets = offsets
        # elements the solves touch (the packing's total may add alignment padding)
        self.touched_elems = int(np.max(self.offsets + self.sizes.astype(np.int64) ** 2)) if len(self.sizes) else 0
        h = ctypes.c_void_p()
        _check(lib().fw_batch_plan_create(ctypes.byref(h), self.sizes.ctypes.data, self.offsets.ctypes.data,
                                          len(self.sizes)))
        self._h = h

    def autotune(self, d_packed, stream=None) -> str:
        _check(lib().fw_batch_plan_autotune(self._h, _dev(d_packed, self.touched_elems, ("int32",), "d_packed"),
                                            _stream(stream)))
        return self.describe()

    def solve(self, d_packed, stream=None) -> None:
        _check(lib().fw_apsp_batched_i32(self._h, _dev(d_packed, self.touched_elems, ("int32",), "d_packed"),
                                         _stream(stream)))

    def describe(self) -> str:
        buf = ctypes.create_string_buffer(512)
        _check(lib().fw_batch_plan_describe(self._h, buf, 512, None))
        return buf.value.decode()

    @property
    def relaxations(self) -> float:
        r = ctypes.c_double(0)
        _check(lib().fw_batch_plan_describe(self._h, None, 0, ctypes.byref(r)))
        return r.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().fw_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------- reference-style registry
def _synchronising(variant: int):
    """The reference's launcher contract in Python: enqueue on the legacy
    default stream, return after the device is synchronised, and fail (here:
    raise FwError) on any error, a missed tile copy included. The C++ shims
    with the same names (libfw103.so) print and exit instead, as the
    reference does."""
    def algo(d_D, n: int, tileSize: int = 0, kappa: int = 0) -> None:
        import torch

        apsp_i32(d_D, n, tileSize, kappa, variant, None)
        torch.cuda.synchronize()
        check_faults(None)

    return algo


fw_baseline_gpu = _synchronising(VARIANT_BASELINE)
fw_tiling_gpu = _synchronising(VARIANT_TILING)
fw_multi_layer_tiling_gpu = _synchronising(VARIANT_MULTI_LAYER)

# src/cuda_utils.cu:7-11
GPU_ALGORITHMS = {
    "baseline_gpu": fw_baseline_gpu,
    "tiling_gpu": fw_tiling_gpu,
    "multi_layer_tiling_gpu": fw_multi_layer_tiling_gpu,
}


def get_gpu_algorithm_func(name: str):
    """src/cuda_utils.cu:13-19 (std::out_of_range there, KeyError here)."""
    try:
        return GPU_ALGORITHMS[name]
    except KeyError:
        raise KeyError("ERROR: Unsupported GPU algorithm: " + name) from None


def is_gpu_algorithm(name: str) -> bool:
    """src/cuda_utils.cu:21-23."""
    return name in GPU_ALGORITHMS
