"""Builds libfw103.so (the CUDA engine + C ABI) and the C++ command-line tools
in place, for sm_103a only.

    python -m fw_cuda_gb300.build          # or fw_cuda_gb300.build.build()

Translation units compile in parallel; outputs land in fw_cuda_gb300/_lib/
(git-ignored). Nothing here needs a GPU: nvcc cross-compiles.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIBDIR = os.path.join(PKG, "_lib")
# Objects are kept per host architecture so that a tree copied between an x86
# and an Arm machine never links objects of the other one.
OBJDIR = os.path.join(LIBDIR, "obj-" + platform.machine())
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              f"-I{INCLUDE}", f"-I{CSRC}"]

CUDA_SOURCES = ["fw_apsp_i32.cu", "fw_capi.cu", "fw_peak.cu", "fw_noalloc.cu", "fw_batched.cu", "fw_diff.cu", "fw_packed16.cu", "fw_graph_io.cu", "fw_ooc.cu", "fw_gen.cu", "fw_stripe.cu"]
HOST_LIB_SOURCES = ["algorithms.cpp"]  # compiled into libfw103.so
TOOL_SOURCE = "runners.cpp"  # bench_runner / tests_runner (one binary, two names)
TOOLS = ("bench_runner", "tests_runner")
LIB_NAME = "libfw103.so"


def nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("build step failed: " + " ".join(cmd))


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def library_path() -> str:
    return os.path.join(LIBDIR, LIB_NAME)


def tool_path(name: str) -> str:
    return os.path.join(LIBDIR, name)


def build(verbose: bool = False) -> str:
    """Compile every CUDA translation unit and link libfw103.so; returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    heads = _headers()
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + heads):
            jobs.append([nvcc(), *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])
    for src in HOST_LIB_SOURCES:
        s = os.path.join(HOST, src)
        o = os.path.join(OBJDIR, src.replace(".cpp", ".o"))
        objs.append(o)
        if _stale(o, [s] + heads):
            jobs.append([nvcc(), *NVCC_FLAGS, "-c", s, "-o", o])
    tool_obj = os.path.join(OBJDIR, TOOL_SOURCE.replace(".cpp", ".o"))
    tsrc = os.path.join(HOST, TOOL_SOURCE)
    if _stale(tool_obj, [tsrc] + heads):
        jobs.append([nvcc(), *NVCC_FLAGS, "-c", tsrc, "-o", tool_obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    lib = library_path()
    if _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", lib, *objs])
    tool = os.path.join(LIBDIR, TOOLS[0])
    if _stale(tool, [tool_obj, lib]):
        _run([nvcc(), *ARCH, "-o", tool, tool_obj, f"-L{LIBDIR}", "-lfw103", "-Xlinker", "-rpath,$ORIGIN"])
    for alias in TOOLS[1:]:
        ap = os.path.join(LIBDIR, alias)
        if os.path.islink(ap) and os.readlink(ap) == TOOLS[0]:
            continue
        try:
            os.remove(ap)
        except FileNotFoundError:
            pass
        os.symlink(TOOLS[0], ap)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(verbose=True)
