"""Synthetic workloads of the benchmark configurations (there is no dataset).

* ``batched_graphs`` — 4096 independent directed graphs, n log-uniform in
  [16, 512], density uniform in [0.05, 1.0], integer weights uniform in
  [1, 100], INF for non-edges, master seed 1234. Per-graph parameters come
  from numpy's PCG64 stream seeded with the master seed, in this order per
  graph: n = round(exp(U(ln 16, ln 512))), density = U(0.05, 1.0), a 32-bit
  generator seed in [1, 2^32 - 1]; each graph is then drawn by the
  reference's generator (src/graph_generator.cpp:7-46, here
  fw_generate_graph_i32) with that seed and the [1, 100] weight range.
* ``diff_graphs`` — fp32 weights uniform in (0.5, 10.0) at density 0.3 for the
  differentiable form, with exact duplicate weights in a graph resampled
  (tie-free), +inf for non-edges and 0 on the diagonal; upstream gradients
  dL/dD ~ N(0, 1).
"""
from __future__ import annotations

import math

import numpy as np


def batched_params(count: int = 4096, seed: int = 1234, nmin: int = 16, nmax: int = 512):
    rng = np.random.default_rng(seed)
    sizes = np.empty(count, dtype=np.int32)
    dens = np.empty(count, dtype=np.float64)
    seeds = np.empty(count, dtype=np.uint32)
    lo, hi = math.log(nmin), math.log(nmax)
    for g in range(count):
        sizes[g] = int(round(math.exp(rng.uniform(lo, hi))))
        dens[g] = rng.uniform(0.05, 1.0)
        seeds[g] = rng.integers(1, 2**32 - 1, dtype=np.uint64)
    return sizes, dens, seeds


def batched_graphs(fw, count: int = 4096, seed: int = 1234, wmin: int = 1, wmax: int = 100, nmin: int = 16,
                   nmax: int = 512):
    """(sizes, offsets, packed int32 host buffer) of the batched workload."""
    sizes, dens, seeds = batched_params(count, seed, nmin, nmax)
    offsets, total = fw.pack_offsets(sizes)
    packed = np.full(total, fw.INF, dtype=np.int32)
    for g in range(count):
        n = int(sizes[g])
        view = packed[offsets[g]: offsets[g] + n * n]
        fw.generate_graph(n, float(dens[g]), int(seeds[g]), wmin, wmax, out=view.reshape(n, n))
    return sizes, offsets, packed


def diff_graph(n: int, rng, density: float = 0.3, lo: float = 0.5, hi: float = 10.0) -> np.ndarray:
    """One tie-free fp32 weight matrix (+inf = no edge, 0 on the diagonal)."""
    mask = rng.random((n, n)) < density
    w = rng.uniform(lo, hi, (n, n)).astype(np.float32)
    while True:  # resample exact duplicates among the present edges
        vals = w[mask]
        _, first, counts = np.unique(vals, return_index=True, return_counts=True)
        if np.all(counts == 1):
            break
        dup = np.ones(vals.shape, dtype=bool)
        dup[first] = False
        vals[dup] = rng.uniform(lo, hi, int(dup.sum())).astype(np.float32)
        w[mask] = vals
    W = np.where(mask, w, np.float32(np.inf)).astype(np.float32)
    np.fill_diagonal(W, 0.0)
    return W
