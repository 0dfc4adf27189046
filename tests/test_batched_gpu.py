"""Batched APSP (one persistent, graph-captured launch for many graphs) against
the oracle's baseline_cpu sweep of every graph, bit for bit."""
from __future__ import annotations

import os

import numpy as np
import pytest

from fw_cuda_gb300 import workloads

INF = 1_000_000_000


def _solve_all(fw, torch, sizes, offsets, packed, autotune=False):
    plan = fw.BatchPlan(sizes, offsets)
    d = torch.from_numpy(packed).cuda()
    if autotune:
        before = d.clone()
        plan.autotune(d)
        assert torch.equal(d, before), "autotune must leave the batch unchanged"
    plan.solve(d)
    torch.cuda.synchronize()
    return plan, d


def _check_all(oracle, sizes, offsets, packed_in, packed_out, which=None):
    for g in (range(len(sizes)) if which is None else which):
        n = int(sizes[g])
        a = packed_in[offsets[g]: offsets[g] + n * n].reshape(n, n)
        b = packed_out[offsets[g]: offsets[g] + n * n].reshape(n, n)
        assert np.array_equal(b, oracle.fw_i32(a)), f"graph {g} (n={n})"


@pytest.mark.gpu
@pytest.mark.parametrize("autotune", [False, True])
def test_every_bucket_every_boundary(fw, cuda, oracle, autotune):
    sizes = np.array([1, 2, 3, 15, 16, 17, 31, 32, 33, 63, 64, 65, 100, 127, 128, 129, 200, 255, 256, 257, 300, 383,
                      384, 385, 511, 512, 600] * 3, dtype=np.int32)
    rng = np.random.default_rng(7 + autotune)
    offsets, total = fw.pack_offsets(sizes)
    packed = np.full(total, -7, dtype=np.int32)  # padding between graphs must stay untouched
    for g, n in enumerate(sizes):
        W = oracle.generate_graph(int(n), float(rng.uniform(0.02, 1.0)), int(1000 + g), 0, 25000)
        packed[offsets[g]: offsets[g] + n * n] = W.ravel()
    plan, d = _solve_all(fw, cuda, sizes, offsets, packed, autotune)
    out = d.cpu().numpy()
    _check_all(oracle, sizes, offsets, packed, out)
    gaps = np.ones(total, dtype=bool)
    for g, n in enumerate(sizes):
        gaps[offsets[g]: offsets[g] + n * n] = False
    assert np.all(out[gaps] == -7)
    assert plan.relaxations == pytest.approx(float(np.sum(sizes.astype(np.float64) ** 3)))
    assert "graphs=81" in plan.describe()


@pytest.mark.gpu
def test_negative_weights_and_replay(fw, cuda, oracle):
    rng = np.random.default_rng(3)
    sizes = rng.integers(1, 300, 60).astype(np.int32)
    offsets, total = fw.pack_offsets(sizes)
    packed = np.zeros(total, dtype=np.int32)
    for g, n in enumerate(sizes):
        W = oracle.generate_graph(int(n), 0.3, 50 + g, 0, 100).astype(np.int64)
        p = rng.integers(0, 40, n)
        W = np.where(W < INF, W + p[:, None] - p[None, :], INF)
        np.fill_diagonal(W, 0)
        packed[offsets[g]: offsets[g] + n * n] = W.astype(np.int32).ravel()
    plan = fw.BatchPlan(sizes, offsets)
    d = cuda.from_numpy(packed).cuda()
    for rep in range(3):  # the captured launch is replayed on fresh copies of the input
        d.copy_(cuda.from_numpy(packed))
        plan.solve(d)
        cuda.cuda.synchronize()
        _check_all(oracle, sizes, offsets, packed, d.cpu().numpy())


@pytest.mark.gpu
def test_batched_workload_config(fw, cuda, oracle):
    """4096 graphs, n log-uniform in [16, 512] (the batched benchmark's
    workload): every graph against the oracle's sweep of that graph (the
    oracle runs graphs in parallel host threads), and a replay of the
    captured launch on a fresh copy gives the same bits."""
    from concurrent.futures import ThreadPoolExecutor

    sizes, offsets, packed = workloads.batched_graphs(fw)
    assert len(sizes) == 4096 and sizes.min() >= 16 and sizes.max() <= 512
    plan, d = _solve_all(fw, cuda, sizes, offsets, packed, autotune=True)
    out = d.cpu().numpy()

    def bad(g):
        n = int(sizes[g])
        a = packed[offsets[g]: offsets[g] + n * n].reshape(n, n)
        b = out[offsets[g]: offsets[g] + n * n].reshape(n, n)
        return None if np.array_equal(b, oracle.fw_i32(a)) else g

    order = sorted(range(len(sizes)), key=lambda g: -int(sizes[g]))  # largest first
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        wrong = [g for g in ex.map(bad, order) if g is not None]
    assert wrong == [], f"{len(wrong)} graphs differ from the oracle, e.g. {wrong[:5]}"
    d.copy_(cuda.from_numpy(packed))
    plan.solve(d)
    cuda.cuda.synchronize()
    assert np.array_equal(d.cpu().numpy(), out)


def test_plan_rejects_bad_batches(fw):
    import ctypes

    L = fw.lib()
    h = ctypes.c_void_p()
    sizes = np.array([4, 0, 5], dtype=np.int32)
    offs = np.array([0, 16, 32], dtype=np.int64)
    assert L.fw_batch_plan_create(ctypes.byref(h), sizes.ctypes.data, offs.ctypes.data, 3) == fw.FW_ERR_INVALID_ARGUMENT
    sizes = np.array([4, 4097], dtype=np.int32)
    offs = np.array([0, 16], dtype=np.int64)
    assert L.fw_batch_plan_create(ctypes.byref(h), sizes.ctypes.data, offs.ctypes.data, 2) == fw.FW_ERR_INVALID_ARGUMENT
    sizes = np.array([4, 4], dtype=np.int32)
    offs = np.array([0, 8], dtype=np.int64)  # overlapping
    assert L.fw_batch_plan_create(ctypes.byref(h), sizes.ctypes.data, offs.ctypes.data, 2) == fw.FW_ERR_INVALID_ARGUMENT
    assert b"overlap" in L.fw_last_error_string()
    offs = np.array([0, -4], dtype=np.int64)
    assert L.fw_batch_plan_create(ctypes.byref(h), sizes.ctypes.data, offs.ctypes.data, 2) == fw.FW_ERR_INVALID_ARGUMENT


def test_pack_offsets(fw):
    offs, total = fw.pack_offsets(np.array([1, 3, 2, 5], dtype=np.int32))
    assert offs.tolist() == [0, 4, 16, 20] and total == 48  # starts on 16-byte boundaries


def test_batched_workload_parameters():
    sizes, dens, seeds = workloads.batched_params()
    assert len(sizes) == 4096 and sizes.min() >= 16 and sizes.max() <= 512
    assert 0.05 <= dens.min() and dens.max() <= 1.0 and seeds.min() >= 1
    # log-uniform: the median size is near sqrt(16 * 512) = 90.5
    assert 80 <= np.median(sizes) <= 100
    s2, d2, e2 = workloads.batched_params()
    assert np.array_equal(sizes, s2) and np.array_equal(seeds, e2)


@pytest.mark.gpu
@pytest.mark.parametrize("autotune", [False, True])
def test_packed_large_graphs_and_their_fallbacks(fw, cuda, oracle, autotune):
    """Graphs with 128 < n <= 1024 take the exact packed 16-bit path unless an
    entry is outside [0, 32767) u {INF} (a negative or a too large weight) or
    a distance comes too close to the 16-bit cap for the proof (a long chain
    of heavy edges); those graphs, and graphs with n > 1024, are solved by the
    int32 path. Every graph against the oracle."""
    rng = np.random.default_rng(11)
    graphs = []
    graphs.append(oracle.generate_graph(200, 0.6, 1, 1, 100))          # packed
    W = oracle.generate_graph(300, 0.3, 2, 1, 100).astype(np.int64)    # a negative edge, no negative cycle
    p = rng.integers(0, 60, 300)
    W = np.where(W < INF, W + p[:, None] - p[None, :], INF)
    np.fill_diagonal(W, 0)
    graphs.append(W.astype(np.int32))
    W = oracle.generate_graph(257, 0.5, 3, 1, 100)                      # one weight >= 32767
    W[5, 7] = 40000
    graphs.append(W)
    chain = np.full((400, 400), INF, dtype=np.int32)                    # distances past the cap
    np.fill_diagonal(chain, 0)
    chain[np.arange(399), np.arange(1, 400)] = 1000
    graphs.append(chain)
    graphs.append(oracle.generate_graph(129, 0.9, 4, 1, 100))          # packed
    graphs.append(oracle.generate_graph(1024, 0.3, 5, 1, 100))         # packed, the largest it takes
    graphs.append(oracle.generate_graph(1025, 0.3, 6, 1, 100))         # int32 (n > 1024)
    graphs.append(oracle.generate_graph(700, 0.05, 7, 0, 25000))       # either, by the proof
    sizes = np.array([g.shape[0] for g in graphs], dtype=np.int32)
    offsets, total = fw.pack_offsets(sizes)
    packed = np.full(total, -7, dtype=np.int32)
    for g, W in enumerate(graphs):
        packed[offsets[g]: offsets[g] + W.size] = W.ravel()
    plan, d = _solve_all(fw, cuda, sizes, offsets, packed, autotune)
    out = d.cpu().numpy()
    _check_all(oracle, sizes, offsets, packed, out)
    assert "n>128:8" in plan.describe()
    for rep in range(2):  # replays on fresh copies (the hand-back list is rebuilt every launch)
        d.copy_(cuda.from_numpy(packed))
        plan.solve(d)
        cuda.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), out)
