"""Path reconstruction (int32 next hops), the CSR front-end and the device
negative-cycle flags, against the oracle."""
from __future__ import annotations

import numpy as np
import pytest

INF = 1_000_000_000


def walk_all(W: np.ndarray, D: np.ndarray, nh: np.ndarray) -> None:
    """Every recorded path i -> j has the length D[i][j] (vectorised walk)."""
    n = W.shape[0]
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    reach = D < INF
    assert np.all(nh[~reach] == -1)
    assert np.all(np.diag(nh) == np.arange(n))
    u = ii.copy()
    tot = np.zeros((n, n), dtype=np.int64)
    active = reach & (ii != jj)
    for _ in range(n + 1):
        if not active.any():
            break
        v = nh[u, jj]
        assert np.all(v[active] >= 0)
        tot[active] += W[u[active], v[active]]
        u = np.where(active, v, u)
        active = active & (u != jj)
    assert not active.any(), "a recorded path does not end"
    off = reach & (ii != jj)
    assert np.array_equal(tot[off], D[off].astype(np.int64))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 7, 130, 300, 1000])
def test_int_paths(fw, cuda, oracle, n):
    # positive weights: every cycle is positive, so recorded paths must end
    W = oracle.generate_graph(n, 0.1 if n > 100 else 0.4, 10 + n, 1, 100)
    d = cuda.from_numpy(W).cuda()
    nh = cuda.empty_like(d)
    fw.apsp_paths_i32(d, nh, n)
    cuda.cuda.synchronize()
    D = d.cpu().numpy()
    assert np.array_equal(D, oracle.fw_i32(W))
    walk_all(W, D, nh.cpu().numpy())


@pytest.mark.gpu
def test_int_paths_batch_and_negative_weights(fw, cuda, oracle):
    rng = np.random.default_rng(1)
    n, B = 200, 5
    Ws = []
    for b in range(B):
        # a potential shift keeps every cycle's (positive) weight: negative edges, no zero cycles
        W = oracle.generate_graph(n, 0.2, 300 + b, 1, 50).astype(np.int64)
        p = rng.integers(0, 30, n)
        W = np.where(W < INF, W + p[:, None] - p[None, :], INF)
        np.fill_diagonal(W, 0)
        Ws.append(W.astype(np.int32))
    Wb = np.stack(Ws)
    d = cuda.from_numpy(Wb).cuda()
    nh = cuda.empty_like(d)
    fw.apsp_paths_i32(d, nh, n, B)
    cuda.cuda.synchronize()
    for b in range(B):
        D = d[b].cpu().numpy()
        assert np.array_equal(D, oracle.fw_i32(Ws[b]))
        walk_all(Ws[b], D, nh[b].cpu().numpy())


@pytest.mark.gpu
def test_zero_weight_cycles_keep_exact_distances(fw, cuda, oracle):
    """Zero-weight cycles: distances stay exact (next hops are only promised for positive cycles)."""
    n = 300
    W = oracle.generate_graph(n, 0.3, 17, 0, 3)  # many zero-weight edges and cycles
    d = cuda.from_numpy(W).cuda()
    nh = cuda.empty_like(d)
    fw.apsp_paths_i32(d, nh, n)
    assert np.array_equal(d.cpu().numpy(), oracle.fw_i32(W))


@pytest.mark.gpu
def test_known_path(fw, cuda):
    W = np.array([[0, 1, INF, 100], [INF, 0, 1, INF], [INF, INF, 0, 1], [INF, INF, INF, 0]], dtype=np.int32)
    d = cuda.from_numpy(W).cuda()
    nh = cuda.empty_like(d)
    fw.apsp_paths_i32(d, nh, 4)
    h = nh.cpu().numpy()
    assert fw.path(h, 0, 3) == [0, 1, 2, 3]
    assert fw.path(h, 3, 0) == []
    assert fw.path(h, 2, 2) == [2]


@pytest.mark.gpu
def test_dense_from_csr(fw, cuda):
    rng = np.random.default_rng(3)
    n, m = 500, 20000
    src = rng.integers(0, n, m)
    dst = rng.integers(0, n, m)
    w = rng.integers(-3, 100, m).astype(np.int32)
    w[::97] = INF  # skipped: weight >= INF
    dst[::101] = n + 5  # skipped: column out of range
    order = np.argsort(src, kind="stable")
    src, dst, w = src[order], dst[order], w[order]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rowptr, src + 1, 1)
    rowptr = np.cumsum(rowptr)
    expect = np.full((n, n), INF, dtype=np.int64)
    np.fill_diagonal(expect, 0)
    ok = (dst < n) & (w < INF)
    np.minimum.at(expect, (src[ok], dst[ok]), w[ok])
    D = cuda.empty((n, n), dtype=cuda.int32, device="cuda")
    bad = cuda.zeros(1, dtype=cuda.int32, device="cuda")
    fw.dense_from_csr(cuda.from_numpy(rowptr).cuda(), cuda.from_numpy(dst.astype(np.int32)).cuda(),
                      cuda.from_numpy(w).cuda(), n, D, bad)
    cuda.cuda.synchronize()
    assert np.array_equal(D.cpu().numpy(), expect.astype(np.int32))
    assert int(bad.item()) == int((~ok).sum())


@pytest.mark.gpu
def test_negative_cycle_flags(fw, cuda, oracle):
    n, B = 64, 6
    Ws = []
    for b in range(B):
        W = oracle.generate_graph(n, 0.1, 70 + b, 5, 50)
        if b % 2:
            W[n - 3, n - 2] = W[n - 2, n - 1] = W[n - 1, n - 3] = -40
        Ws.append(W)
    d = cuda.from_numpy(np.stack(Ws)).cuda()
    for b in range(B):
        fw.apsp_i32(d[b], n, 32, 4, 2, None)
    flags = cuda.full((B,), -1, dtype=cuda.int32, device="cuda")
    fw.negative_cycle_flags(d, n, B, flags)
    got = flags.cpu().numpy().tolist()
    assert got == [int(oracle.has_negative_cycle(oracle.fw_i32(W))) for W in Ws] == [0, 1, 0, 1, 0, 1]


def test_path_helper_on_host(fw):
    nh = np.array([[0, 1, 1], [-1, 1, 2], [-1, -1, 2]], dtype=np.int32)
    assert fw.path(nh, 0, 2) == [0, 1, 2]
    assert fw.path(nh, 2, 0) == []
    bad = np.array([[0, 1], [0, 1]], dtype=np.int32)
    bad[0, 1] = 0  # 0 -> 0 -> ... never reaches 1
    with pytest.raises(fw.FwError):
        fw.path(bad, 0, 1)
