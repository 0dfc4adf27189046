"""Differentiable fp32 Floyd-Warshall: forward (distances + next hops) against
the FP64 oracle sweep, backward against the oracle's path-walk gradient on the
same next hops and against central finite differences of the FP64 oracle."""
from __future__ import annotations

import numpy as np
import pytest

from fw_cuda_gb300 import workloads

pytestmark = pytest.mark.gpu

ULP_TOL = 8  # fp32 distances within 8 units in the last place of the FP64 sweep's


def ulp_distance(a32: np.ndarray, b64: np.ndarray) -> int:
    fin = np.isfinite(b64)
    assert np.array_equal(fin, np.isfinite(a32)), "reachability differs"
    a = a32[fin].astype(np.float32).view(np.int32).astype(np.int64)
    b = b64[fin].astype(np.float32).view(np.int32).astype(np.int64)
    return int(np.max(np.abs(a - b))) if a.size else 0


def walk_ok(W64, D64, nh):
    n = nh.shape[0]
    for i in range(n):
        for j in range(n):
            if i == j:
                assert nh[i, j] == i
                continue
            if not np.isfinite(D64[i, j]):
                assert nh[i, j] == -1
                continue
            u, tot, steps = i, 0.0, 0
            while u != j:
                v = int(nh[u, j])
                assert v >= 0 and steps < n, (i, j)
                tot += W64[u, v]
                u = v
                steps += 1
            assert abs(tot - D64[i, j]) <= 1e-5 * max(1.0, D64[i, j]), (i, j, tot, D64[i, j])


@pytest.mark.parametrize("n", [1, 5, 64, 130, 256, 300])
def test_forward_matches_fp64_sweep(cuda, oracle, n):
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(n)
    W = workloads.diff_graph(n, rng)
    D64, _ = oracle.fw_f64_nexthop(W.astype(np.float64))
    D, nh = A.forward_with_next_hops(cuda.from_numpy(W).cuda())
    D, nh = D.cpu().numpy(), nh.cpu().numpy()
    assert ulp_distance(D, D64) <= ULP_TOL
    walk_ok(W.astype(np.float64), D64, nh)


def test_backward_matches_path_walk_gradient(cuda, oracle):
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(11)
    n = 200
    W = workloads.diff_graph(n, rng)
    G = rng.standard_normal((n, n)).astype(np.float32)
    D, nh = A.forward_with_next_hops(cuda.from_numpy(W).cuda())
    dW, bad = A.backward_from_next_hops(cuda.from_numpy(G).cuda(), nh, check_walks=True)
    assert bad == 0
    ref, bad_cpu = oracle.fw_backward(G.astype(np.float64), nh.cpu().numpy())
    assert bad_cpu == 0
    got = dW.cpu().numpy().astype(np.float64)
    assert np.allclose(got, ref, rtol=1e-5, atol=1e-4)
    assert np.all(got[~np.isfinite(W)] == 0)


def test_gradient_matches_central_differences(cuda, oracle):
    """dL/dW of L = sum(G * D) against (L(W + eps) - L(W - eps)) / (2 eps), eps = 1e-3,
    in FP64 through the oracle sweep, on tie-free weights; 1e-3 relative."""
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(5)
    n = 24
    W = workloads.diff_graph(n, rng)
    G = rng.standard_normal((n, n))
    Wt = cuda.from_numpy(W).cuda().requires_grad_(True)
    D = A.shortest_paths(Wt)
    D.backward(cuda.from_numpy(G.astype(np.float32)).cuda())
    grad = Wt.grad.cpu().numpy().astype(np.float64)
    W64 = W.astype(np.float64)
    eps = 1e-3

    def loss(Wp):
        Dp, _ = oracle.fw_f64_nexthop(Wp)
        fin = np.isfinite(Dp)
        return float(np.sum(G[fin] * Dp[fin]))

    checked = 0
    for u in range(n):
        for v in range(n):
            if u == v or not np.isfinite(W64[u, v]):
                continue
            Wp, Wm = W64.copy(), W64.copy()
            Wp[u, v] += eps
            Wm[u, v] -= eps
            fd = (loss(Wp) - loss(Wm)) / (2 * eps)
            assert abs(fd - grad[u, v]) <= 1e-3 * max(1.0, abs(fd)), (u, v, fd, grad[u, v])
            checked += 1
    assert checked > 50


def test_batch_equals_single_graphs(cuda):
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(2)
    Ws = np.stack([workloads.diff_graph(256, rng) for _ in range(6)])
    Db, nhb = A.forward_with_next_hops(cuda.from_numpy(Ws).cuda())
    G = cuda.from_numpy(rng.standard_normal(Ws.shape).astype(np.float32)).cuda()
    dWb = A.backward_from_next_hops(G, nhb)
    for b in range(Ws.shape[0]):
        D1, nh1 = A.forward_with_next_hops(cuda.from_numpy(Ws[b]).cuda())
        assert cuda.equal(D1, Db[b]) and cuda.equal(nh1, nhb[b])
        dW1 = A.backward_from_next_hops(G[b].contiguous(), nh1)
        assert cuda.allclose(dW1, dWb[b], rtol=1e-5, atol=1e-5)


def test_gradient_matches_central_differences_n96(cuda, oracle):
    """The same check on a larger graph (n = 96), 400 sampled edges (300 on
    shortest paths), central differences in FP64 through the oracle sweep,
    1e-3 relative. With this many paths some pairs have an alternative path
    within eps of the shortest: the loss then has a kink inside [w - eps,
    w + eps] and no difference quotient is its derivative. Such edges are
    recognised by their one-sided differences disagreeing and left out (at
    most 5 % of the sample); every other edge must match."""
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(96)
    n = 96
    W = workloads.diff_graph(n, rng)
    G = rng.standard_normal((n, n))
    Wt = cuda.from_numpy(W).cuda().requires_grad_(True)
    A.shortest_paths(Wt).backward(cuda.from_numpy(G.astype(np.float32)).cuda())
    grad = Wt.grad.cpu().numpy().astype(np.float64)
    W64 = W.astype(np.float64)
    eps = 1e-3

    def loss(Wp):
        Dp, _ = oracle.fw_f64_nexthop(Wp)
        fin = np.isfinite(Dp)
        return float(np.sum(G[fin] * Dp[fin]))

    edges = [(u, v) for u in range(n) for v in range(n) if u != v and np.isfinite(W64[u, v])]
    on_paths = [e for e in edges if grad[e] != 0]
    off_paths = [e for e in edges if grad[e] == 0]
    assert len(on_paths) > 200
    pick = [on_paths[i] for i in rng.choice(len(on_paths), 300, replace=False)]
    pick += [off_paths[i] for i in rng.choice(len(off_paths), 100, replace=False)]
    l0 = loss(W64)
    kinks = 0
    for u, v in pick:
        Wp, Wm = W64.copy(), W64.copy()
        Wp[u, v] += eps
        Wm[u, v] -= eps
        lp, lm = loss(Wp), loss(Wm)
        fwd, bwd = (lp - l0) / eps, (l0 - lm) / eps
        if abs(fwd - bwd) > 1e-6 * max(1.0, abs(fwd)):
            kinks += 1  # a shortest path changes inside the window
            continue
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - grad[u, v]) <= 1e-3 * max(1.0, abs(fd)), (u, v, fd, grad[u, v])
    assert kinks <= 0.05 * len(pick), kinks


def test_batch_workload_against_fp64_sweep(cuda, oracle):
    """The differentiable workload's batch, 256 graphs at n = 256: every
    graph's distances within ULP_TOL of the FP64 sweep with the same k-order,
    and the batched backward equal to the oracle's path-walk gradient."""
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(5)  # the benchmark's batch
    Ws = np.stack([workloads.diff_graph(256, rng) for _ in range(256)])
    D, nh = A.forward_with_next_hops(cuda.from_numpy(Ws).cuda())
    G = np.random.default_rng(6).standard_normal(Ws.shape).astype(np.float32)
    dW, bad = A.backward_from_next_hops(cuda.from_numpy(G).cuda(), nh, check_walks=True)
    assert bad == 0
    D, nh, dW = D.cpu().numpy(), nh.cpu().numpy(), dW.cpu().numpy().astype(np.float64)
    for b in range(Ws.shape[0]):
        D64, _ = oracle.fw_f64_nexthop(Ws[b].astype(np.float64))
        assert ulp_distance(D[b], D64) <= ULP_TOL, b
        ref, bad_cpu = oracle.fw_backward(G[b].astype(np.float64), nh[b])
        assert bad_cpu == 0
        assert np.allclose(dW[b], ref, rtol=1e-5, atol=1e-4), b


def test_large_graph_rows_against_dijkstra(cuda):
    """n = 4096 (the differentiable workload's large graph): 64 sampled rows
    against FP64 Dijkstra, every walk ends, and the backward runs clean."""
    sp = pytest.importorskip("scipy.sparse.csgraph")
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(4096)
    n = 4096
    W = workloads.diff_graph(n, rng)
    D, nh = A.forward_with_next_hops(cuda.from_numpy(W).cuda())
    G = cuda.from_numpy(rng.standard_normal((n, n)).astype(np.float32)).cuda()
    dW, bad = A.backward_from_next_hops(G, nh, check_walks=True)
    assert bad == 0
    Dh = D.cpu().numpy()
    W64 = np.where(np.isfinite(W), W, 0.0).astype(np.float64)  # csgraph: 0 = no edge
    np.fill_diagonal(W64, 0.0)
    rows = sorted({0, 1, 2047, 4095, *[int(x) for x in rng.choice(n, 60, replace=False)]})
    assert len(rows) >= 64
    ref = sp.dijkstra(W64, directed=True, indices=rows)
    for q, i in enumerate(rows):
        ref_row = ref[q].copy()
        assert ulp_distance(Dh[i], ref_row) <= ULP_TOL


def test_autograd_function(cuda):
    from fw_cuda_gb300 import autograd as A

    rng = np.random.default_rng(9)
    W = cuda.from_numpy(workloads.diff_graph(100, rng)).cuda().requires_grad_(True)
    D = A.shortest_paths(W)
    G = cuda.randn_like(D)
    D.backward(G)
    _, nh = A.forward_with_next_hops(W.detach())
    assert cuda.allclose(W.grad, A.backward_from_next_hops(G, nh), rtol=1e-5, atol=1e-5)
