"""The 128-wide blocked sweep with its one-block look-ahead (block t + 1's
cross update, closure and panels on a high-priority stream beside block t's
bulk remainder), at sizes around and above the stripe sweep's range. Bit for
bit against the oracle's baseline_cpu sweep (src/fw_baseline_cpu.cpp:3-16),
or, at n = 6144 / 6145, against the oracle's Dijkstra rows and the schedule
without look-ahead on the same input."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 1_000_000_000
MULTI, TILING = 2, 1


def reference(oracle, W):
    out = np.ascontiguousarray(W, dtype=np.int32).copy()
    oracle.fw_i32_pivots(out, 0, out.shape[0], threads=os.cpu_count() or 1)
    return out


def lookahead_bytes(n: int) -> int:
    """The status block and two pairs of 128-row panels: the look-ahead schedule."""
    ldp = -(-n // 128) * 128
    return 256 + 2 * 2 * 128 * ldp * 4


def solve(fw, torch, W, variant=MULTI, kappa=4, workspace_bytes=None):
    n = W.shape[0]
    d = torch.from_numpy(np.ascontiguousarray(W, dtype=np.int32)).cuda()
    fw.profile_begin()
    if workspace_bytes is None:
        fw.apsp_i32(d, n, 32, kappa, variant, None)
    else:
        ws = torch.empty(workspace_bytes // 4 + 64, dtype=torch.int32, device="cuda")
        fw.apsp_i32_ws(d, n, ws, workspace_bytes, 32, kappa, variant)
    torch.cuda.synchronize()
    ran = fw.profile_end()
    fw.check_faults(None)
    return d.cpu().numpy(), ran


@pytest.mark.parametrize("n", [700, 1001, 1500, 2047])
def test_small_sizes_through_a_lookahead_workspace(fw, cuda, oracle, n):
    """Below n = 2048 a workspace of two panel buffers (less than the stripe
    sweep's) selects the look-ahead schedule."""
    W = oracle.generate_graph(n, 0.2, 60 + n, 0, 25000)
    nbytes = lookahead_bytes(n)
    assert nbytes < fw.workspace_bytes_i32(n, variant=MULTI)
    out, ran = solve(fw, cuda, W, MULTI, 4, nbytes)
    assert "fw_stripe" not in ran and "fw_diag" in ran
    assert np.array_equal(out, reference(oracle, W))


@pytest.mark.parametrize("n", [2049, 2500, 3001, 4097])
def test_sizes_above_the_stripe_sweep(fw, cuda, oracle, n):
    W = oracle.generate_graph(n, 0.5, 70 + n, 1, 100)
    ref = reference(oracle, W)
    for variant in (MULTI, TILING):
        out, ran = solve(fw, cuda, W, variant)
        assert "fw_stripe" not in ran
        assert np.array_equal(out, ref), (n, variant)


def test_negative_weights_and_sparse_input(fw, cuda, oracle):
    rng = np.random.default_rng(2500)
    n = 2500
    W = oracle.generate_graph(n, 0.3, 17, 0, 100)
    p = rng.integers(0, 60, n).astype(np.int64)
    Wn = np.where(W < INF, W.astype(np.int64) + p[:, None] - p[None, :], INF)
    np.fill_diagonal(Wn, 0)
    Wn = Wn.astype(np.int32)
    assert Wn.min() < 0
    out, _ = solve(fw, cuda, Wn)
    assert np.array_equal(out, reference(oracle, Wn))
    S = oracle.generate_graph(3000, 0.0005, 18, 0, 25000)  # many unreachable pairs
    ref = reference(oracle, S)
    assert np.count_nonzero(ref == INF) > 0
    out, _ = solve(fw, cuda, S)
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("n", [6144, 6145])
def test_larger_sizes_against_dijkstra(fw, cuda, oracle, n):
    """A full last pivot block and a one-column one: 16 rows against the
    oracle's Dijkstra rows, and the whole matrix against the schedule without
    look-ahead (the minimal workspace)."""
    W = oracle.generate_graph(n, 0.5, 80 + n, 1, 100)
    out, _ = solve(fw, cuda, W)
    minimum = 256 + 2 * 128 * (-(-n // 128) * 128) * 4
    single, _ = solve(fw, cuda, W, MULTI, 4, minimum)
    assert np.array_equal(out, single)
    rng = np.random.default_rng(n)
    for src in sorted({0, n - 1, *[int(x) for x in rng.choice(n, 14, replace=False)]}):
        assert np.array_equal(out[src], oracle.sssp_row(W, src)), src
