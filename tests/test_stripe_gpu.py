"""The stripe sweep: tiling_gpu / multi_layer_tiling_gpu for n <= 2048 as one
cooperative launch (8-wide pivot blocks handed from CTA to CTA through flags).

Every case is bit for bit against the oracle's baseline_cpu sweep
(src/fw_baseline_cpu.cpp:3-16), and against the 128-wide blocked sweep that a
caller workspace of the blocked minimum selects; the kernel-class profile
shows which of the two ran."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 1_000_000_000
TILING, MULTI = 1, 2

SIZES = (list(range(1, 34)) + [39, 40, 41, 63, 64, 65, 100, 127, 128, 129, 255, 256, 257, 300, 511, 512, 513,
                               777, 1000, 1023, 1024, 1025, 1215, 1216, 1217, 1218, 1500, 1999, 2046, 2047, 2048])


def reference(oracle, W: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(W, dtype=np.int32).copy()
    oracle.fw_i32_pivots(out, 0, out.shape[0], threads=os.cpu_count() or 1)
    return out


def solve(fw, torch, W, variant, kappa=4, workspace_bytes=None):
    """One solve; returns (result, kernel classes that ran)."""
    n = W.shape[0]
    d = torch.from_numpy(np.ascontiguousarray(W, dtype=np.int32)).cuda()
    fw.profile_begin()
    if workspace_bytes is None:
        fw.apsp_i32(d, n, 32, kappa, variant, None)
    else:
        ws = torch.empty(workspace_bytes // 4 + 64, dtype=torch.int32, device="cuda")
        fw.apsp_i32_ws(d, n, ws, workspace_bytes, 32, kappa, variant)
    torch.cuda.synchronize()
    prof = fw.profile_end()
    fw.check_faults(None)
    return d.cpu().numpy(), set(prof)


@pytest.mark.parametrize("n", SIZES)
def test_matches_oracle(fw, cuda, oracle, n):
    rng = np.random.default_rng(n)
    dens = float(rng.choice([0.01, 0.1, 0.5, 0.95]))
    W = oracle.generate_graph(n, dens, 900 + n, 0, 25000)
    ref = reference(oracle, W)
    for variant, kappa in ((TILING, 0), (MULTI, 1), (MULTI, 4), (MULTI, 8)):
        out, ran = solve(fw, cuda, W, variant, kappa)
        assert "fw_stripe" in ran and "fw_remainder" not in ran, (n, variant, kappa, ran)
        assert np.array_equal(out, ref), (n, variant, kappa, int(np.count_nonzero(out != ref)))


@pytest.mark.parametrize("n", [1, 2, 8, 31, 127, 128, 129, 255, 257, 300, 513, 777, 1000, 1023, 1217, 2047, 2048])
def test_equals_blocked_sweep(fw, cuda, oracle, n):
    """The blocked minimum of workspace keeps the 128-wide blocked sweep; both
    schedules give the same matrix."""
    W = oracle.generate_graph(n, 0.3, 31 + n, 1, 100)
    full = fw.workspace_bytes_i32(n, variant=MULTI)
    minimum = 256 + 2 * 128 * (-(-n // 128) * 128) * 4
    a, ran_a = solve(fw, cuda, W, MULTI, 4, full)
    b, ran_b = solve(fw, cuda, W, MULTI, 4, minimum)
    assert "fw_stripe" in ran_a
    assert "fw_stripe" not in ran_b and "fw_diag" in ran_b
    assert np.array_equal(a, b)
    assert np.array_equal(a, reference(oracle, W))


def potential_shift(W: np.ndarray, rng) -> np.ndarray:
    """Negative edge weights without negative cycles: w'(u,v) = w(u,v) + p(u) - p(v)."""
    p = rng.integers(0, 60, W.shape[0]).astype(np.int64)
    out = np.where(W < INF, W.astype(np.int64) + p[:, None] - p[None, :], INF)
    np.fill_diagonal(out, 0)
    return out.astype(np.int32)


@pytest.mark.parametrize("n", [9, 136, 700, 1300, 2048])
def test_negative_weights_and_positive_diagonal(fw, cuda, oracle, n):
    rng = np.random.default_rng(5000 + n)
    W = potential_shift(oracle.generate_graph(n, 0.4, 11 + n, 0, 100), rng)
    assert W.min() < 0
    out, ran = solve(fw, cuda, W, MULTI)
    assert "fw_stripe" in ran
    assert np.array_equal(out, reference(oracle, W))
    # a positive diagonal (self-loops of positive weight): the sweep keeps
    # min(loop, shortest cycle through the vertex)
    W2 = oracle.generate_graph(n, 0.05, 12 + n, 1, 100)
    np.fill_diagonal(W2, rng.integers(1, 300, n).astype(np.int32))
    out2, _ = solve(fw, cuda, W2, TILING)
    assert np.array_equal(out2, reference(oracle, W2))


def test_unreachable_blocks_stay_inf(fw, cuda, oracle):
    n = 1500
    W = oracle.generate_graph(n, 0.02, 77, 0, 25000)
    W[: n // 2, n // 2:] = INF  # nothing from the first half reaches the second
    np.fill_diagonal(W, 0)
    ref = reference(oracle, W)
    assert np.count_nonzero(ref == INF) >= (n // 2) * (n - n // 2)
    out, ran = solve(fw, cuda, W, MULTI)
    assert "fw_stripe" in ran
    assert np.array_equal(out, ref)


def test_streams_and_repeats(fw, cuda, oracle):
    """Solves on two streams at once (each with its library workspace and its
    own flags), then repeated calls of different sizes on one stream."""
    Ws = [oracle.generate_graph(n, 0.4, 3 + n, 1, 100) for n in (1024, 1999)]
    refs = [reference(oracle, W) for W in Ws]
    streams = [cuda.cuda.Stream() for _ in Ws]
    ds = []
    for W, s in zip(Ws, streams):
        with cuda.cuda.stream(s):
            ds.append(cuda.from_numpy(W).cuda())
    for d, W, s in zip(ds, Ws, streams):
        fw.apsp_i32(d, W.shape[0], 32, 4, MULTI, s)
    for d, ref, s in zip(ds, refs, streams):
        s.synchronize()
        assert np.array_equal(d.cpu().numpy(), ref)
        fw.check_faults(s)
    for _ in range(2):
        for W, ref in zip(Ws, refs):
            out, _ = solve(fw, cuda, W, TILING)
            assert np.array_equal(out, ref)


def test_bounded_flag_wait_gives_up_and_context_survives(fw, cuda, oracle):
    """The stripe sweep's flag wait on a flag that nothing sets runs out after
    its limit and reports FW_ERR_TIMEOUT; a solve right after is correct."""
    assert fw.debug_flag_wait(2000, None) == fw.FW_ERR_TIMEOUT
    W = oracle.generate_graph(600, 0.3, 8, 1, 100)
    out, ran = solve(fw, cuda, W, MULTI)
    assert "fw_stripe" in ran
    assert np.array_equal(out, reference(oracle, W))
