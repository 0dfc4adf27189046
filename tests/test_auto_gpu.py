"""FW_VARIANT_AUTO: for n <= 2048 the int32 stripe sweep (faster there than
the packed path); above that the exact packed 16-bit sweep, used only when its
result is provably the int32 result. Every case here must equal the oracle
bit for bit, and the path taken must be the one the rule predicts."""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 1_000_000_000
AUTO = 3


def reference(oracle, W):
    out = np.ascontiguousarray(W, dtype=np.int32).copy()
    oracle.fw_i32_pivots(out, 0, out.shape[0], threads=os.cpu_count() or 1)
    return out


def run_auto(fw, torch, W, kappa=4):
    n = W.shape[0]
    d = torch.from_numpy(np.ascontiguousarray(W, dtype=np.int32)).cuda()
    fw.apsp_i32(d, n, 32, kappa, AUTO, None)
    used = fw.auto_used_packed(None)
    return d.cpu().numpy(), used


@pytest.mark.parametrize("n", [2049, 2100, 2303, 2304, 2305, 2560, 3000])
def test_small_weights_take_the_packed_path(fw, cuda, oracle, n):
    W = oracle.generate_graph(n, 0.5, 77 + n, 1, 100)
    out, used = run_auto(fw, cuda, W)
    assert np.array_equal(out, reference(oracle, W))
    assert used


@pytest.mark.parametrize("n", [1, 2, 255, 513, 1000, 2048])
def test_up_to_2048_the_stripe_sweep_runs(fw, cuda, oracle, n):
    W = oracle.generate_graph(n, 0.5, 77 + n, 1, 100)
    fw.profile_begin()
    out, used = run_auto(fw, cuda, W)
    ran = fw.profile_end()
    assert np.array_equal(out, reference(oracle, W))
    assert not used
    assert "fw_stripe" in ran and "fw_p16_remainder" not in ran and "fw_p16_diag" not in ran


def test_unreachable_pairs_decode_to_inf(fw, cuda, oracle):
    n = 2200
    W = oracle.generate_graph(n, 0.02, 5, 0, 100)  # sparse: many unreachable pairs, zero weights too
    W[: n // 2, n // 2:] = INF  # no edge from the first half to the second
    np.fill_diagonal(W, 0)
    ref = reference(oracle, W)
    assert np.count_nonzero(ref == INF) > 0
    out, used = run_auto(fw, cuda, W)
    assert np.array_equal(out, ref)
    assert used


def test_reference_weight_range(fw, cuda, oracle):
    W = oracle.generate_graph(2200, 0.9, 42, 0, 25000)
    out, _ = run_auto(fw, cuda, W)
    assert np.array_equal(out, reference(oracle, W))


@pytest.mark.parametrize("case", ["negative", "too_large", "long_paths"])
def test_ineligible_inputs_fall_back_exactly(fw, cuda, oracle, case):
    n = 2100
    W = oracle.generate_graph(n, 0.3, 9, 1, 100)
    if case == "negative":
        # every way back from 7 to 3 weighs at least 2, so no cycle is negative
        W[3, 7] = -1
        W[7, 3] = 10
    elif case == "too_large":
        W[1, 2] = 40000  # finite but above the 16-bit range
    else:  # a chain whose distances pass the 16-bit cap
        W = np.full((n, n), INF, dtype=np.int32)
        np.fill_diagonal(W, 0)
        for i in range(n - 1):
            W[i, i + 1] = 20000
    out, used = run_auto(fw, cuda, W)
    assert np.array_equal(out, reference(oracle, W))
    assert not used


def test_kappa_8_fallback_and_repeat(fw, cuda, oracle):
    W = oracle.generate_graph(2200, 0.3, 3, 1, 100)
    W[0, 1] = -1
    ref = reference(oracle, W)
    for _ in range(2):
        out, used = run_auto(fw, cuda, W, kappa=8)
        assert np.array_equal(out, ref) and not used
    W2 = oracle.generate_graph(2200, 0.3, 4, 1, 100)
    out, used = run_auto(fw, cuda, W2, kappa=8)
    assert np.array_equal(out, reference(oracle, W2)) and used
