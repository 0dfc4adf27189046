"""FW_VARIANT_AUTO: the exact packed 16-bit sweep is used only when its result
is provably the int32 result; every case here must equal the oracle bit for
bit, and the path taken must be the one the eligibility rule predicts."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INF = 1_000_000_000
AUTO = 3


def run_auto(fw, torch, W, kappa=4):
    n = W.shape[0]
    d = torch.from_numpy(np.ascontiguousarray(W, dtype=np.int32)).cuda()
    fw.apsp_i32(d, n, 32, kappa, AUTO, None)
    used = fw.auto_used_packed(None)
    return d.cpu().numpy(), used


@pytest.mark.parametrize("n", [1, 2, 255, 256, 257, 511, 513, 1000, 1536])
def test_small_weights_take_the_packed_path(fw, cuda, oracle, n):
    W = oracle.generate_graph(n, 0.5, 77 + n, 1, 100)
    out, used = run_auto(fw, cuda, W)
    assert np.array_equal(out, oracle.fw_i32(W))
    assert used


def test_unreachable_pairs_decode_to_inf(fw, cuda, oracle):
    n = 600
    W = oracle.generate_graph(n, 0.02, 5, 0, 100)  # sparse: many unreachable pairs, zero weights too
    W[:300, 300:] = INF  # no edge from the first half to the second
    np.fill_diagonal(W, 0)
    ref = oracle.fw_i32(W)
    assert np.count_nonzero(ref == INF) > 0
    out, used = run_auto(fw, cuda, W)
    assert np.array_equal(out, ref)
    assert used


def test_reference_weight_range(fw, cuda, oracle):
    W = oracle.generate_graph(700, 0.9, 42, 0, 25000)
    out, _ = run_auto(fw, cuda, W)
    assert np.array_equal(out, oracle.fw_i32(W))


@pytest.mark.parametrize("case", ["negative", "too_large", "long_paths"])
def test_ineligible_inputs_fall_back_exactly(fw, cuda, oracle, case):
    n = 300
    W = oracle.generate_graph(n, 0.3, 9, 1, 100)
    if case == "negative":
        W[3, 7] = -5
        W[7, 3] = 10
    elif case == "too_large":
        W[1, 2] = 40000  # finite but above the 16-bit range
    else:  # a chain whose distances pass the 16-bit cap
        W = np.full((n, n), INF, dtype=np.int32)
        np.fill_diagonal(W, 0)
        for i in range(n - 1):
            W[i, i + 1] = 20000
    out, used = run_auto(fw, cuda, W)
    assert np.array_equal(out, oracle.fw_i32(W))
    assert not used


def test_kappa_8_fallback_and_repeat(fw, cuda, oracle):
    W = oracle.generate_graph(900, 0.3, 3, 1, 100)
    W[0, 1] = -1
    ref = oracle.fw_i32(W)
    for _ in range(2):
        out, used = run_auto(fw, cuda, W, kappa=8)
        assert np.array_equal(out, ref) and not used
    W2 = oracle.generate_graph(900, 0.3, 4, 1, 100)
    out, used = run_auto(fw, cuda, W2, kappa=8)
    assert np.array_equal(out, oracle.fw_i32(W2)) and used
