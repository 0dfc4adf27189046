"""The oracle is pinned before it is trusted: against the reference's own test
vectors (src/tests.cpp:59-132), against hashes and matrices produced by the
reference's own generator and fwBaselineCPU (tests/golden/make_golden.py),
and, where the reference library was built in this checkout, against that
library directly."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_json, sha

INF = 1_000_000_000


def test_known_answer_cases(oracle):
    data = load_json("known_answer.json")
    assert data["inf"] == INF and len(data["cases"]) == 6
    for case in data["cases"]:
        n = case["n"]
        a = np.array(case["input"], dtype=np.int32).reshape(n, n)
        out = oracle.fw_i32(a)
        assert out.ravel().tolist() == case["reference_output"], case["name"]
        if case["expected"] is not None:
            assert out.ravel().tolist() == case["expected"], case["name"]
        else:
            assert oracle.has_negative_cycle(out) and case["reference_negative_cycle"]


def test_small_full_matrices(oracle):
    z = np.load(__import__("os").path.join(__import__("conftest").GOLDEN, "small_full.npz"))
    keys = [k for k in z.files if k.startswith("in_")]
    assert len(keys) >= 40
    for k in keys:
        n = int(k.split("_")[1][1:])
        s = int(k.split("_")[2][1:])
        d = 0.5 if s < 2000 else 0.1
        inp = z[k]
        assert np.array_equal(oracle.generate_graph(n, d, s), inp), k
        assert np.array_equal(oracle.fw_i32(inp), z["out" + k[2:]]), k


@pytest.mark.parametrize("case_id", ["ref_gen_n128_d0.9_s42", "ref_gen_n256_d0.1_s202",
                                     "ref_gen_n512_d0.9_s456", "ref_gen_n1024_d0.1_s404", "w1-100_n1024_d0.9_s42"])
def test_reference_hashes(oracle, case_id):
    cases = {c["id"]: c for c in load_json("reference_cases.json")["cases"]}
    c = cases[case_id]
    a = oracle.generate_graph(c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
    assert sha(a) == c["input_sha256"]
    assert sha(oracle.fw_i32(a)) == c["output_sha256"]


def test_all_reference_input_hashes(oracle):
    for c in load_json("reference_cases.json")["cases"]:
        if c["n"] > 2048:
            continue
        a = oracle.generate_graph(c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
        assert sha(a) == c["input_sha256"], c["id"]


def test_threaded_pivots_match(oracle):
    a = oracle.generate_graph(300, 0.3, 11, 1, 100)
    ref = oracle.fw_i32(a)
    for threads in (1, 3, 8):
        t = a.copy()
        oracle.fw_i32_pivots(t, 0, 150, threads)
        oracle.fw_i32_pivots(t, 150, 300, threads)
        assert np.array_equal(t, ref)


def test_sssp_rows_match_sweep(oracle):
    for n, d, s in ((257, 0.05, 3), (200, 0.9, 4)):
        a = oracle.generate_graph(n, d, s, 0, 25000)
        full = oracle.fw_i32(a)
        for src in (0, 1, n // 2, n - 1):
            assert np.array_equal(oracle.sssp_row(a, src), full[src])


def test_fp64_nexthop_paths_are_consistent(oracle):
    rng = np.random.default_rng(5)
    n = 40
    W = np.where(rng.random((n, n)) < 0.3, rng.uniform(0.5, 10.0, (n, n)), np.inf)
    np.fill_diagonal(W, 0.0)
    D, nh = oracle.fw_f64_nexthop(W)
    # Walking the next hops reproduces every finite distance.
    for i in range(n):
        for j in range(n):
            if i == j or not np.isfinite(D[i, j]):
                assert i == j or nh[i, j] == -1
                continue
            u, tot, steps = i, 0.0, 0
            while u != j:
                v = nh[u, j]
                tot += W[u, v]
                u = v
                steps += 1
                assert steps <= n
            assert abs(tot - D[i, j]) <= 1e-9 * max(1.0, D[i, j])


def test_oracle_gradient_matches_finite_differences(oracle):
    rng = np.random.default_rng(7)
    n = 12
    W = np.where(rng.random((n, n)) < 0.35, rng.uniform(0.5, 10.0, (n, n)), np.inf)
    np.fill_diagonal(W, 0.0)
    G = rng.standard_normal((n, n))
    D, nh = oracle.fw_f64_nexthop(W)
    dW, bad = oracle.fw_backward(G, nh)
    assert bad == 0
    eps = 1e-3

    def loss(Wp):
        Dp, _ = oracle.fw_f64_nexthop(Wp)
        fin = np.isfinite(Dp)
        return float(np.sum(G[fin] * Dp[fin]))

    for u in range(n):
        for v in range(n):
            if u == v or not np.isfinite(W[u, v]):
                continue
            Wp, Wm = W.copy(), W.copy()
            Wp[u, v] += eps
            Wm[u, v] -= eps
            fd = (loss(Wp) - loss(Wm)) / (2 * eps)
            assert abs(fd - dW[u, v]) <= 1e-6 * max(1.0, abs(fd)), (u, v)


def test_reference_library_agrees(oracle):
    if not oracle.ref_available():
        pytest.skip("reference library not built in this checkout")
    R = oracle.ref()
    for n, d, s in ((100, 0.3, 9), (129, 0.9, 10)):
        a = np.empty((n, n), dtype=np.int32)
        assert R.ref_generate_graph(a, n, d, s) == 0
        assert np.array_equal(a, oracle.generate_graph(n, d, s))
        b = a.copy()
        R.ref_fw_baseline_cpu(b, n)
        assert np.array_equal(b, oracle.fw_i32(a))


def test_mt19937_jump_ahead_matches_std(fw, oracle):
    """The device generator's starting states come from polynomial jump-ahead
    (host side of fw_generate_graph_device_i32); its outputs after a skip
    equal std::mt19937 after discard(skip)."""
    for seed, skip in [(5489, 0), (42, 1), (42, 623), (42, 624), (7, 625), (123, 2**25),
                       (99, 3 * 2**25 + 17), (7, 2**28 + 12345), (11, 40 * 2**25 + 5)]:
        count = 1500
        assert np.array_equal(fw.mt19937_outputs(seed, skip, count),
                              oracle.mt19937_outputs(seed, skip, count)), (seed, skip)
