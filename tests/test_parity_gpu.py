"""Bit-exact parity of the int32 APSP engine with the oracle, through the C ABI.

Cases follow the reference's own suites (src/tests_gpu.cu:76-185): the six
known-answer matrices, the eight randomized graphs (n = 128..1024, density
0.9 and 0.1) compared by hash with the reference's fwBaselineCPU output, plus
ragged sizes around every tile boundary, negative weights without negative
cycles, negative cycles, and the benchmark workloads at n = 1024 and n = 8192
(density 0.9, weights 1..100, seed 42).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GOLDEN, load_json, sha

pytestmark = pytest.mark.gpu

INF = 1_000_000_000
VARIANTS = {"baseline_gpu": 0, "tiling_gpu": 1, "multi_layer_tiling_gpu": 2, "auto": 3}


def solve(fw, torch, W: np.ndarray, variant: int, kappa: int = 0, tile: int = 0) -> np.ndarray:
    n = W.shape[0]
    d = torch.from_numpy(np.ascontiguousarray(W, dtype=np.int32)).cuda()
    fw.apsp_i32(d, n, tile, kappa, variant, None)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def potential_shift(W: np.ndarray, rng) -> np.ndarray:
    """Negative edge weights without negative cycles: w'(u,v) = w(u,v) + p(u) - p(v)."""
    n = W.shape[0]
    p = rng.integers(0, 50, n).astype(np.int64)
    Wl = W.astype(np.int64)
    out = np.where(W < INF, Wl + p[:, None] - p[None, :], INF)
    np.fill_diagonal(out, 0)
    return out.astype(np.int32)


@pytest.mark.parametrize("name", list(VARIANTS))
def test_known_answer(fw, cuda, name):
    for case in load_json("known_answer.json")["cases"]:
        n = case["n"]
        a = np.array(case["input"], dtype=np.int32).reshape(n, n)
        out = solve(fw, cuda, a, VARIANTS[name], kappa=4, tile=32)
        if case["expected"] is None:
            assert np.any(np.diag(out) < 0), case["name"]  # hasNegativeCycle, src/utils.cpp:5-12
        else:
            assert out.ravel().tolist() == case["expected"], (name, case["name"])


@pytest.mark.parametrize("name", list(VARIANTS))
def test_reference_random_cases(fw, cuda, name):
    for c in load_json("reference_cases.json")["cases"]:
        if not c["id"].startswith("ref_gen"):
            continue
        a = fw.generate_graph(c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
        assert sha(a) == c["input_sha256"]
        out = solve(fw, cuda, a, VARIANTS[name], kappa=4)
        assert sha(out) == c["output_sha256"], (name, c["id"])


@pytest.mark.parametrize("name", list(VARIANTS))
def test_small_full_matrices(fw, cuda, name):
    z = np.load(os.path.join(GOLDEN, "small_full.npz"))
    for k in z.files:
        if not k.startswith("in_"):
            continue
        out = solve(fw, cuda, z[k], VARIANTS[name], kappa=2)
        assert np.array_equal(out, z["out" + k[2:]]), (name, k)


RAGGED = [1, 2, 3, 4, 5, 7, 8, 31, 33, 63, 64, 65, 100, 127, 128, 129, 130, 191, 255, 256, 257,
          300, 383, 384, 385, 511, 513, 640, 1000]


@pytest.mark.parametrize("n", RAGGED)
def test_ragged_sizes(fw, cuda, oracle, n):
    rng = np.random.default_rng(n)
    dens = float(rng.choice([0.02, 0.2, 0.9]))
    W = oracle.generate_graph(n, dens, 100 + n, 0, 25000)
    ref = oracle.fw_i32(W)
    for name, v in VARIANTS.items():
        if name == "baseline_gpu" and n > 700:
            continue
        for kappa in ((1, 4, 8) if v == 2 else (4, 8) if v == 3 else (0,)):
            assert np.array_equal(solve(fw, cuda, W, v, kappa=kappa), ref), (name, n, kappa)


@pytest.mark.parametrize("n", [5, 130, 257, 517])
def test_negative_weights_without_negative_cycles(fw, cuda, oracle, n):
    rng = np.random.default_rng(1000 + n)
    W = potential_shift(oracle.generate_graph(n, 0.3, 7 + n, 0, 100), rng)
    assert W.min() < 0
    ref = oracle.fw_i32(W)
    for v in VARIANTS.values():
        assert np.array_equal(solve(fw, cuda, W, v), ref), (v, n)


@pytest.mark.parametrize("n", [3, 40, 200, 300])
def test_negative_cycle_detected_and_deterministic(fw, cuda, oracle, n):
    # The cycle sits on the last three vertices, so no later pivot compounds
    # its weight into an int32 overflow (which would wrap in any sweep).
    W = oracle.generate_graph(n, 0.05, 50 + n, 5, 100)
    cyc = np.arange(n - 3, n)
    for a, b in zip(cyc, np.roll(cyc, -1)):
        W[a, b] = -40
    ref = oracle.fw_i32(W)
    assert oracle.has_negative_cycle(ref)
    for v in (0, 1, 2, 3):
        out1 = solve(fw, cuda, W, v)
        out2 = solve(fw, cuda, W, v)
        assert np.any(np.diag(out1) < 0)
        assert np.all(np.diag(out1)[cyc] < 0)
        assert np.array_equal(out1, out2)  # no races: the same input gives the same output


def test_n1024_weights_1_100(fw, cuda):
    """n=1024, density 0.9, weights [1, 100], seed 42 vs the reference baseline_cpu."""
    c = {c["id"]: c for c in load_json("reference_cases.json")["cases"]}["w1-100_n1024_d0.9_s42"]
    a = fw.generate_graph(1024, 0.9, 42, 1, 100)
    assert sha(a) == c["input_sha256"]
    for v in VARIANTS.values():
        assert sha(solve(fw, cuda, a, v, kappa=4)) == c["output_sha256"], v


N8192 = "w1-100_n8192_d0.9_s42"


def test_n8192_kappa_sweep(fw, cuda, oracle):
    """n=8192, density 0.9, weights [1, 100], seed 42; kappa in {1,2,4,6,8}."""
    cases = {c["id"]: c for c in load_json("reference_cases.json")["cases"]}
    a = fw.generate_graph(8192, 0.9, 42, 1, 100)
    want = cases[N8192]["output_sha256"] if N8192 in cases else None
    if want is not None:
        assert sha(a) == cases[N8192]["input_sha256"]
    outs = set()
    for kappa in (1, 2, 4, 6, 8):
        outs.add(sha(solve(fw, cuda, a, 2, kappa=kappa)))
    outs.add(sha(solve(fw, cuda, a, 1)))
    outs.add(sha(solve(fw, cuda, a, 3, kappa=8)))
    assert len(outs) == 1
    if want is not None:
        assert outs == {want}
    else:  # no golden hash in this checkout: check sampled rows against Dijkstra
        out = solve(fw, cuda, a, 2)
        for src in (0, 4095, 8191):
            assert np.array_equal(out[src], oracle.sssp_row(a, src))


def test_workspace_variant_matches(fw, cuda, oracle):
    n = 700
    W = oracle.generate_graph(n, 0.2, 3, 0, 25000)
    ref = oracle.fw_i32(W)
    need = fw.workspace_bytes_i32(n, variant=2)
    ws = cuda.empty(need // 4 + 64, dtype=cuda.int32, device="cuda")
    # full size: look-ahead schedule; the 256-byte status block and one panel
    # buffer: the minimum
    for nbytes in (need, 256 + (need - 256) // 2):
        for v in (1, 2):
            d = cuda.from_numpy(W).cuda()
            fw.apsp_i32_ws(d, n, ws, nbytes, variant=v)
            cuda.cuda.synchronize()
            assert np.array_equal(d.cpu().numpy(), ref), (nbytes, v)


def test_stream_argument(fw, cuda, oracle):
    n = 333
    W = oracle.generate_graph(n, 0.5, 9, 0, 25000)
    ref = oracle.fw_i32(W)
    s = cuda.cuda.Stream()
    with cuda.cuda.stream(s):
        d = cuda.from_numpy(W).cuda()
    fw.apsp_i32(d, n, 0, 4, 2, s)
    s.synchronize()
    assert np.array_equal(d.cpu().numpy(), ref)


def test_registry_functions_synchronise(fw, cuda, oracle):
    n = 200
    W = oracle.generate_graph(n, 0.4, 1, 0, 25000)
    ref = oracle.fw_i32(W)
    for name in fw.GPU_ALGORITHMS:
        d = cuda.from_numpy(W).cuda()
        fw.get_gpu_algorithm_func(name)(d, n, 32, 4)
        assert np.array_equal(d.cpu().numpy(), ref), name


def test_reference_gpu_kernels_agree(fw, cuda, oracle):
    """The reference's own kernels (built for sm_103a from its sources) on the same inputs.

    baseline_gpu, tiling_gpu and multi_layer_tiling_gpu with kappa = 1 must
    agree with this engine bit for bit. For kappa >= 2 the reference's
    multi-layer remainder kernel reuses its shared tiles for the next pivot
    block without a barrier after the inner loop
    (src/fw_multi_layer_tiling_gpu.cu:473-499), so its output varies from run
    to run and can fall below the true distance on this GPU; there the
    reference's baseline_cpu (the oracle of the reference's own test suite) is
    the parity target, and the reference kernel's mismatch count is only
    reported.
    """
    if not oracle.refgpu_available():
        pytest.skip("reference kernels not built in this checkout")
    for n, d, s in ((128, 0.9, 42), (1000, 0.1, 5), (1024, 0.5, 6)):
        W = fw.generate_graph(n, d, s, 1, 100)
        truth = oracle.fw_i32(W)
        mine = solve(fw, cuda, W, 2, kappa=4)
        assert np.array_equal(mine, truth)
        for name, kappa in (("tiling_gpu", 0), ("multi_layer_tiling_gpu", 1), ("baseline_gpu", 0)):
            t = cuda.from_numpy(W).cuda()
            oracle.refgpu_run(name, t.data_ptr(), n, kappa)
            assert np.array_equal(t.cpu().numpy(), mine), (name, kappa, n)
        for kappa in (2, 4):
            t = cuda.from_numpy(W).cuda()
            oracle.refgpu_run("multi_layer_tiling_gpu", t.data_ptr(), n, kappa)
            bad = int(np.count_nonzero(t.cpu().numpy() != truth))
            print(f"reference multi_layer_tiling_gpu kappa={kappa} n={n}: {bad} entries differ from baseline_cpu")


def test_no_tile_copy_faults(fw, cuda):
    """The remainder kernels' TMA copies all arrived within their bounded
    waits during the solves above (a fault would be recorded, not hung on)."""
    assert fw.copy_faults() == 0
