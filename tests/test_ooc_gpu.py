"""Out-of-core sweep (fw_apsp_i32_host): the matrix stays in host memory and
streams through the device in row stripes. Bit-exact against the oracle's
baseline_cpu sweep (src/fw_baseline_cpu.cpp:3-16) at small n with pass
widths and stripe heights that force many passes, ragged last passes and
stripes; and at n = 40000, beyond the reference's MAX_N = 32769
(include/constants.h:5), against the in-core sweep of the same matrix and
the oracle's Dijkstra rows."""
from __future__ import annotations

import numpy as np
import pytest

from test_parity_gpu import potential_shift

INF = 1_000_000_000

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 5, 127, 129, 333, 777, 1000, 1024])
@pytest.mark.parametrize("W,H", [(128, 128), (256, 384), (0, 0)])
def test_matches_oracle(fw, cuda, oracle, n, W, H):
    D = oracle.generate_graph(n, 0.3, 11 + n, 1, 100)
    ref = oracle.fw_i32(D)
    fw.apsp_i32_host(D, n, W, H)  # pageable numpy memory
    assert np.array_equal(D, ref), (n, W, H)


@pytest.mark.parametrize("n", [300, 640])
def test_negative_weights_pinned_tensor(fw, cuda, oracle, n):
    rng = np.random.default_rng(77 + n)
    W = potential_shift(oracle.generate_graph(n, 0.3, 5 + n, 0, 100), rng)
    assert W.min() < 0
    ref = oracle.fw_i32(W)
    h = cuda.from_numpy(W.copy()).pin_memory()
    stream = cuda.cuda.Stream()
    fw.apsp_i32_host(h, n, 128, 256, stream)
    assert np.array_equal(h.numpy(), ref)


def test_reference_default_weights(fw, cuda, oracle):
    """The reference generator's own weight range U{0..25000}."""
    n = 700
    D = oracle.generate_graph(n, 0.9, 42, 0, 25000)
    ref = oracle.fw_i32(D)
    fw.apsp_i32_host(D, n, 256, 128)
    assert np.array_equal(D, ref)


def test_beyond_reference_max_n(fw, cuda, oracle):
    """n = 40000 (6.4 GB): the out-of-core result equals the in-core int32
    and packed results bit for bit, and sampled rows equal the oracle's
    Dijkstra rows."""
    torch = cuda
    n = 40000
    g = torch.Generator(device="cuda").manual_seed(4242)
    w = torch.randint(1, 101, (n, n), device="cuda", dtype=torch.int32, generator=g)
    keep = torch.rand((n, n), device="cuda", generator=g) < 0.02
    d = torch.where(keep, w, torch.full_like(w, INF))
    d.fill_diagonal_(0)
    h = torch.empty((n, n), dtype=torch.int32).pin_memory()
    h.copy_(d)
    rows = [0, 12345, n - 1]
    W_rows = {r: None for r in rows}
    W_host = h.numpy().copy()
    for r in rows:
        W_rows[r] = oracle.sssp_row(W_host, r)
    del W_host

    d_auto = d.clone()
    fw.apsp_i32(d, n, 32, 8, fw.VARIANT_MULTI_LAYER, None)
    fw.apsp_i32(d_auto, n, 32, 8, fw.VARIANT_AUTO, None)
    assert fw.auto_used_packed(None)
    fw.apsp_i32_host(h, n, 2048, 0)
    torch.cuda.synchronize()
    assert torch.equal(d, d_auto)
    del d_auto
    assert torch.equal(d.cpu(), h)
    out = h.numpy()
    for r in rows:
        assert np.array_equal(out[r], W_rows[r]), r


@pytest.mark.parametrize("W,H", [(1024, 512), (4096, 0), (6016, 1024)])
def test_wide_passes_match_in_core(fw, cuda, W, H):
    """Pass widths from a sixth of n up to all of it (one pass), against the
    in-core int32 sweep of the same matrix."""
    torch = cuda
    n = 6000
    d = torch.empty((n, n), dtype=torch.int32, device="cuda")
    fw.generate_graph_device(d, n, 0.4, 99, 1, 100)
    h = torch.empty((n, n), dtype=torch.int32).pin_memory()
    h.copy_(d)
    fw.apsp_i32(d, n, 32, 8, fw.VARIANT_MULTI_LAYER, None)
    fw.apsp_i32_host(h, n, W, H)
    torch.cuda.synchronize()
    assert torch.equal(d.cpu(), h)
