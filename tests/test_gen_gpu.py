"""On-device generator (fw_generate_graph_device_i32) against the
reference's host generator (src/graph_generator.cpp:7-46): the input hashes
of the reference's own test and benchmark cases, and the oracle's
std::mt19937 generator over sizes, densities and weight ranges (including
ranges whose weight draws are rejected about half the time)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_json, sha

pytestmark = pytest.mark.gpu


def device_graph(fw, torch, n, density, seed, wmin, wmax):
    d = torch.empty((n, n), dtype=torch.int32, device="cuda")
    fw.generate_graph_device(d, n, density, seed, wmin, wmax)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def test_reference_case_hashes(fw, cuda):
    for c in load_json("reference_cases.json")["cases"]:
        a = device_graph(fw, cuda, c["n"], c["density"], c["seed"], c["wmin"], c["wmax"])
        assert sha(a) == c["input_sha256"], c["id"]


@pytest.mark.parametrize("n", [1, 2, 3, 17, 100, 999])
@pytest.mark.parametrize("density", [0.0, 0.1, 0.5, 1.0])
def test_matches_host_generator(fw, cuda, oracle, n, density):
    a = device_graph(fw, cuda, n, density, 1000 + n, 1, 100)
    assert np.array_equal(a, oracle.generate_graph(n, density, 1000 + n, 1, 100))


@pytest.mark.parametrize("wmin,wmax", [(0, 25000), (-5, 5), (7, 7), (-1, 2**31 - 1),
                                        (-2**31, 2**31 - 1), (0, 2**31 - 1)])
def test_weight_ranges(fw, cuda, oracle, wmin, wmax):
    n = 300
    a = device_graph(fw, cuda, n, 0.7, 77, wmin, wmax)
    assert np.array_equal(a, oracle.generate_graph(n, 0.7, 77, wmin, wmax))


def test_several_chunks(fw, cuda, oracle):
    """n = 5000: 2.5e7 pairs, so the word stream spans two 2^25-word chunks
    and ~60 000 parse segments."""
    n = 5000
    a = device_graph(fw, cuda, n, 0.9, 4242, 0, 25000)
    assert np.array_equal(a, oracle.generate_graph(n, 0.9, 4242, 0, 25000))
