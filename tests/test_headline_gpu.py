"""The benchmark's headline configuration at full size: n = 32768 (the
reference's maximum, MAX_N - 1, a 4 GiB int32 matrix), density 0.5, weights
uniform in [1, 100], seed 7. The reference checks every GPU result against
fwBaselineCPU (src/tests_gpu.cu:41-74); at this size the k-i-j sweep takes
hours on the host, so the checks are size-independent instead: the three
schedules that stand in for tiling_gpu, multi_layer_tiling_gpu (kappa 8, the
two-block pass) and the exact packed path (FW_VARIANT_AUTO) must agree bit
for bit, and full rows of the result must equal the oracle's Dijkstra rows
from the same sources (exact for non-negative weights)."""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_headline_configuration_n32768(fw, cuda, oracle):
    n = 32768
    W = oracle.generate_graph(n, 0.5, 7, 1, 100)  # the oracle's generator, independent of the product
    pristine = cuda.from_numpy(W).cuda()

    results = {}
    for name, variant, kappa in (("multi_layer_tiling_gpu", fw.VARIANT_MULTI_LAYER, 8),
                                 ("auto", fw.VARIANT_AUTO, 8), ("tiling_gpu", fw.VARIANT_TILING, 0)):
        d = pristine.clone()
        fw.apsp_i32(d, n, 32, kappa, variant, None)
        fw.check_faults(None)
        if variant == fw.VARIANT_AUTO:
            assert fw.auto_used_packed(None), "weights 1..100 at n = 32768 fit the exact packed path"
        results[name] = d
    ref = results.pop("multi_layer_tiling_gpu")
    for name, d in results.items():
        assert cuda.equal(d, ref), f"{name} differs from multi_layer_tiling_gpu"
    del results

    rng = np.random.default_rng(32768)
    rows = sorted({0, 1, n // 2, n - 1, *[int(x) for x in rng.choice(n, 8, replace=False)]})
    got = {s: ref[s].cpu().numpy() for s in rows}
    with ThreadPoolExecutor(max_workers=min(len(rows), os.cpu_count() or 1)) as ex:
        want = dict(zip(rows, ex.map(lambda s: oracle.sssp_row(W, s), rows)))
    wrong = [s for s in rows if not np.array_equal(got[s], want[s])]
    assert wrong == [], f"rows {wrong} differ from Dijkstra"
    # the workload's distances: all pairs reachable at density 0.5, small integers
    assert got[0].max() < 1000 and got[0].min() == 0
