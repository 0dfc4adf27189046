"""Regenerates the golden fixtures in this folder from the reference's own code.

Run where the reference checkout exists (the reference library is compiled
from its sources by ``make -C oracle ref``):

    python tests/golden/make_golden.py            # everything but the n=8192 case
    python tests/golden/make_golden.py --large    # also the n=8192 case (~8 min)

What is written:
* ``known_answer.json`` — the six fixed cases of the reference's test suites
  (src/tests.cpp:59-132, repeated in src/tests_gpu.cu:76-148): input, the
  expected matrix written in those tests, and the matrix the reference's
  fwBaselineCPU actually returns.
* ``reference_cases.json`` — for each randomized case of the reference's test
  suites (src/tests.cpp:156-159, src/tests_gpu.cu:172-180) and for the
  benchmark workloads with integer weights in [1, 100] (n = 1024 and
  n = 8192, density 0.9, seed 42): SHA-256 of the input
  matrix and of fwBaselineCPU's output (int32, row-major, little-endian).
  Inputs of the randomized cases come from the reference's own generator
  (src/graph_generator.cpp:48-80); the [1, 100] inputs, which that generator
  cannot produce, come from the oracle's restatement with the weight range as
  a parameter, and only their outputs are the reference's.
* ``small_full.npz`` — full input/output matrices of small reference-generated
  graphs (n = 1..65), for element-wise comparison.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

INF = O.INF


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def ref_fw(a: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(a, dtype=np.int32).copy()
    O.ref().ref_fw_baseline_cpu(out, out.shape[0])
    return out


def ref_gen(n: int, density: float, seed: int) -> np.ndarray:
    out = np.empty((n, n), dtype=np.int32)
    if O.ref().ref_generate_graph(out, n, density, seed):
        raise RuntimeError("reference generator failed")
    return out


# src/tests.cpp:59-132: (name, n, input, expected or None for the
# negative-cycle case, which the reference checks only through
# hasNegativeCycle).
KNOWN = [
    ("Single node (1x1)", 1, [0], [0]),
    ("No edges (2x2)", 2, [0, INF, INF, 0], [0, INF, INF, 0]),
    ("Simple path optimization (4x4)", 4,
     [0, 1, INF, 100, INF, 0, 1, INF, INF, INF, 0, 1, INF, INF, INF, 0],
     [0, 1, 2, 3, INF, 0, 1, 2, INF, INF, 0, 1, INF, INF, INF, 0]),
    ("Disconnected components (4x4)", 4,
     [0, 1, INF, INF, 1, 0, INF, INF, INF, INF, 0, 2, INF, INF, 2, 0],
     [0, 1, INF, INF, 1, 0, INF, INF, INF, INF, 0, 2, INF, INF, 2, 0]),
    ("Negative weights (3x3)", 3, [0, 5, 10, 0, 0, -1, INF, INF, 0], [0, 5, 4, 0, 0, -1, INF, INF, 0]),
    ("Negative cycle detection (3x3)", 3, [0, 2, INF, INF, 0, 1, INF, -3, 0], None),
]

# src/tests.cpp:156-159 (density 0.9) and src/tests_gpu.cu:172-180 (0.9 and 0.1).
RANDOM_CASES = [(128, 0.9, 42), (256, 0.9, 123), (512, 0.9, 456), (1024, 0.9, 789),
                (128, 0.1, 101), (256, 0.1, 202), (512, 0.1, 303), (1024, 0.1, 404)]

# Benchmark workloads with integer weights in [1, 100]: n = 1024 and 8192, density 0.9, seed 42.
WEIGHTED_CASES = [("w1-100_n1024_d0.9_s42", 1024, 0.9, 42)]
LARGE_CASES = [("w1-100_n8192_d0.9_s42", 8192, 0.9, 42)]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--large", action="store_true")
    args = ap.parse_args()
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        raise SystemExit("reference library not built (needs the reference checkout)")

    known = []
    for name, n, inp, exp in KNOWN:
        a = np.array(inp, dtype=np.int32).reshape(n, n)
        out = ref_fw(a)
        known.append({"name": name, "n": n, "input": a.ravel().tolist(),
                      "expected": exp, "reference_output": out.ravel().tolist(),
                      "reference_negative_cycle": bool(O.ref().ref_has_negative_cycle(out, n))})
    with open(os.path.join(HERE, "known_answer.json"), "w") as f:
        json.dump({"source": "src/tests.cpp:59-132", "inf": INF, "cases": known}, f, indent=1)

    path = os.path.join(HERE, "reference_cases.json")
    cases = {}
    if os.path.exists(path):
        with open(path) as f:
            cases = {c["id"]: c for c in json.load(f)["cases"]}
    for n, d, s in RANDOM_CASES:
        a = ref_gen(n, d, s)
        cases[f"ref_gen_n{n}_d{d}_s{s}"] = {
            "id": f"ref_gen_n{n}_d{d}_s{s}", "n": n, "density": d, "seed": s, "wmin": 0,
            "wmax": O.MAX_EDGE_WEIGHT, "input_generator": "reference",
            "input_sha256": sha(a), "output_sha256": sha(ref_fw(a))}
    todo = WEIGHTED_CASES + (LARGE_CASES if args.large else [])
    for tag, n, d, s in todo:
        a = O.generate_graph(n, d, s, 1, 100)
        print(f"solving {tag} n={n} with the reference baseline_cpu ...", flush=True)
        cases[tag] = {"id": tag, "n": n, "density": d, "seed": s, "wmin": 1, "wmax": 100,
                      "input_generator": "oracle", "input_sha256": sha(a), "output_sha256": sha(ref_fw(a))}
    with open(path, "w") as f:
        json.dump({"hash": "sha256 of int32 little-endian row-major bytes",
                   "cases": sorted(cases.values(), key=lambda c: (c["n"], c["id"]))}, f, indent=1)

    arrays = {}
    for n in list(range(1, 18)) + [31, 32, 33, 47, 63, 64, 65]:
        for d, s in ((0.5, 1000 + n), (0.1, 2000 + n)):
            a = ref_gen(n, d, s)
            arrays[f"in_n{n}_s{s}"] = a
            arrays[f"out_n{n}_s{s}"] = ref_fw(a)
    np.savez_compressed(os.path.join(HERE, "small_full.npz"), **arrays)
    print("wrote", len(known), "known-answer cases,", len(cases), "hashed cases,", len(arrays) // 2, "small matrices")


if __name__ == "__main__":
    main()
