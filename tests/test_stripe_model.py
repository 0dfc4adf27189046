"""A numpy model of the stripe sweep's schedule (fw_cuda_gb300/csrc/fw_stripe.cu),
checked against the oracle's baseline_cpu sweep (src/fw_baseline_cpu.cpp:3-16)
and the reference's known answers (src/tests.cpp:59-132) on the CPU.

The model follows the kernel's arithmetic stage by stage: 8-row stripes;
stage z's owner closes the 8 x 8 diagonal block with the k-sequential sweep
(each pivot reading row and column k as they were before it), turns its
stripe into min(R, Dg* (x) R) and sets the diagonal block to Dg*; every other
stripe becomes min(D, C (x) R') with C its own pivot columns from before the
stage. int32 sums wrap as on the GPU. This pins the algebra the kernel relies
on (C' (x) R' = C (x) R' for a closed Dg*) independently of the GPU."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_json

INF = 1_000_000_000
R = 8


def wrap(x: np.ndarray) -> np.ndarray:
    return ((x + 2**31) % 2**32 - 2**31).astype(np.int64)


def stripe_model(W: np.ndarray) -> np.ndarray:
    n = W.shape[0]
    ns = -(-n // R)
    A = np.full((ns * R, ns * R), INF, dtype=np.int64)
    A[:n, :n] = W

    def close_publish(z: int) -> np.ndarray:
        rows = slice(z * R, z * R + R)
        dg = A[rows, z * R:z * R + R].copy()
        for k in range(R):
            a, b = dg[:, k].copy(), dg[k, :].copy()
            dg = np.minimum(wrap(a[:, None] + b[None, :]), dg)
        S = A[rows, :].copy()
        out = S.copy()
        for k in range(R):
            out = np.minimum(wrap(dg[:, k][:, None] + S[k][None, :]), out)
        out[:, z * R:z * R + R] = dg
        A[rows, :] = out
        return out.copy()

    published = {0: close_publish(0)}
    for s in range(ns):
        C = A[:, s * R:s * R + R].copy()
        P = published[s]
        for z in range(ns):
            if z == s:
                continue
            rows = slice(z * R, z * R + R)
            D = A[rows, :]
            c = C[rows, :]
            for k in range(R):
                D = np.minimum(wrap(c[:, k][:, None] + P[k][None, :]), D)
            A[rows, :] = D
            if z == s + 1:
                published[z] = close_publish(z)
    return A[:n, :n].astype(np.int32)


def test_known_answers():
    for case in load_json("known_answer.json")["cases"]:
        n = case["n"]
        a = np.array(case["input"], dtype=np.int64).reshape(n, n)
        assert stripe_model(a).ravel().tolist() == case["reference_output"], case["name"]


@pytest.mark.parametrize("n", [1, 2, 5, 8, 9, 16, 17, 40, 100, 130])
def test_against_the_oracle(oracle, n):
    rng = np.random.default_rng(n)
    for dens in (0.05, 0.5):
        W = oracle.generate_graph(n, dens, n + int(dens * 100), 0, 25000)
        assert np.array_equal(stripe_model(W), oracle.fw_i32(W)), (n, dens)
        # negative weights without negative cycles: w + p(u) - p(v)
        p = rng.integers(0, 60, n).astype(np.int64)
        Wn = np.where(W < INF, W.astype(np.int64) + p[:, None] - p[None, :], INF)
        np.fill_diagonal(Wn, 0)
        Wn = Wn.astype(np.int32)
        assert np.array_equal(stripe_model(Wn), oracle.fw_i32(Wn)), (n, dens, "negative")
        # positive self-loops
        W2 = W.copy()
        np.fill_diagonal(W2, rng.integers(1, 300, n).astype(np.int32))
        assert np.array_equal(stripe_model(W2), oracle.fw_i32(W2)), (n, dens, "loops")
