"""GPU parity of FRI fold_matrix over BabyBear^4 (p3g_fold_matrix_bb4) against
the reference's TwoAdicFriFolding::fold_matrix (golden) and the oracle."""
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_fold_golden(gpu_ctx, golden):
    for case in golden["fold"]:
        lh = case["log_height"]
        raw = O.mt19937(case["seed"], 4 * (1 << lh) + 4) % np.uint32(O.BB_P)
        vals = raw[: 4 * (1 << lh)].reshape(-1, 4)
        out = gpu_ctx.fold_matrix_bb4(vals, lh, case["log_arity"], case["beta"])
        if "values" in case["out"]:
            assert out.reshape(-1).tolist() == case["out"]["values"], case


@pytest.mark.parametrize("log_arity", [1, 2, 3])
def test_fold_random_vs_oracle(gpu_ctx, log_arity):
    rng = np.random.default_rng(log_arity)
    for lh in (log_arity, log_arity + 1, 9, 14):
        v = rng.integers(0, O.BB_P, size=(1 << lh, 4), dtype=np.uint32)
        beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
        got = gpu_ctx.fold_matrix_bb4(v, lh, log_arity, beta)
        want = O.fold_matrix_bb4(v, lh, log_arity, beta, nthreads=os.cpu_count() or 1)
        assert np.array_equal(got, want), (lh, log_arity)


@pytest.mark.parametrize("log_arity", [1, 2, 3])
def test_fold_beta_on_a_node(gpu_ctx, log_arity):
    """beta equal to an interpolation node (base-field beta) takes the
    reference's early return (fri_folding.hpp:138-144)."""
    rng = np.random.default_rng(10 + log_arity)
    lh = 8
    v = rng.integers(0, O.BB_P, size=(1 << lh, 4), dtype=np.uint32)
    for beta in ([1, 0, 0, 0], [O.BB_P - 1, 0, 0, 0], [5, 0, 0, 0]):
        got = gpu_ctx.fold_matrix_bb4(v, lh, log_arity, beta)
        want = O.fold_matrix_bb4(v, lh, log_arity, beta)
        assert np.array_equal(got, want)


def test_fold_config3_size(gpu_ctx):
    """fold of a 2^19 BabyBear^4 quotient, log_arity 1 (the batched workload's fold)."""
    rng = np.random.default_rng(19)
    v = rng.integers(0, O.BB_P, size=(1 << 19, 4), dtype=np.uint32)
    beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
    got = gpu_ctx.fold_matrix_bb4(v, 19, 1, beta)
    want = O.fold_matrix_bb4(v, 19, 1, beta, nthreads=os.cpu_count() or 1)
    assert np.array_equal(got, want)


def test_fold_rejects_bad_arity(gpu_ctx):
    import p3g_gb300 as P
    v = np.zeros((16, 4), np.uint32)
    with pytest.raises(P.P3GError):
        gpu_ctx.fold_matrix_bb4(v, 4, 4, [1, 2, 3, 4])
    with pytest.raises(P.P3GError):
        gpu_ctx.fold_matrix_bb4(v, 4, 1, [O.BB_P, 0, 0, 0])
