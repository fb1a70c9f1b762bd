"""TwoAdicFriPcs::open on a resident LDE (p3g_pcs_open_values, p3g_pcs_reduce),
bit-exact: the reference's own opened values and first FRI commitment for
every golden case (GPU LDE -> GPU opened values -> GPU reduced opening ->
GPU commit_matrix), random shapes against the oracle in both row orders and
both q orders with up to four points, and a commit's resident bit-reversed
LDE opened directly."""
import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P
from test_oracle import _bitrev_rows

pytestmark = pytest.mark.gpu


def test_golden_pcs_open_on_gpu(gpu_ctx, golden):
    for case in golden["pcs_open"]:
        shapes = [tuple(int(v) for v in s.split("x")) for s in case["shapes"]]
        qs, ap, opened_all = {}, 0, []
        bufs = []
        for i, (lh, w) in enumerate(shapes):
            t = O.bb_random_matrix(1 << lh, w, case["seed"] + i)
            d_t = gpu_ctx.to_device(t)
            log_n = lh + case["log_blowup"]
            d_lde = gpu_ctx.alloc((1 << log_n) * w * 4)
            gpu_ctx.coset_lde_device(P.BABYBEAR, d_t.ptr, lh, w, case["log_blowup"], case["shift"], False, d_lde.ptr)
            ov = gpu_ctx.pcs_open_values_device(d_lde.ptr, log_n, w, False, case["shift"], [case["zeta"]])
            opened_all.append(ov.reshape(-1))
            if log_n not in qs:
                qs[log_n] = gpu_ctx.to_device(np.zeros((1 << log_n, 4), np.uint32))
            gpu_ctx.pcs_reduce_device(d_lde.ptr, log_n, w, False, case["shift"], [case["zeta"]], ov, case["alpha"],
                                      ap, True, qs[log_n].ptr)
            ap += w
            bufs += [d_t, d_lde]
        assert np.concatenate(opened_all).tolist() == case["opened"]
        tallest = max(qs)
        arity = 1 << case["log_arity0"]
        # prove_fri's first round commits the bit-reversed vector as (H / arity) x arity BabyBear^4
        tree = gpu_ctx.commit_matrix_device(P.BABYBEAR, qs[tallest].ptr, (1 << tallest) // arity, arity * 4)
        assert tree.layers()[-1][0].tolist() == case["commit0"]
        tree.free()
        for b in bufs + list(qs.values()):
            b.free()


@pytest.mark.parametrize("log_n,w,m,bitrev_rows,q_bitrev", [
    (4, 1, 1, False, False), (8, 5, 2, True, False), (11, 300, 1, False, True), (12, 17, 4, True, True),
    (14, 64, 2, True, True)])
def test_random_shapes_vs_oracle(gpu_ctx, log_n, w, m, bitrev_rows, q_bitrev):
    rng = np.random.default_rng(log_n * 10 + m)
    lde = rng.integers(0, O.BB_P, size=(1 << log_n, w), dtype=np.uint32)
    shift = 31
    pts = rng.integers(0, O.BB_P, size=(m, 4), dtype=np.uint32)
    alpha = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
    stored = _bitrev_rows(lde) if bitrev_rows else lde
    d = gpu_ctx.to_device(stored)
    got = gpu_ctx.pcs_open_values_device(d.ptr, log_n, w, bitrev_rows, shift, pts)
    want = np.stack([O.pcs_open_values(lde, shift, z, nthreads=8) for z in pts])
    assert np.array_equal(got, want)
    q0 = rng.integers(0, O.BB_P, size=(1 << log_n, 4), dtype=np.uint32)
    d_q = gpu_ctx.to_device(_bitrev_rows(q0) if q_bitrev else q0)
    gpu_ctx.pcs_reduce_device(d.ptr, log_n, w, bitrev_rows, shift, pts, want, alpha, 5, q_bitrev, d_q.ptr)
    got_q = d_q.download(np.uint32, ((1 << log_n), 4))
    want_q = O.pcs_reduce(lde, shift, pts, want, alpha, 5, q0.copy(), nthreads=8)
    assert np.array_equal(_bitrev_rows(got_q) if q_bitrev else got_q, want_q)
    d.free()
    d_q.free()


def test_open_the_commits_resident_lde(gpu_ctx):
    """The bit-reversed LDE a commit leaves on the device, opened in place,
    equals the opening of the natural-order LDE."""
    rng = np.random.default_rng(5)
    t = rng.integers(0, O.BB_P, size=(1 << 12, 24), dtype=np.uint32)
    d_t = gpu_ctx.to_device(t)
    tree = gpu_ctx.commit_traces_device(P.BABYBEAR, [(d_t.ptr, 12, 24, 1, 31)], 0)
    pts = rng.integers(0, O.BB_P, size=(2, 4), dtype=np.uint32)
    got = gpu_ctx.pcs_open_values_device(tree.leaf_ptr(0), 13, 24, True, 31, pts)
    lde = O.bb_coset_lde(t, 1, 31, bitrev=False)
    want = np.stack([O.pcs_open_values(lde, 31, z, nthreads=8) for z in pts])
    assert np.array_equal(got, want)
    tree.free()
    d_t.free()


def test_bad_arguments(gpu_ctx):
    d = gpu_ctx.alloc(1 << 12)
    with pytest.raises(P.P3GError):
        gpu_ctx.pcs_open_values_device(d.ptr, 4, 4, False, 0, [[1, 2, 3, 4]])  # shift 0
    with pytest.raises(P.P3GError):
        gpu_ctx.pcs_open_values_device(d.ptr, 4, 4, False, 31, np.zeros((5, 4), np.uint32))  # 5 points
    with pytest.raises(P.P3GError):
        gpu_ctx.pcs_open_values_device(d.ptr, 4, 4, False, 31, [[O.BB_P, 0, 0, 0]])  # not canonical
    d.free()
