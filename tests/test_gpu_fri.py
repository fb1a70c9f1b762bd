"""The FRI commit phase of prove_fri (fri_prover.hpp:73-195) with every data
step on the GPU -- each round's commitment (p3g_commit_matrix of the current
vector as (n / arity) x (4 arity) BabyBear), fold (p3g_fold_matrix_bb4) and
mix-in of the next reduced opening (p3g_bb4_axpy) -- and the reduced openings
themselves from the GPU's PCS-open passes, driven by the oracle's restated
transcript, and the query-phase proof-of-work witness from p3g_grind.  Every
round's root, the final polynomial and the witness must equal the reference's
proof for each golden case."""
import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P
from test_oracle import fri_commit_phase, fri_query_pow, open_transcript

pytestmark = pytest.mark.gpu


class Dev:
    """A device BabyBear^4 vector of n values."""

    def __init__(self, buf, n):
        self.buf, self.n = buf, n


def test_fri_commit_phase_on_gpu_vs_reference(gpu_ctx, golden):
    for case in golden["pcs_open"]:
        tr, zeta, alpha = open_transcript(case)
        shapes = [tuple(int(v) for v in s.split("x")) for s in case["shapes"]]
        qs, ap, keep = {}, 0, []
        for i, (lh, w) in enumerate(shapes):
            t = O.bb_random_matrix(1 << lh, w, case["seed"] + i)
            d_t = gpu_ctx.to_device(t)
            log_n = lh + case["log_blowup"]
            d_lde = gpu_ctx.alloc((1 << log_n) * w * 4)
            gpu_ctx.coset_lde_device(P.BABYBEAR, d_t.ptr, lh, w, case["log_blowup"], case["shift"], False, d_lde.ptr)
            ov = gpu_ctx.pcs_open_values_device(d_lde.ptr, log_n, w, False, case["shift"], [zeta])
            for v in ov.reshape(-1, 4):
                tr.observe_ext(v)
            if log_n not in qs:
                qs[log_n] = gpu_ctx.to_device(np.zeros((1 << log_n, 4), np.uint32))
            gpu_ctx.pcs_reduce_device(d_lde.ptr, log_n, w, False, case["shift"], [zeta], ov, alpha, ap, True,
                                      qs[log_n].ptr)
            ap += w
            keep += [d_t, d_lde]
        inputs = [Dev(qs[h], 1 << h) for h in sorted(qs, reverse=True)]

        def commit(cur, arity):
            tree = gpu_ctx.commit_matrix_device(P.BABYBEAR, cur.buf.ptr, cur.n // arity, 4 * arity)
            root = tree.layers()[-1][0]
            tree.free()
            return root

        def fold(cur, lh, la, beta):
            out = gpu_ctx.alloc((cur.n >> la) * 16)
            gpu_ctx.fold_matrix_bb4_device(cur.buf.ptr, lh, la, beta, out.ptr)
            keep.append(out)
            return Dev(out, cur.n >> la)

        def axpy(cur, a, nxt):
            gpu_ctx.bb4_axpy_device(cur.buf.ptr, nxt.buf.ptr, cur.n, a)
            return cur

        roots, final, arities = fri_commit_phase(case, inputs, tr, commit, fold, axpy, length=lambda c: c.n,
                                                 download=lambda c: c.buf.download(np.uint32, (c.n, 4)))
        assert [r.tolist() for r in roots] == case["commits"]
        assert final.tolist() == case["final_poly"]

        def gpu_grind(t, bits):  # the query-phase witness from the GPU search
            w = gpu_ctx.grind(P.BABYBEAR, t.state, t.inp, bits)
            assert t.check_witness(bits, w)
            return w

        assert fri_query_pow(case, tr, final, arities, gpu_grind) == case["fri"]["query_pow_witness"]
        for b in keep + list(qs.values()):
            b.free()


def test_bb4_axpy_matches_oracle(gpu_ctx):
    rng = np.random.default_rng(3)
    for n in (1, 7, 4096):
        y = rng.integers(0, O.BB_P, size=(n, 4), dtype=np.uint32)
        x = rng.integers(0, O.BB_P, size=(n, 4), dtype=np.uint32)
        a = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
        dy, dx = gpu_ctx.to_device(y), gpu_ctx.to_device(x)
        gpu_ctx.bb4_axpy_device(dy.ptr, dx.ptr, n, a)
        assert np.array_equal(dy.download(np.uint32, (n, 4)), O.bb4_axpy(y, a, x))
        dy.free()
        dx.free()
