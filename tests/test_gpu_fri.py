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
from test_oracle import fri_commit_phase, fri_query_openings, fri_query_pow, open_transcript

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


def _oracle_fri(case, tr, vectors):
    """The oracle's prove_fri from the transcript tr over host vectors (tallest
    first): roots, final polynomial, query witness, indices and openings."""
    committed = []

    def commit(cur, arity):
        mat = cur.reshape(-1, 4 * arity)
        layers = O.commit_matrix(O.bb16_params(), mat)
        committed.append((mat, layers, arity.bit_length() - 1))
        return layers[-1][0]

    roots, final, arities = fri_commit_phase(case, vectors, tr, commit=commit,
                                             fold=lambda cur, lh, la, beta: O.fold_matrix_bb4(cur, lh, la, beta),
                                             axpy=O.bb4_axpy, length=len, download=lambda c: c)
    w = fri_query_pow(case, tr, final, arities, lambda t, bits: t.grind(bits))
    idx, openings = fri_query_openings(case, tr, committed)
    return roots, final, w, idx, openings


def _check_fri_result(res, case, roots, final, w, idx, openings, tr):
    assert res["commits"].tolist() == [r.tolist() for r in roots]
    assert res["final_poly"].tolist() == final.tolist()
    assert res["query_witness"] == w
    assert res["query_indices"].tolist() == idx
    for q, steps in enumerate(openings):
        cur = idx[q]
        for r, step in enumerate(steps):
            la = step["log_arity"]
            pos = cur & ((1 << la) - 1)
            vals = res["rows"][r][q].reshape(-1, 4)
            assert [vals[j].tolist() for j in range(1 << la) if j != pos] == step["siblings"], (q, r)
            assert res["paths"][r][q].tolist() == step["path"], (q, r)
            cur >>= la
    # the challenger afterwards is the oracle transcript's
    assert res["state"].tolist() == [int(x) for x in tr.state]
    assert res["pending"] == tr.inp and res["outputs"] == tr.out


def _params(case):
    fri = case["fri"]
    return dict(log_blowup=case["log_blowup"], log_final_poly_len=fri["log_final_poly_len"],
                max_log_arity=fri["max_log_arity"], num_queries=case["num_queries"],
                commit_proof_of_work_bits=fri["commit_pow_bits"], query_proof_of_work_bits=fri["query_pow_bits"])


def reduced_openings(gpu_ctx, case):
    """TwoAdicFriPcs::open up to prove_fri for a golden case, on the GPU: the
    transcript (oracle) after zeta, alpha and the opened values, and the
    bit-reversed reduced openings per LDE height (device buffers)."""
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
    for b in keep:
        b.free()
    return tr, qs


def test_fri_prove_on_device_vs_reference(gpu_ctx, golden):
    """p3g_fri_prove -- every round, the transcript and the query openings on
    the device -- against the reference's proofs: roots, final polynomial,
    query proof-of-work witness and every query's siblings and Merkle path."""
    for case in golden["pcs_open"]:
        tr, qs = reduced_openings(gpu_ctx, case)
        keep = []
        heights = sorted(qs, reverse=True)
        before = tr.copy()
        res = gpu_ctx.fri_prove_device([(qs[h].ptr, h) for h in heights], _params(case), tr.state, tr.inp, tr.out)
        assert res["commits"].tolist() == case["commits"]
        assert res["final_poly"].tolist() == case["final_poly"]
        assert res["query_witness"] == case["fri"]["query_pow_witness"]
        vectors = [qs[h].download(np.uint32, (1 << h, 4)) for h in heights]
        roots, final, w, idx, openings = _oracle_fri(case, before, vectors)
        assert openings == case["query_openings"]
        _check_fri_result(res, case, roots, final, w, idx, openings, before)
        for b in keep + list(qs.values()):
            b.free()


@pytest.mark.parametrize("heights,max_la,log_fpl,pows,nq", [
    ([12, 10, 9, 5], 3, 2, (6, 10), 20),   # arities 2/4/8, mix-ins, proofs of work in every round
    ([14], 2, 0, (0, 12), 7),
    ([9, 8, 7, 6, 5, 4], 1, 1, (3, 0), 1),
    ([11, 6], 3, 3, (0, 0), 33),
])
def test_fri_prove_on_device_vs_oracle(gpu_ctx, heights, max_la, log_fpl, pows, nq):
    rng = np.random.default_rng(sum(heights) + nq)
    vectors = [rng.integers(0, O.BB_P, size=(1 << h, 4), dtype=np.uint32) for h in heights]
    bufs = [gpu_ctx.to_device(v) for v in vectors]
    tr = O.Transcript(O.bb16_params())
    for v in rng.integers(0, O.BB_P, size=int(rng.integers(0, 20))):
        tr.observe(int(v))
    case = {"log_blowup": 1, "num_queries": nq,
            "fri": {"log_final_poly_len": log_fpl, "max_log_arity": max_la, "commit_pow_bits": pows[0],
                    "query_pow_bits": pows[1]}}
    before = tr.copy()
    res = gpu_ctx.fri_prove_device([(b.ptr, h) for b, h in zip(bufs, heights)], _params(case), tr.state, tr.inp,
                                   tr.out)
    roots, final, w, idx, openings = _oracle_fri(case, before, vectors)
    _check_fri_result(res, case, roots, final, w, idx, openings, before)
    for b, v in zip(bufs, vectors):  # inputs untouched
        assert np.array_equal(b.download(np.uint32, v.shape), v)
        b.free()


def test_fri_prove_rejects_bad_arguments(gpu_ctx):
    d = gpu_ctx.to_device(np.zeros((1 << 6, 4), np.uint32))
    st = np.zeros(16, np.uint32)
    base = dict(log_blowup=1, log_final_poly_len=0, max_log_arity=1, num_queries=2, commit_proof_of_work_bits=0,
                query_proof_of_work_bits=0)
    for bad, status in ((dict(max_log_arity=4), 5), (dict(max_log_arity=0), 1), (dict(log_blowup=6), 1),
                        (dict(query_proof_of_work_bits=25), 1)):
        with pytest.raises(P.P3GError) as e:
            gpu_ctx.fri_prove_device([(d.ptr, 6)], {**base, **bad}, st, [], [])
        assert e.value.status == status, bad
    with pytest.raises(P.P3GError) as e:  # heights must decrease
        gpu_ctx.fri_prove_device([(d.ptr, 6), (d.ptr, 6)], base, st, [], [])
    assert e.value.status == 1
    d.free()
