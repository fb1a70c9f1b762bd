"""The continuous-batching serving loop (p3g_server_*): every request's root,
whole fold output and openings are identical when it runs alone and when it
runs mixed with others on several slots, and match the oracle; resident data
serves openings and fold reads until released; host-side failure paths
return statuses."""
import time

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu


def _requests(seed, n):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        lh = int(rng.integers(3, 13))
        w = int(rng.integers(4, 40))
        lb = int(rng.integers(1, 4))
        t = rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32)
        beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
        reqs.append((i + 1, t, lh, w, lb, 31, beta))
    return reqs


def _drain(server, n, timeout=60.0):
    out, t0 = {}, time.time()
    while len(out) < n:
        for r in server.poll():
            out[r.id] = r
        assert time.time() - t0 < timeout, "server did not finish in time"
        time.sleep(0.001)
    return out


def _run(ctx, reqs, slots, together):
    server = P.Server(ctx, max_slots=slots)
    res = {}
    try:
        if together:
            for rid, t, lh, w, lb, sh, beta in reqs:
                server.submit(rid, t.ctypes.data, lh, w, lb, sh, beta)
            res = _drain(server, len(reqs))
        else:
            for rid, t, lh, w, lb, sh, beta in reqs:
                server.submit(rid, t.ctypes.data, lh, w, lb, sh, beta)
                res.update(_drain(server, 1))
        opens = {}
        for rid, t, lh, w, lb, sh, beta in reqs:
            H = 1 << (lh + lb)
            idx = np.array([0, H - 1, H // 3], np.uint64)
            opens[rid] = server.open(rid, idx, w, lh + lb + 1) + (server.read_fold(rid, H),)
            server.release(rid)
        assert server.pending()[2] == 0
    finally:
        server.close()
    return res, opens


def test_alone_and_mixed_results_identical_and_match_oracle(gpu_ctx):
    reqs = _requests(5, 24)
    alone, open_a = _run(gpu_ctx, reqs, 1, False)
    mixed, open_m = _run(gpu_ctx, reqs, 6, True)
    p = O.bb16_params()
    for rid, t, lh, w, lb, sh, beta in reqs:
        a, m = alone[rid], mixed[rid]
        assert a.status == 0 and m.status == 0
        assert list(a.root) == list(m.root) and list(a.fold_head) == list(m.fold_head)
        for k in range(3):  # opened rows, Merkle paths, the whole fold output
            assert np.array_equal(open_a[rid][k], open_m[rid][k])
        assert m.t_submit_ns <= m.t_admit_ns <= m.t_done_ns
    for rid, t, lh, w, lb, sh, beta in reqs:
        lde = O.bb_coset_lde(t, lb, sh, True)
        layers = O.mmcs_commit(p, [lde], 0)
        assert list(mixed[rid].root) == layers[-1][0].tolist()
        fold = O.fold_matrix_bb4(np.ascontiguousarray(lde[:, :4]), lh + lb, 1, beta)
        assert list(mixed[rid].fold_head) == fold[0].tolist()
        assert np.array_equal(open_m[rid][2], fold)
        rows, proof, _ = open_m[rid]
        H = 1 << (lh + lb)
        for q, index in enumerate([0, H - 1, H // 3]):
            assert np.array_equal(rows[q], lde[index])
            assert O.mmcs_verify_batch(p, layers[-1], [H], [w], index, [rows[q]], list(proof[q]))


def test_budget_too_small_is_reported_not_hung(gpu_ctx):
    server = P.Server(gpu_ctx, max_slots=2, mem_budget=1 << 20)
    try:
        t = np.ones((1 << 12, 16), np.uint32)
        server.submit(7, t.ctypes.data, 12, 16, 1, 31, [1, 2, 3, 4])
        res = _drain(server, 1, timeout=10)
        assert res[7].status == 2  # P3G_ENOMEM
    finally:
        server.close()


def test_bad_requests_rejected_on_the_host(gpu_ctx):
    server = P.Server(gpu_ctx, max_slots=1)
    try:
        t = np.ones((16, 8), np.uint32)
        with pytest.raises(P.P3GError):
            server.submit(1, t.ctypes.data, 4, 3, 1, 31, [0, 0, 0, 0])   # width < 4
        with pytest.raises(P.P3GError):
            server.submit(2, t.ctypes.data, 4, 8, 1, 0, [0, 0, 0, 0])    # zero shift
        with pytest.raises(P.P3GError):
            server.open(99, [0], 8, 2)                                   # unknown id
        with pytest.raises(P.P3GError):
            server.read_fold(99, 16)                                     # unknown id
    finally:
        server.close()


def test_destroy_with_work_in_flight(gpu_ctx):
    server = P.Server(gpu_ctx, max_slots=2)
    t = np.ones((1 << 14, 64), np.uint32)
    for i in range(6):
        server.submit(i + 1, t.ctypes.data, 14, 64, 1, 31, [1, 2, 3, 4])
    server.close()  # must return: queued requests dropped, in-flight ones drained
