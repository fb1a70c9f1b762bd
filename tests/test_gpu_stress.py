"""Randomised consistency runs over many shapes: the host-trace commit (column
chunks, staged row hashes, the context's copy stream reused call after call)
against the device commit, and the device FRI prover against itself (the same
inputs and transcript give the same proof).  Seeded; a few seconds."""
import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu


def test_host_commit_matches_device_commit_over_random_shapes(gpu_ctx):
    rng = np.random.default_rng(2024)
    for it in range(96):
        field = P.BABYBEAR if it % 4 else P.GOLDILOCKS
        p, dt, shift = (O.BB_P, np.uint32, 31) if field == P.BABYBEAR else (O.GL_P, np.uint64, 7)
        n = int(rng.integers(1, 6))
        shapes = [(int(rng.integers(10, 17)), int(rng.integers(1, 300))) for _ in range(n)]
        lb = int(rng.integers(1, 3))
        traces = [rng.integers(0, p, size=(1 << lh, w), dtype=dt) for lh, w in shapes]
        bufs = [gpu_ctx.to_device(t) for t in traces]
        cap = int(rng.integers(0, 3))
        dev = gpu_ctx.commit_traces_device(field, [(b.ptr, lh, w, lb, shift) for b, (lh, w) in zip(bufs, shapes)], cap)
        host = gpu_ctx.commit_traces_host(field, [(t.ctypes.data, lh, w, lb, shift)
                                                  for t, (lh, w) in zip(traces, shapes)], cap)
        for a, b in zip(host.layers(), dev.layers()):
            assert np.array_equal(a, b), (it, shapes, lb, cap)
        host.free()
        dev.free()
        for b in bufs:
            b.free()


def test_fri_prove_is_deterministic(gpu_ctx):
    rng = np.random.default_rng(7)
    heights = [16, 13, 9]
    bufs = [gpu_ctx.to_device(rng.integers(0, O.BB_P, size=(1 << h, 4), dtype=np.uint32)) for h in heights]
    prm = dict(log_blowup=1, log_final_poly_len=2, max_log_arity=3, num_queries=40, commit_proof_of_work_bits=5,
               query_proof_of_work_bits=12)
    st = rng.integers(0, O.BB_P, size=16, dtype=np.uint32)
    runs = [gpu_ctx.fri_prove_device([(b.ptr, h) for b, h in zip(bufs, heights)], prm, st, [3, 4], [])
            for _ in range(5)]
    for r in runs[1:]:
        for k in ("commits", "commit_witnesses", "final_poly", "query_indices", "state"):
            assert np.array_equal(r[k], runs[0][k]), k
        assert r["query_witness"] == runs[0]["query_witness"]
        for a, b in zip(r["rows"] + r["paths"], runs[0]["rows"] + runs[0]["paths"]):
            assert np.array_equal(a, b)
    for b in bufs:
        b.free()
