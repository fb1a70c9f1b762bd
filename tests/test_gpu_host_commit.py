"""p3g_commit_traces_host: traces in host memory, copied in column chunks on a
second stream while earlier chunks' LDEs and row hashes run (a large first
trace starts with narrow chunks; each chunk's row hashes resume the sponge
state of the chunks before it where the row length so far is a multiple of the
rate).  The commitment and every opening must equal p3g_commit_traces on the
same traces (and the oracle's), whatever the chunking."""
import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu


def _shapes_bb():
    return [(12, 300), (12, 128), (10, 7), (12, 129), (9, 256)]


def test_host_commit_matches_device_commit_and_oracle(gpu_ctx):
    rng = np.random.default_rng(61)
    traces = [rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32) for lh, w in _shapes_bb()]
    bufs = [gpu_ctx.to_device(t) for t in traces]
    dev = gpu_ctx.commit_traces_device(P.BABYBEAR, [(b.ptr, t.shape[0].bit_length() - 1, t.shape[1], 1, 31)
                                                    for b, t in zip(bufs, traces)], 1)
    cap = np.zeros((2, 8), np.uint32)
    host = gpu_ctx.commit_traces_host(P.BABYBEAR, [(t.ctypes.data, t.shape[0].bit_length() - 1, t.shape[1], 1, 31)
                                                   for t in traces], 1, cap_out=cap)
    want = O.mmcs_commit(O.bb16_params(), [O.bb_coset_lde(t, 1, 31, True) for t in traces], 1)
    got_h, got_d = host.layers(), dev.layers()
    assert len(got_h) == len(want)
    for a, b, c in zip(got_h, got_d, want):
        assert np.array_equal(a, c)
        assert np.array_equal(b, c)
    assert np.array_equal(cap, want[-1])
    # openings: same concatenated rows and the same sibling paths
    idx = np.array([0, 1, 777, 4095, 8191], dtype=np.uint64)
    total_w = sum(t.shape[1] for t in traces)
    rows_h, proof_h = host.open_batch(idx, total_w)
    rows_d, proof_d = dev.open_batch(idx, total_w)
    assert np.array_equal(rows_h, rows_d)
    assert np.array_equal(proof_h, proof_d)
    host.free()
    dev.free()
    for b in bufs:
        b.free()


def test_host_commit_goldilocks_and_zero_width(gpu_ctx):
    rng = np.random.default_rng(62)
    shapes = [(10, 100), (10, 0), (8, 64), (10, 3)]
    traces = [rng.integers(0, O.GL_P, size=(1 << lh, w), dtype=np.uint64) for lh, w in shapes]
    host = gpu_ctx.commit_traces_host(P.GOLDILOCKS, [(t.ctypes.data if t.size else 0, lh, w, 2, 7)
                                                     for t, (lh, w) in zip(traces, shapes)], 0)
    want = O.mmcs_commit(O.gl8_params(), [O.gl_coset_lde(t, 2, 7, True) if t.size else
                                          np.zeros((1 << (lh + 2), 0), np.uint64)
                                          for t, (lh, w) in zip(traces, shapes)], 0)
    for a, c in zip(host.layers(), want):
        assert np.array_equal(a, c)
    host.free()


def test_host_commit_rejects_bad_arguments(gpu_ctx):
    with pytest.raises(P.P3GError):
        gpu_ctx.commit_traces_host(P.BABYBEAR, [(0, 4, 4, 1, 31)], 0)  # null trace
    t = np.zeros((16, 4), np.uint32)
    with pytest.raises(P.P3GError):
        gpu_ctx.commit_traces_host(P.BABYBEAR, [(t.ctypes.data, 4, 4, 1, P.BB_P)], 0)  # shift not canonical


@pytest.mark.parametrize("field,shapes", [
    # first trace 32+32+64+128+44 columns; then equal-height traces after a
    # row length that is not a multiple of the rate (no cut), then a cut again
    (P.BABYBEAR, [(14, 300), (14, 5), (14, 3), (14, 64), (12, 9)]),
    (P.BABYBEAR, [(15, 256)]),
    (P.BABYBEAR, [(14, 20), (15, 8)]),  # narrow first trace, shorter than a chunk
    (P.GOLDILOCKS, [(14, 100), (14, 3), (13, 8)]),
])
def test_host_commit_staged_row_hashes(gpu_ctx, field, shapes):
    rng = np.random.default_rng(63 + len(shapes))
    p = O.BB_P if field == P.BABYBEAR else O.GL_P
    dt = np.uint32 if field == P.BABYBEAR else np.uint64
    shift = 31 if field == P.BABYBEAR else 7
    traces = [rng.integers(0, p, size=(1 << lh, w), dtype=dt) for lh, w in shapes]
    bufs = [gpu_ctx.to_device(t) for t in traces]
    dev = gpu_ctx.commit_traces_device(field, [(b.ptr, lh, w, 1, shift) for b, (lh, w) in zip(bufs, shapes)], 0)
    host = gpu_ctx.commit_traces_host(field, [(t.ctypes.data, lh, w, 1, shift) for t, (lh, w) in zip(traces, shapes)], 0)
    for a, b in zip(host.layers(), dev.layers()):
        assert np.array_equal(a, b)
    if field == P.GOLDILOCKS:
        want = O.mmcs_commit(O.gl8_params(), [O.gl_coset_lde(t, 1, 7, True) for t in traces], 0)
        assert np.array_equal(host.layers()[-1], want[-1])
    host.free()
    dev.free()
    for b in bufs:
        b.free()


def test_commit_above_three_pass_height(gpu_ctx):
    """A 2^22-row trace (LDE through the split transform) next to a short one:
    the host-trace commit equals the device commit, and the device commit's
    leaf digests equal the oracle's sponge over the oracle's LDE rows."""
    rng = np.random.default_rng(22)
    shapes = [(22, 9), (12, 8)]
    traces = [rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32) for lh, w in shapes]
    bufs = [gpu_ctx.to_device(t) for t in traces]
    dev = gpu_ctx.commit_traces_device(P.BABYBEAR, [(b.ptr, lh, w, 1, 31) for b, (lh, w) in zip(bufs, shapes)], 0)
    host = gpu_ctx.commit_traces_host(P.BABYBEAR, [(t.ctypes.data, lh, w, 1, 31)
                                                   for t, (lh, w) in zip(traces, shapes)], 0)
    for a, b in zip(host.layers(), dev.layers()):
        assert np.array_equal(a, b)
    lde = O.bb_coset_lde(traces[0], 1, 31, True, nthreads=8)
    leaves = dev.layers()[0]
    p = O.bb16_params()
    for r in (0, 1, 12345, (1 << 23) - 1):
        assert np.array_equal(leaves[r], O.hash_iter(p, lde[r])), r
    host.free()
    dev.free()
    for b in bufs:
        b.free()
