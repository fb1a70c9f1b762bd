"""Batched commit captured as one CUDA graph (p3g_plan_*): every digest layer
and the fold against the oracle, replays after refilling the trace buffers,
the autotuned stream count, and launch accounting.  Bit-exact."""
import os

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _batch(rng, n, lo=3, hi=11, wmax=40):
    traces = []
    for i in range(n):
        lh = int(rng.integers(lo, hi + 1))
        w = int(rng.integers(1, wmax))
        traces.append(rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32))
    # a repeated shape makes a multi-matrix height group
    traces.append(rng.integers(0, O.BB_P, size=traces[0].shape, dtype=np.uint32))
    return traces


def _oracle_commit(traces, cap=0):
    ldes = [O.bb_coset_lde(t, 1, 31, True, nthreads=NT) for t in traces]
    return O.mmcs_commit(O.bb16_params(), ldes, cap, nthreads=NT), ldes


@pytest.mark.parametrize("n_streams", [1, 4])
def test_plan_batched_commit_and_fold(gpu_ctx, n_streams):
    rng = np.random.default_rng(40 + n_streams)
    traces = _batch(rng, 9)
    bufs = [gpu_ctx.to_device(t) for t in traces]
    lh_fold = 12
    fv = rng.integers(0, O.BB_P, size=(1 << lh_fold, 4), dtype=np.uint32)
    beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
    d_fin = gpu_ctx.to_device(fv)
    d_fout = gpu_ctx.alloc((1 << (lh_fold - 1)) * 16)
    plan = P.Plan(gpu_ctx, P.BABYBEAR, [(b.ptr, t.shape[0].bit_length() - 1, t.shape[1], 1, 31)
                                        for b, t in zip(bufs, traces)],
                  cap_height=1, fold=(d_fin.ptr, d_fout.ptr, lh_fold, 1, beta), n_streams=n_streams)
    assert plan.n_streams == n_streams
    plan.launch()
    gpu_ctx.sync()
    want, ldes = _oracle_commit(traces, 1)
    got = plan.tree.layers()
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    assert np.array_equal(d_fout.download(np.uint32, ((1 << (lh_fold - 1)), 4)),
                          O.fold_matrix_bb4(fv, lh_fold, 1, beta))
    # replay with new trace contents in the same buffers
    traces2 = [rng.integers(0, O.BB_P, size=t.shape, dtype=np.uint32) for t in traces]
    for b, t in zip(bufs, traces2):
        b.upload(t)
    gpu_ctx.sync()
    plan.launch()
    gpu_ctx.sync()
    want2, _ = _oracle_commit(traces2, 1)
    assert np.array_equal(plan.tree.layers()[-1], want2[-1])
    plan.destroy()
    for b in bufs + [d_fin, d_fout]:
        b.free()


def test_plan_autotuned_streams_and_launch_count(gpu_ctx, tmp_path, monkeypatch):
    monkeypatch.setenv("P3G_TUNE_CACHE", str(tmp_path / "tune.json"))
    rng = np.random.default_rng(7)
    traces = _batch(rng, 5, 5, 12, 20)
    bufs = [gpu_ctx.to_device(t) for t in traces]
    plan = P.Plan(gpu_ctx, P.BABYBEAR, [(b.ptr, t.shape[0].bit_length() - 1, t.shape[1], 1, 31)
                                        for b, t in zip(bufs, traces)], n_streams=0)
    assert plan.n_streams in (1, 2, 4, 8)
    assert plan.kernels_per_launch > 0
    before = P.kernel_launches()
    plan.launch()
    plan.launch()
    gpu_ctx.sync()
    assert P.kernel_launches() - before == 2 * plan.kernels_per_launch
    want, _ = _oracle_commit(traces, 0)
    assert np.array_equal(plan.tree.layers()[-1], want[-1])
    with pytest.raises(P.P3GError):
        plan.tree.free()
    plan.destroy()
    for b in bufs:
        b.free()


def test_plan_goldilocks(gpu_ctx):
    rng = np.random.default_rng(8)
    traces = [(rng.integers(0, 2**63, size=(1 << lh, w), dtype=np.uint64) * 2 % np.uint64(O.GL_P)).astype(np.uint64)
              for lh, w in ((6, 5), (9, 3), (6, 2))]
    bufs = [gpu_ctx.to_device(t) for t in traces]
    plan = P.Plan(gpu_ctx, P.GOLDILOCKS, [(b.ptr, t.shape[0].bit_length() - 1, t.shape[1], 2, 7)
                                          for b, t in zip(bufs, traces)], n_streams=2)
    plan.launch()
    gpu_ctx.sync()
    ldes = [O.gl_coset_lde(t, 2, 7, True) for t in traces]
    want = O.mmcs_commit(O.gl8_params(), ldes, 0)
    for g, w in zip(plan.tree.layers(), want):
        assert np.array_equal(g, w)
    plan.destroy()
    for b in bufs:
        b.free()


@pytest.mark.parametrize("n_streams", [1, 3])
def test_host_input_plan_copies_and_commits(gpu_ctx, n_streams):
    """p3g_plan_commit_host: traces and the fold input in pinned host memory,
    copied in by the graph on every launch; the same tree and fold as the
    oracle, and again after the host buffers are refilled."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(60 + n_streams)
    traces = _batch(rng, 7, 3, 13, 30)
    traces.append(np.zeros((1 << 5, 0), np.uint32))  # a zero-width trace: nothing to copy
    pinned = []
    for t in traces:
        pt = torch.empty(t.size, dtype=torch.int32, pin_memory=True)
        pt.numpy().view(np.uint32)[:] = t.reshape(-1)
        pinned.append(pt)
    lh_fold = 11
    fv = rng.integers(0, O.BB_P, size=(1 << lh_fold, 4), dtype=np.uint32)
    pf = torch.empty(fv.size, dtype=torch.int32, pin_memory=True)
    pf.numpy().view(np.uint32)[:] = fv.reshape(-1)
    beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
    d_fout = gpu_ctx.alloc((1 << (lh_fold - 1)) * 16)
    plan = P.Plan(gpu_ctx, P.BABYBEAR, [(p.data_ptr() if t.size else 0, t.shape[0].bit_length() - 1, t.shape[1], 1, 31)
                                        for p, t in zip(pinned, traces)],
                  fold=(pf.data_ptr(), d_fout.ptr, lh_fold, 1, beta), n_streams=n_streams, host=True)
    for rep in range(2):
        if rep == 1:  # new contents in the same host buffers
            traces = [rng.integers(0, O.BB_P, size=t.shape, dtype=np.uint32) for t in traces]
            for p, t in zip(pinned, traces):
                p.numpy().view(np.uint32)[:] = t.reshape(-1)
        plan.launch()
        gpu_ctx.sync()
        want, _ = _oracle_commit(traces, 0)
        got = plan.tree.layers()
        assert len(got) == len(want)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)
        assert np.array_equal(d_fout.download(np.uint32, ((1 << (lh_fold - 1)), 4)),
                              O.fold_matrix_bb4(fv, lh_fold, 1, beta))
    plan.destroy()
    d_fout.free()


def test_host_input_plan_rejects_pageable_memory(gpu_ctx):
    t = np.ones((1 << 6, 8), np.uint32)  # numpy memory is pageable
    with pytest.raises(P.P3GError) as e:
        P.Plan(gpu_ctx, P.BABYBEAR, [(t.ctypes.data, 6, 8, 1, 31)], n_streams=1, host=True)
    assert e.value.status == 1


def test_plan_batches_equal_shapes_into_one_launch_per_pass(gpu_ctx):
    """Eight traces of one shape (three-pass height) and four of another
    (single-kernel height) in a plan with fixed streams: the LDEs run as one
    launch per pass for each shape group, so adding traces of an existing
    shape adds no kernels; the tree equals the oracle's."""
    rng = np.random.default_rng(17)
    shapes = [(12, int(rng.integers(5, 70))) for _ in range(8)] + [(9, int(rng.integers(1, 30))) for _ in range(4)]
    traces = [rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32) for lh, w in shapes]
    bufs = [gpu_ctx.to_device(t) for t in traces]
    kernels = []
    for n in (len(traces), 2):
        sel = [0, 8] if n == 2 else list(range(n))
        plan = P.Plan(gpu_ctx, P.BABYBEAR, [(bufs[i].ptr, shapes[i][0], shapes[i][1], 1, 31) for i in sel],
                      n_streams=1)
        plan.launch()
        gpu_ctx.sync()
        kernels.append(plan.kernels_per_launch)
        if n == len(traces):
            want, _ = _oracle_commit(traces, 0)
            got = plan.tree.layers()
            for g, w in zip(got, want):
                assert np.array_equal(g, w)
        plan.destroy()
    # the same LDE launches for 12 traces as for one trace of each shape; only
    # the row-hash and tree kernels may differ
    assert kernels[0] <= kernels[1] + 2, kernels
    for b in bufs:
        b.free()
