"""Full-size workloads against the oracle: config 1 (2^20 x 256) and config 3
(the bench's own 64 traces and quotient) tree layer by tree layer and fold
value by fold value, the Goldilocks 2^18 x 128 workload whole; and through
size-independent properties: every Merkle opening the GPU tree produces
verifies under the oracle's restatement of MerkleTreeMmcs::verify_batch
(merkle_tree_mmcs.hpp:168-254) against the GPU's root."""
import os

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _verify_openings(tree, heights, widths, n_queries, seed):
    p = O.bb16_params()
    sizes, _ = tree.info()
    layers = tree.layers()
    cap = layers[-1]
    max_h = sizes[0]
    idx = np.random.default_rng(seed).integers(0, max_h, size=n_queries, dtype=np.uint64)
    rows, proof = tree.open_batch(idx, sum(widths))
    for q, index in enumerate(idx.tolist()):
        opened, off = [], 0
        for w in widths:
            opened.append(rows[q, off:off + w])
            off += w
        assert O.mmcs_verify_batch(p, cap, heights, widths, index, opened, list(proof[q]))
        # a flipped element must fail
        bad = [o.copy() for o in opened]
        bad[0][0] = (int(bad[0][0]) + 1) % O.BB_P
        assert not O.mmcs_verify_batch(p, cap, heights, widths, index, bad, list(proof[q]))


def test_config1_commit_every_layer_matches_oracle(gpu_ctx):
    """Config 1 (2^20 x 256, log_blowup 1): every digest layer of the GPU tree,
    leaves to root, equals the oracle's tree over the oracle's LDE, and
    openings verify under the oracle's verify_batch."""
    rng = np.random.default_rng(21)
    t = rng.integers(0, O.BB_P, size=(1 << 20, 256), dtype=np.uint32)
    d = gpu_ctx.to_device(t)
    tree = gpu_ctx.commit_traces_device(P.BABYBEAR, [(d.ptr, 20, 256, 1, 31)], 0)
    _verify_openings(tree, [1 << 21], [256], 12, 1)
    lde = O.bb_coset_lde(t, 1, 31, True, nthreads=NT)
    want = O.mmcs_commit(O.bb16_params(), [lde], 0, nthreads=NT)
    got = tree.layers()
    assert len(got) == len(want) == 22
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    tree.free()
    d.free()


def test_config3_bench_workload_root_and_fold_match_oracle(gpu_ctx):
    """Config 3 exactly as the bench runs it (bench.config3_inputs: the same
    seeded 64 traces, 2^19 quotient and beta; the autotuned plan): every digest
    layer of the one mixed-height tree and the whole fold output equal the
    oracle's."""
    import bench
    shapes, traces, fold_in, beta = bench.config3_inputs(3)
    bufs = [gpu_ctx.to_device(t) for t in traces]
    d_fin = gpu_ctx.to_device(fold_in)
    d_fout = gpu_ctx.alloc((1 << 18) * 16)
    plan = P.Plan(gpu_ctx, P.BABYBEAR, [(b.ptr, lh, w, 1, 31) for b, (lh, w) in zip(bufs, shapes)], 0,
                  fold=(d_fin.ptr, d_fout.ptr, 19, 1, beta), n_streams=0)
    plan.launch()
    gpu_ctx.sync()
    got = plan.tree.layers()
    fold = d_fout.download(np.uint32, (1 << 18, 4))
    plan.destroy()
    for b in bufs + [d_fin, d_fout]:
        b.free()
    assert np.array_equal(fold, O.fold_matrix_bb4(fold_in, 19, 1, beta, nthreads=NT))
    ldes = [O.bb_coset_lde(t, 1, 31, True, nthreads=NT) for t in traces]
    want = O.mmcs_commit(O.bb16_params(), ldes, 0, nthreads=NT)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_config1_host_commit_equals_device_commit(gpu_ctx):
    """The end-to-end call (pinned host trace, narrow first chunks, row hashes
    resumed across chunks) gives every digest layer of the device commit."""
    rng = np.random.default_rng(22)
    t = rng.integers(0, O.BB_P, size=(1 << 20, 256), dtype=np.uint32)
    d = gpu_ctx.to_device(t)
    dev = gpu_ctx.commit_traces_device(P.BABYBEAR, [(d.ptr, 20, 256, 1, 31)], 0)
    host = gpu_ctx.commit_traces_host(P.BABYBEAR, [(t.ctypes.data, 20, 256, 1, 31)], 0)
    for a, b in zip(host.layers(), dev.layers()):
        assert np.array_equal(a, b)
    _verify_openings(host, [1 << 21] * 4, [32, 32, 64, 128], 6, 2)  # leaf matrices = the column chunks
    host.free()
    dev.free()
    d.free()


def test_config3_batched_plan_openings_verify(gpu_ctx):
    rng = np.random.default_rng(3)
    shapes = [(int(rng.integers(12, 19)), int(rng.integers(8, 513))) for _ in range(64)]
    bufs, small = [], {}
    for i, (lh, w) in enumerate(shapes):
        t = np.random.default_rng(100 + i).integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32)
        bufs.append(gpu_ctx.to_device(t))
        if lh <= 13 and len(small) < 6:
            small[i] = t
    plan = P.Plan(gpu_ctx, P.BABYBEAR, [(b.ptr, lh, w, 1, 31) for b, (lh, w) in zip(bufs, shapes)], n_streams=4)
    plan.launch()
    gpu_ctx.sync()
    heights = [1 << (lh + 1) for lh, _ in shapes]
    widths = [w for _, w in shapes]
    _verify_openings(plan.tree, heights, widths, 16, 2)
    for i, t in small.items():
        lde = O.bb_coset_lde(t, 1, 31, True, nthreads=NT)
        got = np.empty_like(lde)
        P.check(P.load().p3g_memcpy_d2h(gpu_ctx.handle, got.ctypes.data, plan.tree.leaf_ptr(i), got.nbytes, None))
        assert np.array_equal(got, lde)
    plan.destroy()
    for b in bufs:
        b.free()


def test_config2_goldilocks_full_size_matches_oracle(gpu_ctx):
    """Goldilocks 2^18 x 128, log_blowup 2, shift 7: the full 2^20 x 128 LDE and
    every digest layer of the Poseidon2-8 tree, element for element."""
    t = np.random.default_rng(22).integers(0, O.GL_P, size=(1 << 18, 128), dtype=np.uint64)
    d = gpu_ctx.to_device(t)
    tree = gpu_ctx.commit_traces_device(P.GOLDILOCKS, [(d.ptr, 18, 128, 2, 7)], 0)
    lde = O.gl_coset_lde(t, 2, 7, True, nthreads=NT)
    got = np.empty_like(lde)
    P.check(P.load().p3g_memcpy_d2h(gpu_ctx.handle, got.ctypes.data, tree.leaf_ptr(0), got.nbytes, None))
    assert np.array_equal(got, lde)
    want = O.mmcs_commit(O.gl8_params(), [lde], 0, nthreads=NT)
    layers = tree.layers()
    assert len(layers) == len(want)
    for g, w in zip(layers, want):
        assert np.array_equal(g, w)
    tree.free()
    d.free()
