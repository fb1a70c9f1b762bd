"""GPU parity of Poseidon2, the mixed-height MerkleTreeMmcs, the flat
commit_matrix MMCS, openings and the LDE+commit pipeline, against golden
vectors from the reference and the oracle.  Bit-exact."""
import os

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 1


def _mats(kind, shapes, seed):
    out = []
    for i, s in enumerate(shapes):
        h, w = (int(v) for v in s.split("x"))
        out.append(O.gl_random_matrix(h, w, seed + i) if kind == "gl8" else O.bb_random_matrix(h, w, seed + i))
    return out


def _use(ctx, kind):
    if kind == "bb16zero":
        ctx.set_poseidon2(P.BABYBEAR, 16, 8, 22, 7, np.zeros(64), np.zeros(64), np.zeros(22))
    else:
        ctx.set_default_poseidon2()


def test_permutation_golden(gpu_ctx, golden):
    for case in golden["perm"]:
        kind = case["kind"]
        _use(gpu_ctx, "bb16zero" if kind.startswith("bb16zero") else kind)
        field = P.GOLDILOCKS if kind == "gl8" else P.BABYBEAR
        dt = np.uint64 if field == P.GOLDILOCKS else np.uint32
        got = gpu_ctx.permute(field, np.array(case["inputs"], dtype=dt))
        assert [[int(x) for x in r] for r in got] == case["outputs"]
    gpu_ctx.set_default_poseidon2()


def test_permutation_many_vs_oracle(gpu_ctx):
    rng = np.random.default_rng(1)
    s = rng.integers(0, O.BB_P, size=(1000, 16), dtype=np.uint32)
    s[0] = 0
    s[1] = O.BB_P - 1
    got = gpu_ctx.permute(P.BABYBEAR, s)
    p = O.bb16_params()
    for i in (0, 1, 2, 500, 999):
        assert got[i].tolist() == O.permute(p, s[i]).tolist()
    g = (rng.integers(0, 2**63, size=(300, 8), dtype=np.uint64) * 2) % np.uint64(O.GL_P)
    got = gpu_ctx.permute(P.GOLDILOCKS, g.astype(np.uint64))
    pg = O.gl8_params()
    for i in (0, 7, 299):
        assert [int(x) for x in got[i]] == [int(x) for x in O.permute(pg, g[i])]


def test_mmcs_golden(gpu_ctx, golden):
    for case in golden["mmcs"]:
        _use(gpu_ctx, case["kind"])
        mats = _mats(case["kind"], case["shapes"], case["seed"])
        tree, bufs = gpu_ctx.mmcs_commit(mats, case["cap_height"])
        layers = tree.layers()
        assert [len(l) for l in layers] == case["sizes"], case["shapes"]
        for got, want in zip(layers, case["layers"]):
            assert [[int(x) for x in d] for d in got] == want, case["shapes"]
        tree.free()
        for b in bufs:
            b.free()
    gpu_ctx.set_default_poseidon2()


def test_commit_matrix_golden(gpu_ctx, golden):
    for case in golden["commit_matrix"]:
        m = O.bb_random_matrix(case["h"], case["w"], case["seed"])
        tree, buf = gpu_ctx.commit_matrix(m)
        layers = tree.layers()
        assert [len(l) for l in layers] == case["sizes"]
        for got, want in zip(layers, case["layers"]):
            assert got.tolist() == want
        tree.free()
        buf.free()


@pytest.mark.parametrize("seed", range(6))
def test_mmcs_random_mixed_heights_vs_oracle(gpu_ctx, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 9))
    mats = []
    for _ in range(n):
        lh = int(rng.integers(0, 11))
        w = int(rng.integers(0, 70)) if seed % 2 else int(rng.integers(1, 40))
        mats.append(rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32))
    if all(m.shape[1] == 0 for m in mats):
        mats[0] = np.ones((mats[0].shape[0], 3), np.uint32)
    cap = int(rng.integers(0, 3))
    tree, bufs = gpu_ctx.mmcs_commit(mats, cap)
    want = O.mmcs_commit(O.bb16_params(), mats, cap, nthreads=NT)
    got = tree.layers()
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    # openings: rows and sibling paths as merkle_tree_mmcs.hpp:120-152
    max_h = max(m.shape[0] for m in mats)
    idx = rng.integers(0, max_h, size=5, dtype=np.uint64)
    rows, proof = tree.open_batch(idx, sum(m.shape[1] for m in mats))
    for q, index in enumerate(idx.tolist()):
        off = 0
        for m in mats:
            r = index // (max_h // m.shape[0])
            assert np.array_equal(rows[q, off:off + m.shape[1]], m[r])
            off += m.shape[1]
        for l in range(len(want) - 1):
            assert np.array_equal(proof[q, l], want[l][(index >> l) ^ 1])
    tree.free()
    for b in bufs:
        b.free()


def test_mmcs_goldilocks_vs_oracle(gpu_ctx):
    rng = np.random.default_rng(3)
    mats = [(rng.integers(0, 2**63, size=(h, w), dtype=np.uint64) * 2 % np.uint64(O.GL_P)).astype(np.uint64)
            for h, w in ((256, 13), (64, 4), (256, 5), (8, 1))]
    tree, bufs = gpu_ctx.mmcs_commit(mats, 0)
    want = O.mmcs_commit(O.gl8_params(), mats, 0, nthreads=NT)
    for g, w in zip(tree.layers(), want):
        assert np.array_equal(g, w)
    tree.free()
    for b in bufs:
        b.free()


def test_flat_commit_random_heights(gpu_ctx):
    rng = np.random.default_rng(9)
    for h in (1, 2, 3, 7, 100, 1023, 4097):
        m = rng.integers(0, O.BB_P, size=(h, int(rng.integers(1, 20))), dtype=np.uint32)
        tree, buf = gpu_ctx.commit_matrix(m)
        want = O.commit_matrix(O.bb16_params(), m, nthreads=NT)
        for g, w in zip(tree.layers(), want):
            assert np.array_equal(g, w)
        idx = np.array([0, h - 1, h // 2], np.uint64)
        rows, proof = tree.open_batch(idx, m.shape[1])
        for q, i in enumerate(idx.tolist()):
            assert np.array_equal(rows[q], m[i])
            for l in range(len(want) - 1):
                sib = (i >> l) ^ 1
                exp = want[l][sib] if sib < len(want[l]) else np.zeros(8, np.uint32)
                assert np.array_equal(proof[q, l], exp)
        tree.free()
        buf.free()


def test_commit_pipeline_golden_config0(gpu_ctx, golden):
    """LDE (bit-reversed) + MMCS root, the reference's commit of config 0 and friends."""
    for case in golden["commit"]:
        t = O.bb_random_matrix(1 << case["log_h"], case["w"], case["seed"])
        d = gpu_ctx.to_device(t)
        cap = np.zeros((1 << case["cap_height"], 8), np.uint32)
        tree = gpu_ctx.commit_traces_device(P.BABYBEAR, [(d.ptr, case["log_h"], case["w"], case["log_blowup"],
                                                          case["shift"])], case["cap_height"], cap_out=cap)
        assert cap[: len(case["cap"])].tolist() == case["cap"]
        layers = tree.layers()
        assert [len(l) for l in layers] == case["sizes"]
        import hashlib
        allb = np.concatenate([l.reshape(-1) for l in layers])
        assert hashlib.sha256(allb.tobytes()).hexdigest() == case["layers_sha256"]
        tree.free()
        d.free()


def test_commit_pipeline_batched_vs_oracle(gpu_ctx):
    """Many traces of uneven height and width -> one mixed-height commit."""
    rng = np.random.default_rng(77)
    traces = []
    for _ in range(10):
        lh = int(rng.integers(2, 13))
        w = int(rng.integers(1, 40))
        traces.append(rng.integers(0, O.BB_P, size=(1 << lh, w), dtype=np.uint32))
    bufs = [gpu_ctx.to_device(t) for t in traces]
    tree = gpu_ctx.commit_traces_device(P.BABYBEAR, [(b.ptr, t.shape[0].bit_length() - 1, t.shape[1], 1, 31)
                                                     for b, t in zip(bufs, traces)], 0)
    ldes = [O.bb_coset_lde(t, 1, 31, True) for t in traces]
    want = O.mmcs_commit(O.bb16_params(), ldes, 0, nthreads=NT)
    got = tree.layers()
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    # leaf matrices are the LDEs
    for i, l in enumerate(ldes):
        p = tree.leaf_ptr(i)
        arr = np.empty_like(l)
        P.check(P.load().p3g_memcpy_d2h(gpu_ctx.handle, arr.ctypes.data, p, arr.nbytes, None))
        assert np.array_equal(arr, l)
    tree.free()
    for b in bufs:
        b.free()


@pytest.mark.parametrize("field", ["bb", "gl"])
def test_commit_traces_same_shape_batches_vs_oracle(gpu_ctx, field):
    """Traces sharing (log_h, log_blowup, shift) run as one LDE batch (one
    launch per pass for the whole group, single-kernel and three-pass heights,
    ragged widths, a zero-width trace among them): the same tree as the oracle."""
    rng = np.random.default_rng(91 if field == "bb" else 92)
    fid, p, dt, shift, params = ((P.BABYBEAR, O.BB_P, np.uint32, 31, O.bb16_params()) if field == "bb"
                                 else (P.GOLDILOCKS, O.GL_P, np.uint64, 7, O.gl8_params()))
    shapes = [(11, 5), (11, 40), (6, 3), (11, 17), (6, 30), (13, 9), (11, 1), (13, 24), (6, 0), (6, 16)]
    traces = [rng.integers(0, p, size=(1 << lh, w), dtype=dt) for lh, w in shapes]
    bufs = [gpu_ctx.to_device(t) if t.size else None for t in traces]
    tree = gpu_ctx.commit_traces_device(fid, [(b.ptr if b else 0, lh, w, 2, shift)
                                              for b, (lh, w) in zip(bufs, shapes)], 0)
    lde = O.bb_coset_lde if field == "bb" else O.gl_coset_lde
    ldes = [lde(t, 2, shift, True) if t.size else np.zeros((1 << (lh + 2), 0), dt)
            for t, (lh, w) in zip(traces, shapes)]
    want = O.mmcs_commit(params, ldes, 0, nthreads=NT)
    got = tree.layers()
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    tree.free()
    for b in bufs:
        if b:
            b.free()


def test_missing_poseidon2_is_an_error():
    ctx = P.Context(0)
    try:
        m = np.ones((4, 4), np.uint32)
        with pytest.raises(P.P3GError) as e:
            ctx.mmcs_commit([m])
        assert e.value.status == 6
    finally:
        ctx.close()


def test_unsupported_schedule_is_an_error(gpu_ctx):
    gpu_ctx.set_poseidon2(P.BABYBEAR, 16, 8, 9, 7, np.zeros(64), np.zeros(64), np.zeros(9))
    with pytest.raises(P.P3GError) as e:
        gpu_ctx.permute(P.BABYBEAR, np.zeros((1, 16), np.uint32))
    assert e.value.status == 5
    gpu_ctx.set_default_poseidon2()
