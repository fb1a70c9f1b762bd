"""The C++ adapters (include/p3g_adapters.hpp) on the GPU, driven by
tests/cpp/adapters_standin.cpp with stand-ins of the reference's types, against
the oracle: GpuDft::coset_lde_batch (natural order), GpuInputMmcs::commit_matrix
(every layer, odd heights), GpuMerkleTreeMmcs::commit (mixed heights, caps,
both fields) and gpu_fold_matrix; GpuDuplexChallenger against the reference's
own grind witnesses.  Bit-exact."""
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import compile_cpp
from test_gpu_fri import _oracle_fri, _params, reduced_openings

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("adapters") / "standin")
    rc, log = compile_cpp("adapters_standin.cpp", out)
    assert rc == 0, log
    return out


def _run(prog, tmp_path, cmd, field, rest, data: np.ndarray):
    """adapters_standin <cmd> [<field>] <in> <out> <rest...>"""
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    data.tofile(fin)
    argv = [prog, cmd] + ([field] if field else []) + [fin, fout] + [str(x) for x in rest]
    r = subprocess.run(argv, capture_output=True, text=True, timeout=120)
    return r.returncode, r.stderr, fout


def _layers(raw: np.ndarray, sizes, digest):
    out, off = [], 0
    for s in sizes:
        out.append(raw[off:off + s * digest].reshape(s, digest))
        off += s * digest
    assert off == raw.size
    return out


@pytest.mark.parametrize("field,log_h,w,bits,shift", [
    ("bb", 6, 5, 1, 31), ("bb", 11, 3, 2, 31), ("bb", 14, 9, 1, 31), ("gl", 7, 4, 2, 7), ("gl", 12, 3, 1, 7)])
def test_gpu_dft_coset_lde_batch(prog, tmp_path, field, log_h, w, bits, shift):
    rng = np.random.default_rng(log_h * 31 + w)
    if field == "bb":
        t = rng.integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
        want = O.bb_coset_lde(t, bits, shift, bitrev=False)
    else:
        t = rng.integers(0, O.GL_P, size=(1 << log_h, w), dtype=np.uint64)
        want = O.gl_coset_lde(t, bits, shift, bitrev=False)
    rc, err, fout = _run(prog, tmp_path, "lde", field, [log_h, w, bits, shift], t)
    assert rc == 0, err
    got = np.fromfile(fout, dtype=t.dtype).reshape(want.shape)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("field,log_h,kind", [("bb", 5, 0), ("bb", 12, 1), ("bb", 11, 2), ("bb", 13, 3),
                                               ("gl", 9, 0), ("gl", 12, 3)])
def test_gpu_dft_other_members(prog, tmp_path, field, log_h, kind):
    """GpuDft::dft_batch / idft_batch / coset_dft_batch / coset_idft_batch."""
    w, shift = 3, 7
    rng = np.random.default_rng(log_h * 4 + kind)
    if field == "bb":
        t = rng.integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
        want = O.bb_dft(["dft", "idft", "coset_dft", "coset_idft"][kind], t, shift)
    else:
        t = rng.integers(0, O.GL_P, size=(1 << log_h, w), dtype=np.uint64)
        want = None  # the oracle restates the BabyBear DFTs; Goldilocks is checked by inversion
    rc, err, fout = _run(prog, tmp_path, "dft", field, [log_h, w, kind, shift], t)
    assert rc == 0, err
    got = np.fromfile(fout, dtype=t.dtype).reshape(t.shape)
    if want is not None:
        assert np.array_equal(got, want)
    else:
        back = 1 if kind == 0 else 2  # dft -> idft, coset_idft -> coset_dft
        rc, err, fout2 = _run(prog, tmp_path, "dft", field, [log_h, w, back, shift], got)
        assert rc == 0, err
        assert np.array_equal(np.fromfile(fout2, dtype=t.dtype).reshape(t.shape), t)


@pytest.mark.parametrize("h,w", [(1, 8), (37, 8), (256, 16), (1000, 3)])
def test_gpu_input_mmcs_commit_matrix(prog, tmp_path, h, w):
    rng = np.random.default_rng(h + w)
    m = rng.integers(0, O.BB_P, size=(h, w), dtype=np.uint32)
    rc, err, fout = _run(prog, tmp_path, "commit_matrix", None, [h, w], m)
    assert rc == 0, err
    want = O.commit_matrix(O.bb16_params(), m)
    got = _layers(np.fromfile(fout, dtype=np.uint32), [l.shape[0] for l in want], 8)
    for g, wl in zip(got, want):
        assert np.array_equal(g, wl)


@pytest.mark.parametrize("field,cap,shapes", [
    ("bb", 0, [(1024, 7), (256, 3), (1024, 2), (64, 5)]),
    ("bb", 2, [(512, 16), (512, 1), (8, 4)]),
    ("gl", 1, [(256, 5), (128, 3), (256, 1)]),
])
def test_gpu_merkle_tree_mmcs_commit(prog, tmp_path, field, cap, shapes):
    _mixed_tree(prog, tmp_path, "mmcs", field, cap, shapes)


@pytest.mark.parametrize("field,cap,shapes", [
    ("bb", 0, [(64, 9), (32, 4), (64, 16)]), ("bb", 2, [(256, 8)]), ("gl", 1, [(128, 5), (32, 3), (128, 2)])])
def test_build_merkle_tree_cuda_adapter(prog, tmp_path, field, cap, shapes):
    """build_merkle_tree_cuda with the reference's signature (constants taken
    from a Poseidon2Cuda-like struct) builds the oracle's layers."""
    _mixed_tree(prog, tmp_path, "build_tree", field, cap, shapes)


def _mixed_tree(prog, tmp_path, cmd, field, cap, shapes):
    rng = np.random.default_rng(len(shapes) * 7 + cap)
    if field == "bb":
        mats = [rng.integers(0, O.BB_P, size=s, dtype=np.uint32) for s in shapes]
        params, digest = O.bb16_params(), 8
    else:
        mats = [rng.integers(0, O.GL_P, size=s, dtype=np.uint64) for s in shapes]
        params, digest = O.gl8_params(), 4
    flat = np.concatenate([m.reshape(-1) for m in mats])
    rest = [cap] + [x for s in shapes for x in s]
    rc, err, fout = _run(prog, tmp_path, cmd, field, rest, flat)
    assert rc == 0, err
    want = O.mmcs_commit(params, mats, cap)
    got = _layers(np.fromfile(fout, dtype=flat.dtype), [l.shape[0] for l in want], digest)
    for g, wl in zip(got, want):
        assert np.array_equal(g, wl)


@pytest.mark.parametrize("log_arity", [1, 2, 3])
def test_gpu_fold_matrix(prog, tmp_path, log_arity):
    rng = np.random.default_rng(50 + log_arity)
    log_h = 11
    v = rng.integers(0, O.BB_P, size=(1 << log_h, 4), dtype=np.uint32)
    beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
    rc, err, fout = _run(prog, tmp_path, "fold", None, [log_h, log_arity],
                         np.concatenate([beta, v.reshape(-1)]))
    assert rc == 0, err
    got = np.fromfile(fout, dtype=np.uint32).reshape(-1, 4)
    assert np.array_equal(got, O.fold_matrix_bb4(v, log_h, log_arity, beta))


@pytest.mark.parametrize("log_arity", [1, 2, 3])
def test_fold_matrix_cuda_forms(prog, tmp_path, log_arity):
    """fold_matrix_cuda / fold_matrix_cuda_device (the reference's GPU fold
    signatures, fri_fold_cuda.hpp:250-348) agree with each other and the oracle."""
    rng = np.random.default_rng(60 + log_arity)
    log_h = 12
    v = rng.integers(0, O.BB_P, size=(1 << log_h, 4), dtype=np.uint32)
    beta = rng.integers(0, O.BB_P, size=4, dtype=np.uint32)
    rc, err, fout = _run(prog, tmp_path, "fold_cuda", None, [log_h, log_arity], np.concatenate([beta, v.reshape(-1)]))
    assert rc == 0, err
    got = np.fromfile(fout, dtype=np.uint32).reshape(-1, 4)
    assert np.array_equal(got, O.fold_matrix_bb4(v, log_h, log_arity, beta))


def test_gpu_prove_fri_adapter(prog, tmp_path, gpu_ctx, golden):
    """p3g::gpu_prove_fri with the reference's prove_fri signature (stand-in
    proof types, a transcript wrapper holding a GpuDuplexChallenger) builds the
    reference's proofs -- roots, final polynomial, query witness, every query's
    siblings and path -- and leaves the challenger where the oracle's does."""
    for case in golden["pcs_open"]:
        tr, qs = reduced_openings(gpu_ctx, case)
        heights = sorted(qs, reverse=True)
        vectors = [qs[h].download(np.uint32, (1 << h, 4)) for h in heights]
        before = tr.copy()
        st = np.zeros(16 + 8 + 8 + 2, np.uint32)
        st[:16] = tr.state
        st[16:16 + len(tr.inp)] = tr.inp
        st[24:24 + len(tr.out)] = tr.out
        st[32], st[33] = len(tr.inp), len(tr.out)
        fch = tmp_path / "ch.bin"
        st.tofile(fch)
        prm = _params(case)
        rc, err, fout = _run(prog, tmp_path, "prove_fri", None,
                             [str(fch), prm["num_queries"], prm["log_blowup"], prm["log_final_poly_len"],
                              prm["max_log_arity"], prm["commit_proof_of_work_bits"],
                              prm["query_proof_of_work_bits"]] + heights, np.concatenate(vectors).reshape(-1))
        assert rc == 0, err
        raw = np.fromfile(fout, dtype=np.uint8)
        pos = [0]

        def take(n, dt=np.uint32):
            v = raw[pos[0]:pos[0] + n * np.dtype(dt).itemsize].view(dt)
            pos[0] += n * np.dtype(dt).itemsize
            return v

        nr = int(take(1)[0])
        assert take(8 * nr).reshape(nr, 8).tolist() == case["commits"]
        nf = int(take(1)[0])
        assert take(4 * nf).reshape(nf, 4).tolist() == case["final_poly"]
        assert int(take(1, np.uint64)[0]) == case["fri"]["query_pow_witness"]
        nq = int(take(1)[0])
        _, _, _, idx, openings = _oracle_fri(case, before, vectors)
        assert openings == case["query_openings"]
        for q in range(nq):
            assert int(take(1, np.uint64)[0]) == idx[q]
            for step in case["query_openings"][q]:
                assert int(take(1)[0]) == step["log_arity"]
                ns = int(take(1)[0])
                assert take(4 * ns).reshape(ns, 4).tolist() == step["siblings"]
                npth = int(take(1)[0])
                assert take(8 * npth).reshape(npth, 8).tolist() == step["path"]
        after = take(34)
        assert after[:16].tolist() == [int(x) for x in before.state]
        assert after[32] == len(before.inp) and after[16:16 + after[32]].tolist() == before.inp
        assert after[33] == len(before.out) and after[24:24 + after[33]].tolist() == before.out
        assert pos[0] == raw.size
        for b in qs.values():
            b.free()


def test_gpu_duplex_challenger_grind(prog, tmp_path, golden):
    """GpuDuplexChallenger's observe / grind / sample sequence gives the
    witnesses and samples of the reference's DuplexChallenger."""
    for c in golden["grind"]:
        fout = str(tmp_path / "ch.bin")
        r = subprocess.run([prog, "challenger", fout, str(c["seed"]), str(c["n_obs"])] + [str(b) for b in c["bits"]],
                           capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        raw = open(fout, "rb").read()
        for i, (w, after) in enumerate(zip(c["witness"], c["sample_after"])):
            assert int.from_bytes(raw[12 * i:12 * i + 8], "little") == w, (c, i)
            assert int.from_bytes(raw[12 * i + 8:12 * i + 12], "little") == after, (c, i)


def test_adapter_reports_bad_dimensions_as_invalid_argument(prog, tmp_path):
    rc, err, _ = _run(prog, tmp_path, "commit_matrix", None, [0, 0], np.zeros(0, np.uint32))
    assert rc == 4, err
    assert "bad dimensions" in err


def test_gpu_pcs_commit_composition_matches_reference_roots(prog, tmp_path, golden):
    """TwoAdicFriPcs::commit (two_adic_fri_pcs.hpp:207-266) chained as the PCS
    chains its members -- GpuDft::coset_lde_batch per matrix, rows joined with
    r % height, zero columns up to a power-of-two width, GpuInputMmcs::commit_matrix
    -- gives the reference's own commitment roots on the GPU, and the flat
    matrix it commits equals the oracle's."""
    p = O.bb16_params()
    for case in golden["pcs_commit"]:
        shapes = [tuple(int(v) for v in s.split("x")) for s in case["shapes"]]
        traces = [O.bb_random_matrix(1 << lh, w, case["seed"] + i) for i, (lh, w) in enumerate(shapes)]
        data = np.concatenate([t.reshape(-1) for t in traces])
        rest = [case["log_blowup"], case["shift"]] + [x for lh_w in shapes for x in lh_w]
        rc, err, fout = _run(prog, tmp_path, "pcs_commit", None, rest, data)
        assert rc == 0, err
        got = np.fromfile(fout, dtype=np.uint32)
        assert got[:8].tolist() == case["root"]
        root, flat = O.pcs_commit(p, traces, case["log_blowup"], case["shift"])
        assert np.array_equal(got[8:].reshape(flat.shape), flat)
