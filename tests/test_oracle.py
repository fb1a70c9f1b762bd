"""Pins the CPU oracle (oracle/oracle.c) against golden vectors produced by the
reference's own code (tests/golden/make_golden.py) and against the known-answer
constants that the reference's tests hold.  CPU only."""
import hashlib

import numpy as np
import pytest

import oracle as O


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _check(out, summary):
    assert out.size == summary["n"]
    if "values" in summary:
        assert out.reshape(-1).tolist() == summary["values"]
    assert _sha(out) == summary["sha256"]


# ---------------------------------------------------------------- KATs
def test_known_answers_from_reference_tests(golden):
    L = O.lib()
    # test_two_adic.cpp:95  primitive 2^27-th root
    assert L.orc_bb_two_adic_generator(27) == 440564289
    # test_extension_field.cpp:76  dth_root
    assert L.orc_bb4_dth_root() == 1728404513
    k = golden["kat"]
    assert k["bb_two_adic_27"] == 440564289
    assert [L.orc_bb_two_adic_generator(i) for i in range(28)] == k["bb_two_adic"]
    assert [L.orc_gl_two_adic_generator(i) for i in range(33)] == k["gl_two_adic"]
    # two-adic generator orders
    for bits in range(1, 28):
        g = L.orc_bb_two_adic_generator(bits)
        assert L.orc_bb_pow(g, 1 << bits) == 1
        assert L.orc_bb_pow(g, 1 << (bits - 1)) != 1


def test_mt19937_standard_values():
    # The C++ standard's conformance values: the 10000th draw of a
    # default-seeded (5489) mt19937 / mt19937_64.
    assert int(O.mt19937(5489, 10000)[-1]) == 4123659995
    assert int(O.mt19937_64(5489, 10000)[-1]) == 9981545732273789042


def test_poseidon2_constants_match_reference(golden):
    c = golden["consts"]
    ini, ter, inr = O.example_constants_bb16()
    assert ini.reshape(-1).tolist() == c["bb16_initial"]
    assert ter.reshape(-1).tolist() == c["bb16_terminal"]
    assert inr.tolist() == c["bb16_internal"]
    ini, ter, inr = O.example_constants_gl8()
    assert [int(x) for x in ini.reshape(-1)] == c["gl8_initial"]
    assert [int(x) for x in ter.reshape(-1)] == c["gl8_terminal"]
    assert [int(x) for x in inr] == c["gl8_internal"]


def test_field_edge_values():
    L = O.lib()
    p = O.BB_P
    for a in (0, 1, 2, p - 1, p - 2, 1 << 30, (1 << 31) - 1 - (1 << 27)):
        for b in (0, 1, p - 1, 12345678):
            assert L.orc_bb_add(a, b) == (a + b) % p
            assert L.orc_bb_sub(a, b) == (a - b) % p
            assert L.orc_bb_mul(a, b) == (a * b) % p
        if a:
            assert L.orc_bb_mul(a, L.orc_bb_inv(a)) == 1
    q = O.GL_P
    for a in (0, 1, q - 1, 1 << 63, (1 << 64) - 1 - q + 5, 0xFFFFFFFF):
        for b in (0, 1, q - 1, 1 << 32):
            assert L.orc_gl_add(a, b) == (a + b) % q
            assert L.orc_gl_mul(a, b) == (a * b) % q
            assert L.orc_gl_sub(a, b) == (a - b) % q


def test_bb4_inverse_and_mul():
    rng = np.random.default_rng(5)
    for _ in range(20):
        a = rng.integers(0, O.BB_P, 4, dtype=np.uint32)
        if not a.any():
            continue
        assert O.bb4_mul(a, O.bb4_inv(a)).tolist() == [1, 0, 0, 0]


# ---------------------------------------------------------------- DFT / LDE
def test_dft_variants_vs_reference(golden):
    for case in golden["dft"]:
        m = O.bb_random_matrix(1 << case["log_h"], case["w"], case["seed"])
        out = O.bb_dft(case["kind"], m, case["shift"])
        _check(out, case["out"])


def test_dft_known_answers():
    # test_dft.cpp:410-451: DFT of e_k gives omega^{jk}; f(x)=1+2x at omega^j.
    L = O.lib()
    n, k = 8, 2
    e = np.zeros((n, 1), np.uint32)
    e[k, 0] = 1
    out = O.bb_dft("dft", e)
    om = L.orc_bb_two_adic_generator(3)
    assert out[:, 0].tolist() == [L.orc_bb_pow(om, j * k) for j in range(n)]
    c = np.array([[1], [2], [0], [0]], np.uint32)
    out = O.bb_dft("dft", c)
    om = L.orc_bb_two_adic_generator(2)
    assert out[:, 0].tolist() == [(1 + 2 * L.orc_bb_pow(om, j)) % O.BB_P for j in range(4)]


def test_lde_vs_reference(golden):
    for case in golden["lde"]:
        h = 1 << case["log_h"]
        if case["field"] == "bb":
            t = O.bb_random_matrix(h, case["w"], case["seed"])
            out = O.bb_coset_lde(t, case["log_blowup"], case["shift"], bool(case["bitrev"]))
        else:
            t = O.gl_random_matrix(h, case["w"], case["seed"])
            out = O.gl_coset_lde(t, case["log_blowup"], case["shift"], bool(case["bitrev"]))
        _check(out, case["out"])


def test_lde_threads_identical():
    t = O.bb_random_matrix(1 << 9, 13, 4)
    a = O.bb_coset_lde(t, 2, nthreads=1)
    b = O.bb_coset_lde(t, 2, nthreads=4)
    assert np.array_equal(a, b)


def test_lde_low_degree_property():
    # The LDE of h evaluations has degree < h: re-interpolating the natural-order
    # LDE on the coset yields zero coefficients above h.
    t = O.bb_random_matrix(1 << 5, 3, 9)
    lde = O.bb_coset_lde(t, 2, shift=31, bitrev=False)
    coeffs = O.bb_dft("coset_idft", lde, 31)
    assert not coeffs[1 << 5:].any()


# ---------------------------------------------------------------- Poseidon2 / sponge
def _p2(kind):
    return {"bb16": O.bb16_params, "bb16zero": O.bb16_zero_params,
            "bb16zero_generic": O.bb16_zero_params, "gl8": O.gl8_params}[kind]()


def test_permutation_vs_reference(golden):
    for case in golden["perm"]:
        p = _p2(case["kind"])
        for i, o in zip(case["inputs"], case["outputs"]):
            assert [int(x) for x in O.permute(p, np.array(i, dtype=np.uint64))] == o


def test_generic_and_pod_poseidon2_agree(golden):
    by = {c["kind"]: c for c in golden["perm"]}
    assert by["bb16zero"]["outputs"] == by["bb16zero_generic"]["outputs"]


def test_sponge_vs_reference(golden):
    for case in golden["hash"]:
        p = _p2(case["kind"])
        if case["kind"] == "gl8":
            data = O.gl_random_matrix(1, case["len"], case["seed"]) if case["len"] else np.zeros(0, np.uint64)
        else:
            data = O.bb_random_matrix(1, case["len"], case["seed"]) if case["len"] else np.zeros(0, np.uint32)
        assert [int(x) for x in O.hash_iter(p, data)] == case["digest"]


def test_sponge_edge_semantics_mock_free():
    # padding_free_sponge.hpp:63-87: empty input -> zero digest without a
    # permutation; a partial last chunk keeps the previous rate positions.
    p = O.bb16_params()
    assert not O.hash_iter(p, np.zeros(0, np.uint32)).any()
    x = np.arange(1, 12, dtype=np.uint32)
    st = np.zeros(16, np.uint32)
    st[:8] = x[:8]
    st = O.permute(p, st)
    st[:3] = x[8:]
    st = O.permute(p, st)
    assert O.hash_iter(p, x).tolist() == st[:8].tolist()


def test_compress_vs_reference(golden):
    for case in golden["compress"]:
        p = _p2(case["kind"])
        if case["kind"] == "gl8":
            m = O.gl_random_matrix(2, 4, case["seed"])
        else:
            m = O.bb_random_matrix(2, 8, case["seed"])
        assert [int(x) for x in O.compress(p, m[0], m[1])] == case["digest"]


# ---------------------------------------------------------------- Merkle
def _mats(kind, shapes, seed):
    out = []
    for i, s in enumerate(shapes):
        h, w = (int(v) for v in s.split("x"))
        if kind == "gl8":
            out.append(O.gl_random_matrix(h, w, seed + i))
        else:
            out.append(O.bb_random_matrix(h, w, seed + i))
    return out


def test_mixed_height_mmcs_vs_reference(golden):
    for case in golden["mmcs"]:
        p = _p2(case["kind"])
        layers = O.mmcs_commit(p, _mats(case["kind"], case["shapes"], case["seed"]), case["cap_height"])
        assert [len(l) for l in layers] == case["sizes"]
        for got, want in zip(layers, case["layers"]):
            assert [[int(x) for x in d] for d in got] == want


def test_commit_matrix_vs_reference(golden):
    p = O.bb16_params()
    for case in golden["commit_matrix"]:
        m = O.bb_random_matrix(case["h"], case["w"], case["seed"])
        layers = O.commit_matrix(p, m)
        assert [len(l) for l in layers] == case["sizes"]
        for got, want in zip(layers, case["layers"]):
            assert got.tolist() == want


def test_lde_commit_vs_reference(golden):
    p = O.bb16_params()
    for case in golden["commit"]:
        t = O.bb_random_matrix(1 << case["log_h"], case["w"], case["seed"])
        lde = O.bb_coset_lde(t, case["log_blowup"], case["shift"], True)
        layers = O.mmcs_commit(p, [lde], case["cap_height"])
        assert [len(l) for l in layers] == case["sizes"]
        assert layers[-1].tolist() == case["cap"]
        assert _sha(np.concatenate([l.reshape(-1) for l in layers])) == case["layers_sha256"]


def test_pcs_commit_vs_reference(golden):
    p = O.bb16_params()
    for case in golden["pcs_commit"]:
        traces = []
        for i, s in enumerate(case["shapes"]):
            lh, w = (int(v) for v in s.split("x"))
            traces.append(O.bb_random_matrix(1 << lh, w, case["seed"] + i))
        root, _ = O.pcs_commit(p, traces, case["log_blowup"], case["shift"])
        assert root.tolist() == case["root"]


# ---------------------------------------------------------------- FRI fold
def test_fold_vs_reference(golden):
    for case in golden["fold"]:
        lh = case["log_height"]
        raw = O.mt19937(case["seed"], 4 * (1 << lh) + 4) % np.uint32(O.BB_P)
        vals = raw[: 4 * (1 << lh)].reshape(-1, 4)
        beta = case["beta"]
        if case["beta_mode"] == 0:
            assert raw[4 * (1 << lh):].tolist() == beta
        out = O.fold_matrix_bb4(vals, lh, case["log_arity"], beta)
        _check(out, case["out"])


def test_fold_arity2_closed_form():
    # For arity 2 the reference Lagrange formula equals
    # (e0+e1)/2 + beta*(e0-e1)/(2x) (fri_fold_cuda.hpp:81-109).
    L = O.lib()
    p = O.BB_P
    lh = 6
    raw = O.mt19937(3, 4 * (1 << lh) + 4) % np.uint32(p)
    vals = raw[:-4].reshape(-1, 4)
    beta = raw[-4:]
    out = O.fold_matrix_bb4(vals, lh, 1, beta)
    inv2 = L.orc_bb_inv(2)
    om = L.orc_bb_two_adic_generator(lh)
    for i in range(1 << (lh - 1)):
        x = L.orc_bb_pow(om, int("{:0{}b}".format(i, lh - 1)[::-1], 2) if lh > 1 else 0)
        e0, e1 = vals[2 * i], vals[2 * i + 1]
        s = [(int(a) + int(b)) * inv2 % p for a, b in zip(e0, e1)]
        d = [(int(a) - int(b)) * inv2 % p * L.orc_bb_inv(x) % p for a, b in zip(e0, e1)]
        bd = O.bb4_mul(beta, np.array(d, np.uint32))
        assert out[i].tolist() == [(a + int(b)) % p for a, b in zip(s, bd)]


def test_mmcs_verify_batch_against_reference_trees(golden):
    # verify_batch restated in the oracle accepts the reference's own trees and
    # rejects a tampered row (merkle_tree_mmcs.hpp:168-254).
    for case in golden["mmcs"]:
        if case["kind"] == "gl8":
            continue
        p = _p2(case["kind"])
        mats = _mats(case["kind"], case["shapes"], case["seed"])
        layers = [np.array(l, dtype=np.uint32) for l in case["layers"]]
        heights = [m.shape[0] for m in mats]
        max_h = max(heights)
        for index in (0, max_h - 1, max_h // 2):
            rows = [m[index // (max_h // m.shape[0])] for m in mats]
            proof = [layers[l][(index >> l) ^ 1] for l in range(len(layers) - 1)]
            assert O.mmcs_verify_batch(p, layers[-1], heights, [m.shape[1] for m in mats], index, rows, proof)
            if rows[0].size:
                bad = [r.copy() for r in rows]
                bad[0][0] ^= 1
                assert not O.mmcs_verify_batch(p, layers[-1], heights, [m.shape[1] for m in mats], index, bad, proof)


# ---------------------------------------------------------------- PCS open
def _bitrev_rows(a):
    n = a.shape[0]
    bits = n.bit_length() - 1
    idx = [int(format(i, f"0{bits}b")[::-1], 2) if bits else 0 for i in range(n)]
    return a[idx]


def pcs_open_case(case, open_values=None, reduce=None):
    """Opened values and the first FRI commitment of TwoAdicFriPcs::open for one
    golden case, from the restated formulas (or the functions passed in)."""
    open_values = open_values or (lambda lde, z: O.pcs_open_values(lde, case["shift"], z))
    reduce = reduce or (lambda lde, z, ov, ap, q: O.pcs_reduce(lde, case["shift"], [z], ov[None], case["alpha"],
                                                               ap, q))
    shapes = [tuple(int(v) for v in s.split("x")) for s in case["shapes"]]
    traces = [O.bb_random_matrix(1 << lh, w, case["seed"] + i) for i, (lh, w) in enumerate(shapes)]
    ldes = [O.bb_coset_lde(t, case["log_blowup"], case["shift"], bitrev=False) for t in traces]
    z = case["zeta"]
    opened = [open_values(l, z) for l in ldes]
    qs, ap = {}, 0
    for lde, ov in zip(ldes, opened):
        q = qs.setdefault(lde.shape[0], np.zeros((lde.shape[0], 4), np.uint32))
        reduce(lde, z, ov, ap, q)
        ap += lde.shape[1]
    tallest = max(qs)
    arity = 1 << case["log_arity0"]
    flat = _bitrev_rows(qs[tallest]).reshape(tallest // arity, arity * 4)
    root = O.commit_matrix(O.bb16_params(), flat)[-1][0]
    return np.concatenate([o.reshape(-1) for o in opened]), root, ldes, qs


def test_pcs_open_vs_reference(golden):
    for case in golden["pcs_open"]:
        opened, root, _, _ = pcs_open_case(case)
        assert opened.tolist() == case["opened"]
        assert root.tolist() == case["commit0"]


def fri_final_poly(current: np.ndarray, log_final_poly_len: int) -> np.ndarray:
    """prove_fri's final polynomial (fri_prover.hpp:141-179): truncate, bit-reverse,
    naive inverse DFT."""
    n = 1 << log_final_poly_len
    cur = _bitrev_rows(current[:n])
    L = O.lib()
    om_inv = L.orc_bb_pow(L.orc_bb_two_adic_generator(log_final_poly_len), n - 1)
    n_inv = L.orc_bb_inv(n % O.BB_P)
    out = np.zeros((n, 4), np.uint32)
    for k in range(n):
        s = np.zeros(4, np.uint32)
        for j in range(n):
            wkj = L.orc_bb_pow(om_inv, k * j)
            s = np.array([(int(s[e]) + int(cur[j][e]) * wkj) % O.BB_P for e in range(4)], np.uint32)
        out[k] = [int(v) * n_inv % O.BB_P for v in s]
    return out


def fri_commit_phase(case, inputs, tr, commit, fold, axpy, length, download):
    """prove_fri's commit phase (fri_prover.hpp:73-139) over the given inputs
    (bit-reversed reduced openings, tallest first) with the operations passed
    in; returns the per-round roots, the final polynomial and the per-round
    log arities."""
    fri = case["fri"]
    log_final = case["log_blowup"] + fri["log_final_poly_len"]
    current, idx, roots, arities = inputs[0], 1, [], []
    while length(current) > (1 << log_final):
        log_h = length(current).bit_length() - 1
        has_next = idx < len(inputs)
        nxt = length(inputs[idx]).bit_length() - 1 if has_next else 0
        la = O.fri_log_arity(log_h, has_next, nxt, log_final, fri["max_log_arity"])
        if la == 0:
            break
        root = commit(current, 1 << la)
        tr.observe_cap([root])
        roots.append(root)
        arities.append(la)
        tr.grind(fri["commit_pow_bits"])
        beta = tr.sample_ext()
        current = fold(current, log_h, la, beta)
        if idx < len(inputs) and length(inputs[idx]) == length(current):
            current = axpy(current, O.bb4_pow(beta, 1 << la), inputs[idx])
            idx += 1
    return roots, fri_final_poly(download(current), fri["log_final_poly_len"]), arities


def fri_query_pow(case, tr, final, arities, grind):
    """prove_fri after the commit phase up to the query-phase witness
    (fri_prover.hpp:179-195): observe the final polynomial and every round's
    arity, then grind query_pow_bits with `grind(transcript, bits)`."""
    for c in final:
        tr.observe_ext(c)
    for la in arities:
        tr.observe(la)
    return grind(tr, case["fri"]["query_pow_bits"])


def fri_query_openings(case, tr, rounds):
    """prove_fri's query phase (fri_prover.hpp:199-257) after the query proof
    of work: sample each query index, then per round the committed row holding
    it (siblings = the row without the query's position) and the row's Merkle
    path.  rounds: per round (committed matrix rows x 4 arity, its layers, log
    arity).  Returns (indices, openings in the golden's layout)."""
    fri = case["fri"]
    log_max = case["log_blowup"] + fri["log_final_poly_len"] + sum(la for _, _, la in rounds)
    idx = [tr.sample_bits(log_max) for _ in range(case["num_queries"])]
    out = []
    for q in idx:
        steps, cur = [], q
        for mat, layers, la in rounds:
            row, pos = cur >> la, cur & ((1 << la) - 1)
            vals = mat[row].reshape(-1, 4)
            sib = [vals[j].tolist() for j in range(1 << la) if j != pos]
            path = []
            for lvl in range(len(layers) - 1):
                s = (row >> lvl) ^ 1
                path.append(layers[lvl][s].tolist() if s < len(layers[lvl]) else [0] * 8)
            steps.append({"log_arity": la, "siblings": sib, "path": path})
            cur = row
        out.append(steps)
    return idx, out


def open_transcript(case):
    """The transcript up to prove_fri: observe the PCS commitment, sample zeta
    (the caller's opening point) and alpha (TwoAdicFriPcs::open's first sample)."""
    tr = O.Transcript(O.bb16_params())
    tr.observe_cap([case["pcs_root"]])
    zeta = tr.sample_ext()
    alpha = tr.sample_ext()
    return tr, zeta, alpha


def test_transcript_and_fri_commit_phase_vs_reference(golden):
    for case in golden["pcs_open"]:
        tr, zeta, alpha = open_transcript(case)
        assert zeta == case["zeta"] and alpha == case["alpha"]
        opened, _, ldes, qs = pcs_open_case(case)
        for v in opened.reshape(-1, 4):  # two_adic_fri_pcs.hpp:338-346
            tr.observe_ext(v)
        inputs = [_bitrev_rows(qs[h]) for h in sorted(qs, reverse=True)]
        committed = []

        def commit(cur, arity):
            mat = cur.reshape(-1, 4 * arity)
            layers = O.commit_matrix(O.bb16_params(), mat)
            committed.append((mat, layers, arity.bit_length() - 1))
            return layers[-1][0]

        roots, final, arities = fri_commit_phase(
            case, inputs, tr, commit=commit,
            fold=lambda cur, lh, la, beta: O.fold_matrix_bb4(cur, lh, la, beta),
            axpy=O.bb4_axpy, length=len, download=lambda c: c)
        assert [r.tolist() for r in roots] == case["commits"]
        assert final.tolist() == case["final_poly"]
        w = fri_query_pow(case, tr, final, arities, lambda t, bits: t.grind_py(bits))
        assert w == case["fri"]["query_pow_witness"]
        _, openings = fri_query_openings(case, tr, committed)
        assert openings == case["query_openings"]
        for pc in golden["pcs_commit"]:  # the same commitment where the commit cases overlap
            if pc["seed"] == case["seed"] and pc["shapes"] == case["shapes"]:
                assert pc["root"] == case["pcs_root"]


def test_grind_vs_reference(golden):
    """DuplexChallenger::grind (duplex_challenger.hpp:234-251) after 0..15
    observations (every pending-input count, including RATE - 1 where the
    witness's low half fills the buffer), bits 0..20, and the sample that
    follows: the C restatement, and the Python one for the small cases."""
    p = O.bb16_params()
    for c in golden["grind"]:
        tr, tr_py = O.Transcript(p), O.Transcript(p)
        for v in O.mt19937(c["seed"], c["n_obs"]):
            tr.observe(int(v) % O.BB_P)
            tr_py.observe(int(v) % O.BB_P)
        for bits, w, after in zip(c["bits"], c["witness"], c["sample_after"]):
            assert tr.grind(bits) == w, (c, bits)
            assert tr.sample() == after
            if bits <= 12:
                assert tr_py.grind_py(bits) == w
                assert tr_py.sample() == after
            else:
                assert tr_py.check_witness(bits, w) and tr_py.sample() == after


def test_grind_oracle_goldilocks_and_limits():
    """The restatement over Goldilocks (width 8, rate 4; the reference's grind
    does not compile for its Goldilocks, so this is unpinned) agrees with a
    direct replay; a limit below the first hit reports no witness."""
    p = O.gl8_params()
    rng = np.random.default_rng(5)
    for k in range(4):
        st = rng.integers(0, O.GL_P, size=8, dtype=np.uint64)
        pend = [int(x) for x in rng.integers(0, O.GL_P, size=k, dtype=np.uint64)]
        w = O.grind(p, st, pend, 6)
        for cand in range(w + 1):  # replay: candidate w passes, every smaller one fails
            s = st.copy()
            inp = pend + [cand & 0xFFFFFFFF, cand >> 32]
            s[:min(len(inp), 4)] = inp[:4]
            s = O.permute(p, s)
            if len(inp) > 4:
                s[0] = inp[4]
                s = O.permute(p, s)
            assert (int(s[3]) & 63 == 0) == (cand == w), (k, cand, w)
        with pytest.raises(ValueError):
            O.grind(p, st, pend, 6, limit=w)
