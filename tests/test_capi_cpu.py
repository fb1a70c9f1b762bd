"""C-ABI checks that need no GPU: the library loads, exports every function
include/p3g.h declares, and reports errors through status codes."""
import ctypes as C
import os
import re

import pytest

import p3g_gb300 as P

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(REPO, "include", "p3g.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(p3g_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_expected_entry_points():
    assert set(P.EXPORTS) <= set(_declared())


def test_library_exports_every_declared_symbol():
    L = P.load()
    missing = [n for n in _declared() if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_status_strings():
    L = P.load()
    assert L.p3g_version() == 1
    assert L.p3g_status_string(0) == b"ok"
    assert L.p3g_status_string(1) == b"invalid argument"


def test_null_arguments_rejected_without_gpu_work():
    L = P.load()
    # a null context is rejected before any CUDA call
    rc = L.p3g_coset_lde(None, 0, None, 4, 4, 1, 31, 1, None, None)
    assert rc == 1
    buf = C.create_string_buffer(256)
    L.p3g_last_error(buf, 256)
    assert b"null" in buf.value
    assert L.p3g_ctx_create(0, None) == 1
    assert L.p3g_dft(None, 0, P.DFT, None, 4, 4, 0, 0, None, None) == 1
    assert L.p3g_bb4_axpy(None, None, None, 4, None, None) == 1
    assert L.p3g_pcs_open_values(None, None, 4, 4, 0, 31, None, 1, None, None) == 1


def test_seeded_constants_match_oracle():
    import oracle as O
    ini, ter, inr = P.seeded_constants_bb16(13)
    oi, ot, on = O.example_constants_bb16()
    assert ini.tolist() == oi.reshape(-1).tolist()
    assert ter.tolist() == ot.reshape(-1).tolist()
    assert inr.tolist() == on.tolist()
    ini, ter, inr = P.seeded_constants_gl8(22)
    oi, ot, on = O.example_constants_gl8()
    assert [int(x) for x in ini] == [int(x) for x in oi.reshape(-1)]
    assert [int(x) for x in inr] == [int(x) for x in on]


def _fri_rounds(heights, **kw):
    prm = P.FriParams(**{**dict(log_blowup=1, log_final_poly_len=0, max_log_arity=1, num_queries=4,
                                commit_proof_of_work_bits=0, query_proof_of_work_bits=0), **kw})
    lh = (C.c_uint32 * len(heights))(*heights)
    n = C.c_uint32()
    las = (C.c_uint32 * 32)()
    st = P.load().p3g_fri_rounds(lh, len(heights), C.byref(prm), C.byref(n), las)
    return st, [las[i] for i in range(n.value)]


@pytest.mark.parametrize("heights,max_la,log_fpl", [
    ([21], 1, 0), ([12, 10, 9, 5], 3, 2), ([14], 2, 0), ([9, 8, 7, 6, 5, 4], 1, 1), ([11, 6], 3, 3),
    ([27, 3], 3, 0)])
def test_fri_rounds_follow_compute_log_arity_for_round(heights, max_la, log_fpl):
    """p3g_fri_rounds (host logic, no GPU) against the oracle's restatement of
    compute_log_arity_for_round (fri_params.hpp:36-57) driving prove_fri's loop."""
    import oracle as O
    st, got = _fri_rounds(heights, max_log_arity=max_la, log_final_poly_len=log_fpl)
    assert st == 0
    log_final = 1 + log_fpl
    want, cur, idx = [], heights[0], 1
    while cur > log_final:
        has_next = idx < len(heights)
        la = O.fri_log_arity(cur, has_next, heights[idx] if has_next else 0, log_final, max_la)
        if la == 0:
            break
        want.append(la)
        cur -= la
        if has_next and heights[idx] == cur:
            idx += 1
    assert got == want


@pytest.mark.parametrize("heights,kw,status", [
    ([6, 6], {}, 1),                           # heights must strictly decrease
    ([6], dict(max_log_arity=0), 1),
    ([6], dict(max_log_arity=4), 5),           # fold arities up to 8
    ([1], {}, 1),                              # smallest input not above the final domain (2^1)
    ([28], {}, 1),
    ([12], dict(num_queries=1025), 1),
    ([12], dict(commit_proof_of_work_bits=25), 1),
])
def test_fri_rounds_rejects_bad_arguments(heights, kw, status):
    assert _fri_rounds(heights, **kw)[0] == status


def test_pool_statistics_reject_null_context():
    assert P.load().p3g_ctx_memory(None, None, None, None, None) == 1
