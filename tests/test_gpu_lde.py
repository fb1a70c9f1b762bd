"""GPU parity of the coset LDE (p3g_coset_lde) against the oracle and the
golden vectors produced by the reference's Radix2Dit::coset_lde_batch.
Bit-exact: integer field arithmetic."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_lde_golden(gpu_ctx, golden):
    for case in golden["lde"]:
        h = 1 << case["log_h"]
        if case["field"] == "bb":
            t = O.bb_random_matrix(h, case["w"], case["seed"])
        else:
            t = O.gl_random_matrix(h, case["w"], case["seed"])
        out = gpu_ctx.coset_lde(t, case["log_blowup"], case["shift"], bool(case["bitrev"]))
        assert _sha(out) == case["out"]["sha256"], case


@pytest.mark.parametrize("log_h", list(range(0, 17)))
def test_lde_bb_all_heights(gpu_ctx, log_h):
    rng = np.random.default_rng(log_h)
    for w, lb in ((1, 1), (7, 2), (16, 1), (33, 3), (5, 0)):
        if log_h + lb > 27 or (log_h >= 15 and w > 16):
            continue
        t = rng.integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
        shift = int(rng.integers(1, O.BB_P))
        for br in (True, False):
            got = gpu_ctx.coset_lde(t, lb, shift, br)
            want = O.bb_coset_lde(t, lb, shift, br, nthreads=os.cpu_count() or 1)
            assert np.array_equal(got, want), (log_h, w, lb, br)


@pytest.mark.parametrize("log_h", [1, 4, 9, 10, 11, 12, 15])
def test_lde_gl_heights(gpu_ctx, log_h):
    rng = np.random.default_rng(100 + log_h)
    for w, lb in ((3, 2), (8, 1), (9, 0)):
        t = (rng.integers(0, 2**63, size=(1 << log_h, w), dtype=np.uint64) * 2 + 1) % np.uint64(O.GL_P)
        t = t.astype(np.uint64)
        for br in (True, False):
            got = gpu_ctx.coset_lde(t, lb, 7, br)
            want = O.gl_coset_lde(t, lb, 7, br, nthreads=os.cpu_count() or 1)
            assert np.array_equal(got, want), (log_h, w, lb, br)


def test_lde_edge_values(gpu_ctx):
    # all p-1, all zero, one-hot columns
    h = 1 << 11
    t = np.full((h, 8), O.BB_P - 1, np.uint32)
    t[:, 1] = 0
    t[:, 2] = 0
    t[5, 2] = 1
    for lb in (1, 2):
        assert np.array_equal(gpu_ctx.coset_lde(t, lb), O.bb_coset_lde(t, lb))


def test_lde_rejects_bad_arguments(gpu_ctx):
    L = P.load()
    d = gpu_ctx.alloc(64)
    # log_h + log_blowup beyond two-adicity
    assert L.p3g_coset_lde(gpu_ctx.handle, 0, d.ptr, 26, 1, 2, 31, 1, d.ptr, None) == 1
    # zero shift
    assert L.p3g_coset_lde(gpu_ctx.handle, 0, d.ptr, 2, 1, 1, 0, 1, d.ptr, None) == 1
    # non-canonical shift
    assert L.p3g_coset_lde(gpu_ctx.handle, 0, d.ptr, 2, 1, 1, O.BB_P, 1, d.ptr, None) == 1
    # unknown field
    assert L.p3g_coset_lde(gpu_ctx.handle, 7, d.ptr, 2, 1, 1, 3, 1, d.ptr, None) == 1
    d.free()


def test_lde_full_size_config1(gpu_ctx):
    """2^20 x 256 BabyBear, log_blowup 1: every LDE element against the oracle
    (multithreaded restatement of Radix2Dit)."""
    rng = np.random.default_rng(20)
    t = rng.integers(0, O.BB_P, size=(1 << 20, 256), dtype=np.uint32)
    got = gpu_ctx.coset_lde(t, 1)
    want = O.bb_coset_lde(t, 1, nthreads=os.cpu_count() or 1)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("log_h,w,lb,field", [(21, 3, 1, "bb"), (21, 1, 2, "bb"), (17, 20, 3, "bb"),
                                              (21, 2, 1, "gl"), (19, 3, 2, "gl")])
def test_lde_largest_supported_heights(gpu_ctx, log_h, w, lb, field):
    """The three-pass limit (h = 2^21) and deep blowups, odd widths, both orders."""
    rng = np.random.default_rng(log_h * 7 + w)
    if field == "bb":
        t = rng.integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
        ref = lambda br: O.bb_coset_lde(t, lb, 31, br, nthreads=os.cpu_count() or 1)
        shift = 31
    else:
        t = rng.integers(0, O.GL_P, size=(1 << log_h, w), dtype=np.uint64)
        ref = lambda br: O.gl_coset_lde(t, lb, 7, br, nthreads=os.cpu_count() or 1)
        shift = 7
    for br in (True, False):
        assert np.array_equal(gpu_ctx.coset_lde(t, lb, shift, br), ref(br)), (log_h, w, lb, br)


@pytest.mark.parametrize("log_h,w,lb,field", [(22, 3, 1, "bb"), (23, 1, 2, "bb"), (22, 2, 1, "gl")])
def test_lde_split_transform_heights(gpu_ctx, log_h, w, lb, field):
    """Above 2^21 rows the coefficients and each coset's evaluations go through
    the split transform (2^21-point inner transforms, 2- or 4-point outer
    steps): every element against the oracle, both orders."""
    rng = np.random.default_rng(log_h * 11 + w)
    if field == "bb":
        t = rng.integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
        ref = lambda br: O.bb_coset_lde(t, lb, 31, br, nthreads=os.cpu_count() or 1)
        shift = 31
    else:
        t = rng.integers(0, O.GL_P, size=(1 << log_h, w), dtype=np.uint64)
        ref = lambda br: O.gl_coset_lde(t, lb, 7, br, nthreads=os.cpu_count() or 1)
        shift = 7
    for br in (True, False):
        assert np.array_equal(gpu_ctx.coset_lde(t, lb, shift, br), ref(br)), (log_h, w, lb, br)


def test_lde_split_transform_eight_point_outer_step(gpu_ctx):
    """2^24 rows: 2^21-point inner transforms and an 8-point outer step, both
    orders, against the oracle."""
    t = np.random.default_rng(24).integers(0, O.BB_P, size=(1 << 24, 2), dtype=np.uint32)
    want = O.bb_coset_lde(t, 1, 31, False, nthreads=2)
    assert np.array_equal(gpu_ctx.coset_lde(t, 1, 31, False), want)
    idx = np.arange(1 << 25, dtype=np.int64)
    rev = np.zeros_like(idx)
    for b in range(25):
        rev |= ((idx >> b) & 1) << (24 - b)
    assert np.array_equal(gpu_ctx.coset_lde(t, 1, 31, True), want[rev])


def test_lde_beyond_supported_height_is_reported(gpu_ctx):
    d = gpu_ctx.alloc(64)
    L = P.load()
    # 2^27 rows: within BabyBear's two-adicity (no blowup) but above the split transform's 2^26
    assert L.p3g_coset_lde(gpu_ctx.handle, 0, d.ptr, 27, 1, 0, 31, 1, d.ptr, None) == 5  # unsupported
    assert L.p3g_coset_lde(gpu_ctx.handle, 1, d.ptr, 27, 1, 1, 7, 1, d.ptr, None) == 5
    assert L.p3g_coset_lde(gpu_ctx.handle, 0, d.ptr, 27, 1, 1, 31, 1, d.ptr, None) == 1  # beyond two-adicity
    # above 2^21 rows the width is limited to 2^17 (checked before anything is allocated or launched)
    assert L.p3g_coset_lde(gpu_ctx.handle, 0, d.ptr, 22, (1 << 17) + 1, 1, 31, 1, d.ptr, None) == 1
    assert L.p3g_dft(gpu_ctx.handle, 0, P.DFT, d.ptr, 22, (1 << 17) + 1, 0, 0, d.ptr + 32, None) == 1
    d.free()
