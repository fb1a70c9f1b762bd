"""dft / idft / coset_dft / coset_idft through p3g_dft (Radix2Dit's other Dft
members, radix2_dit.hpp:82-210), bit-exact: every golden case of the
reference, random shapes against the oracle for both orders and every kind
(single-kernel and two-pass sizes, up to 2^21 rows), Goldilocks against a
direct O(n^2) evaluation and through identities, and argument errors."""
import hashlib

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu

KIND = {"dft": P.DFT, "idft": P.IDFT, "coset_dft": P.COSET_DFT, "coset_idft": P.COSET_IDFT}
BITREV = lambda a: a[[int(format(i, f"0{a.shape[0].bit_length() - 1}b")[::-1] or "0", 2)
                       for i in range(a.shape[0])]]


def test_golden_dft_variants(gpu_ctx, golden):
    for case in golden["dft"]:
        m = O.bb_random_matrix(1 << case["log_h"], case["w"], case["seed"])
        got = gpu_ctx.dft(KIND[case["kind"]], m, case["shift"])
        assert got.size == case["out"]["n"]
        if "values" in case["out"]:
            assert got.reshape(-1).tolist() == case["out"]["values"], (case["kind"], case["log_h"])
        assert hashlib.sha256(got.tobytes()).hexdigest() == case["out"]["sha256"], (case["kind"], case["log_h"])


@pytest.mark.parametrize("log_h,w", [(1, 3), (4, 17), (9, 5), (10, 33), (11, 7), (12, 16), (15, 9), (16, 40)])
@pytest.mark.parametrize("kind", ["dft", "idft", "coset_dft", "coset_idft"])
def test_random_shapes_vs_oracle(gpu_ctx, log_h, w, kind):
    rng = np.random.default_rng(log_h * 1000 + w)
    m = rng.integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
    shift = 31 if kind.startswith("coset") else 0
    want = O.bb_dft(kind, m, shift or 31)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, shift), want)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, shift, bitrev=True), BITREV(want))


@pytest.mark.parametrize("log_h,w,kind", [(20, 8, "dft"), (21, 2, "coset_idft"), (20, 3, "idft")])
def test_large_heights_vs_oracle(gpu_ctx, log_h, w, kind):
    m = np.random.default_rng(log_h).integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, 7), O.bb_dft(kind, m, 7))


@pytest.mark.parametrize("log_h,w", [(22, 2), (23, 1)])
@pytest.mark.parametrize("kind", ["dft", "idft", "coset_dft", "coset_idft"])
def test_split_transform_heights_vs_oracle(gpu_ctx, log_h, w, kind):
    """Above 2^21 rows the transform splits once more (inner 2^21-point
    transforms, outer 2- and 4-point steps): every kind, both orders."""
    m = np.random.default_rng(log_h + w).integers(0, O.BB_P, size=(1 << log_h, w), dtype=np.uint32)
    want = O.bb_dft(kind, m, 11)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, 11), want)
    br = np.arange(1 << log_h, dtype=np.int64)
    rev = np.zeros_like(br)
    for b in range(log_h):
        rev |= ((br >> b) & 1) << (log_h - 1 - b)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, 11, bitrev=True), want[rev])


def _bitrev_rows(log_h):
    idx = np.arange(1 << log_h, dtype=np.int64)
    rev = np.zeros_like(idx)
    for b in range(log_h):
        rev |= ((idx >> b) & 1) << (log_h - 1 - b)
    return rev


@pytest.mark.parametrize("log_h,kind", [(24, "coset_idft"), (25, "dft"), (26, "coset_dft")])
def test_split_transform_outer_sizes_vs_oracle(gpu_ctx, log_h, kind):
    """Outer steps of 8, 16 and 32 points (2^24 .. 2^26 rows, one column),
    forward, inverse with the coset scaling, both orders."""
    m = np.random.default_rng(log_h).integers(0, O.BB_P, size=(1 << log_h, 1), dtype=np.uint32)
    want = O.bb_dft(kind, m, 31)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, 31), want)
    assert np.array_equal(gpu_ctx.dft(KIND[kind], m, 31, bitrev=True), want[_bitrev_rows(log_h)])


@pytest.mark.parametrize("log_h", [25, 26])
def test_goldilocks_split_transform_outer_sizes(gpu_ctx, log_h):
    x = np.random.default_rng(log_h).integers(0, O.GL_P, size=(1 << log_h, 1), dtype=np.uint64)
    fwd = gpu_ctx.dft(P.COSET_DFT, x, 7)
    assert np.array_equal(gpu_ctx.dft(P.COSET_IDFT, fwd, 7), x)
    assert np.array_equal(gpu_ctx.dft(P.COSET_DFT, x, 7, bitrev=True), fwd[_bitrev_rows(log_h)])


def test_goldilocks_split_transform_identities(gpu_ctx):
    x = np.random.default_rng(22).integers(0, O.GL_P, size=(1 << 22, 2), dtype=np.uint64)
    assert np.array_equal(gpu_ctx.dft(P.IDFT, gpu_ctx.dft(P.DFT, x)), x)
    assert np.array_equal(gpu_ctx.dft(P.COSET_IDFT, gpu_ctx.dft(P.COSET_DFT, x, 7), 7), x)
    lde = gpu_ctx.coset_lde(x, 0, 7, bitrev=False)
    assert np.array_equal(lde, gpu_ctx.dft(P.COSET_DFT, gpu_ctx.dft(P.IDFT, x), 7))


def _gl_pow(a, e):
    return pow(int(a), int(e), O.GL_P)


@pytest.mark.parametrize("log_h,w", [(3, 2), (6, 3), (11, 2)])
def test_goldilocks_direct_evaluation(gpu_ctx, log_h, w):
    """out[j] = sum_k x_k w^(jk) (dft) and shift^(-j)/h sum_k x_k w^(-jk) (coset_idft),
    with w = 7^((p-1)/2^log_h)."""
    h = 1 << log_h
    rng = np.random.default_rng(log_h)
    x = rng.integers(0, O.GL_P, size=(h, w), dtype=np.uint64)
    om = _gl_pow(7, (O.GL_P - 1) >> log_h)
    rows = list(range(h)) if h <= 64 else [0, 1, 2, h // 2, h - 1]
    got_f = gpu_ctx.dft(P.DFT, x)
    got_ci = gpu_ctx.dft(P.COSET_IDFT, x, 7)
    inv_h, inv_s = _gl_pow(h, O.GL_P - 2), _gl_pow(7, O.GL_P - 2)
    for j in rows:
        for c in range(w):
            fwd = sum(int(x[k, c]) * _gl_pow(om, j * k) for k in range(h)) % O.GL_P
            inv = sum(int(x[k, c]) * _gl_pow(om, (h - j) * k % h) for k in range(h)) % O.GL_P
            assert int(got_f[j, c]) == fwd
            assert int(got_ci[j, c]) == inv * inv_h % O.GL_P * _gl_pow(inv_s, j) % O.GL_P


@pytest.mark.parametrize("log_h,w", [(5, 4), (12, 6), (17, 3)])
def test_goldilocks_identities(gpu_ctx, log_h, w):
    x = np.random.default_rng(log_h).integers(0, O.GL_P, size=(1 << log_h, w), dtype=np.uint64)
    assert np.array_equal(gpu_ctx.dft(P.IDFT, gpu_ctx.dft(P.DFT, x)), x)
    assert np.array_equal(gpu_ctx.dft(P.COSET_IDFT, gpu_ctx.dft(P.COSET_DFT, x, 7), 7), x)
    # coset_lde with no blowup = coset_dft(idft(x))  (radix2_dit.hpp:221-233)
    lde = gpu_ctx.coset_lde(x, 0, 7, bitrev=False)
    assert np.array_equal(lde, gpu_ctx.dft(P.COSET_DFT, gpu_ctx.dft(P.IDFT, x), 7))
    assert np.array_equal(lde, O.gl_coset_lde(x, 0, 7, False))


def test_single_row_is_identity(gpu_ctx):
    x = np.array([[5, 6, 7]], dtype=np.uint32)
    for k in (P.DFT, P.IDFT, P.COSET_DFT, P.COSET_IDFT):
        assert np.array_equal(gpu_ctx.dft(k, x, 3), x)


def test_bad_arguments(gpu_ctx):
    L = P.load()
    d = gpu_ctx.alloc(1 << 12)
    assert L.p3g_dft(gpu_ctx.handle, P.BABYBEAR, 4, d.ptr, 4, 4, 0, 0, d.ptr + 2048, None) == 1
    assert L.p3g_dft(gpu_ctx.handle, P.BABYBEAR, P.DFT, d.ptr, 4, 4, 0, 0, d.ptr, None) == 1  # in == out
    assert L.p3g_dft(gpu_ctx.handle, P.BABYBEAR, P.COSET_DFT, d.ptr, 2, 2, 0, 0, d.ptr + 64, None) == 1
    # 2^27 rows is within the field's two-adicity but above the split transform's 2^26
    assert L.p3g_dft(gpu_ctx.handle, P.BABYBEAR, P.DFT, d.ptr, 27, 1, 0, 0, d.ptr + 64, None) == 5
    assert L.p3g_dft(gpu_ctx.handle, P.BABYBEAR, P.DFT, d.ptr, 28, 1, 0, 0, d.ptr + 64, None) == 1
    assert L.p3g_dft(gpu_ctx.handle, 7, P.DFT, d.ptr, 2, 2, 0, 0, d.ptr + 64, None) == 1
    d.free()
