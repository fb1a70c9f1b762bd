"""GPU parity of the proof-of-work search (p3g_grind) with the reference's
DuplexChallenger::grind (duplex_challenger.hpp:234-251): the golden witnesses
the reference produced, the oracle's sequential search on random challenger
states (every pending-input count, both fields), and at search sizes the oracle
cannot reach, the defining property -- the witness passes, and a search bounded
by it finds nothing smaller."""
import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu


def _passes(params, state, pending, w, bits, rate):
    """observe_witness(w) + sample() on a copy of the challenger (oracle)."""
    s = np.array(state).copy()
    inp = list(pending) + [w & 0xFFFFFFFF, w >> 32]
    mod = O.BB_P if params.field == 0 else O.GL_P
    inp = [v % mod for v in inp]
    s[:min(len(inp), rate)] = inp[:rate]
    s = O.permute(params, s)
    if len(inp) > rate:
        s[0] = inp[rate]
        s = O.permute(params, s)
    return int(s[rate - 1]) & ((1 << bits) - 1) == 0


def test_grind_golden(gpu_ctx, golden):
    p = O.bb16_params()
    for c in golden["grind"]:
        tr = O.Transcript(p)
        for v in O.mt19937(c["seed"], c["n_obs"]):
            tr.observe(int(v) % O.BB_P)
        for bits, w, after in zip(c["bits"], c["witness"], c["sample_after"]):
            got = gpu_ctx.grind(P.BABYBEAR, tr.state, tr.inp, bits)
            assert got == w, (c, bits)
            assert tr.check_witness(bits, got)
            assert tr.sample() == after


@pytest.mark.parametrize("field", [P.BABYBEAR, P.GOLDILOCKS])
def test_grind_matches_oracle_every_pending_count(gpu_ctx, field):
    params = O.bb16_params() if field == P.BABYBEAR else O.gl8_params()
    width, rate = (16, 8) if field == P.BABYBEAR else (8, 4)
    rng = np.random.default_rng(40 + field)
    for k in range(rate):
        for bits in (3, 11, 15):
            if field == P.BABYBEAR:
                st = rng.integers(0, O.BB_P, size=width, dtype=np.uint32)
                pend = [int(x) for x in rng.integers(0, O.BB_P, size=k, dtype=np.uint32)]
            else:
                st = rng.integers(0, O.GL_P, size=width, dtype=np.uint64)
                pend = [int(x) for x in rng.integers(0, O.GL_P, size=k, dtype=np.uint64)]
            got = gpu_ctx.grind(field, st, pend, bits)
            assert got == O.grind(params, st, pend, bits), (field, k, bits)


@pytest.mark.parametrize("bits", [22, 26])
def test_grind_large_is_smallest_passing_witness(gpu_ctx, bits):
    """2^22 and 2^26 expected candidates: the witness passes (checked by the
    oracle's permutation) and the GPU search bounded below it finds none."""
    p = O.bb16_params()
    rng = np.random.default_rng(bits)
    for k in (0, 7):
        st = rng.integers(0, O.BB_P, size=16, dtype=np.uint32)
        pend = [int(x) for x in rng.integers(0, O.BB_P, size=k, dtype=np.uint32)]
        w = gpu_ctx.grind(P.BABYBEAR, st, pend, bits)
        assert _passes(p, st, pend, w, bits, 8)
        if w > 0:
            with pytest.raises(P.P3GError) as e:
                gpu_ctx.grind(P.BABYBEAR, st, pend, bits, max_witness=w)
            assert e.value.status == 7  # P3G_ENOTFOUND


def test_grind_low_half_is_reduced(gpu_ctx):
    """BabyBear(uint32_t) takes its argument mod p (baby_bear.hpp:51), so the
    witnesses w and w + p sample the same element: the smallest passing
    witness is below p and its alias passes too (oracle)."""
    p = O.bb16_params()
    st = np.random.default_rng(9).integers(0, O.BB_P, size=16, dtype=np.uint32)
    w = gpu_ctx.grind(P.BABYBEAR, st, [], 10)
    assert w < O.BB_P
    assert _passes(p, st, [], w + O.BB_P, 10, 8)


def test_grind_arguments(gpu_ctx):
    st = np.zeros(16, np.uint32)
    assert gpu_ctx.grind(P.BABYBEAR, st, [], 0) == 0  # a zero-bit mask accepts witness 0
    for bad in (dict(bits=31), dict(pending=[1] * 8), dict(state_val=O.BB_P)):
        s = st.copy()
        if "state_val" in bad:
            s[3] = bad["state_val"]
        with pytest.raises(P.P3GError) as e:
            gpu_ctx.grind(P.BABYBEAR, s, bad.get("pending", []), bad.get("bits", 4))
        assert e.value.status == 1
    with pytest.raises(P.P3GError) as e:
        gpu_ctx.grind(P.GOLDILOCKS, np.zeros(8, np.uint64), [1, 2, 3, 4], 4)
    assert e.value.status == 1
    with pytest.raises(P.P3GError) as e:
        gpu_ctx.grind(P.GOLDILOCKS, np.zeros(8, np.uint64), [], 64)
    assert e.value.status == 1
