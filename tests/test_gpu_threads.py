"""Distinct contexts are independent (the threading rule of include/p3g.h): two
host threads, each with its own context and stream, commit different traces
and grind at the same time (ctypes releases the interpreter lock during each
call), and every result equals the one a single thread gets."""
import threading

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu


def _work(ctx, seed, out, errors):
    try:
        rng = np.random.default_rng(seed)
        roots = []
        for k in range(6):
            t = rng.integers(0, O.BB_P, size=(1 << 14, 24 + 8 * k), dtype=np.uint32)
            d = ctx.to_device(t)
            cap = np.zeros((1, 8), np.uint32)
            tree = ctx.commit_traces_device(P.BABYBEAR, [(d.ptr, 14, t.shape[1], 1, 31)], 0, cap_out=cap)
            roots.append(cap[0].copy())
            tree.free()
            d.free()
        st = rng.integers(0, O.BB_P, size=16, dtype=np.uint32)
        roots.append(np.array([ctx.grind(P.BABYBEAR, st, [], 14)], np.uint64))
        out[seed] = roots
    except Exception as e:  # reported by the main thread
        errors.append(e)


def test_two_contexts_on_two_threads():
    ctxs = [P.Context(0), P.Context(0)]
    for c in ctxs:
        c.set_default_poseidon2()
    alone, errors = {}, []
    for seed, c in zip((1, 2), ctxs):
        _work(c, seed, alone, errors)
    together = {}
    threads = [threading.Thread(target=_work, args=(c, seed, together, errors)) for seed, c in zip((1, 2), ctxs)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for seed in (1, 2):
        assert len(together[seed]) == len(alone[seed])
        for a, b in zip(together[seed], alone[seed]):
            assert np.array_equal(a, b), seed
    for c in ctxs:
        c.close()
