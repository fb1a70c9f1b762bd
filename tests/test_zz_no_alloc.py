"""The allocation-free BabyBear LDE entry point (p3g_coset_lde_bb_noalloc).

It exists for callers that must not enter the CUDA allocator while they prove
(a service that reserves its device memory up front, or a host whose own
memory manager owns the GPU): it keeps its scratch in a fixed device array
instead of the context pool.  These tests call it through the C ABI and
compare every output element with the allocating entry point p3g_coset_lde
and with the oracle on the same inputs, for two calls in a row (the array
keeps the previous call's contents, which must not leak into the next
result), and check that warm calls leave the device's free memory
unchanged.  This file is collected last on purpose; it also passes alone in
a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
import p3g_gb300 as P

pytestmark = pytest.mark.gpu

BB_P = 0x78000001


def _noalloc(ctx, d_in, log_h, w, log_b, shift, bitrev, d_out):
    return P.load().p3g_coset_lde_bb_noalloc(d_in, log_h, w, log_b, shift, int(bitrev), d_out, None)


@pytest.mark.parametrize("log_h,w,log_b,bitrev", [(9, 24, 1, True), (14, 40, 1, True), (13, 17, 2, False)])
def test_noalloc_matches_allocating_lde_two_calls(log_h, w, log_b, bitrev):
    rng = np.random.default_rng(log_h * 100 + w)
    with P.Context(0) as ctx:
        H = 1 << (log_h + log_b)
        for call in range(2):
            t = rng.integers(0, BB_P, size=(1 << log_h, w), dtype=np.uint32)
            shift = int(rng.integers(1, BB_P))
            d_in = ctx.to_device(t)
            d_ref = ctx.alloc(H * w * 4)
            d_out = ctx.alloc(H * w * 4)
            ctx.coset_lde_device(P.BABYBEAR, d_in.ptr, log_h, w, log_b, shift, bitrev, d_ref.ptr)
            rc = _noalloc(ctx, d_in.ptr, log_h, w, log_b, shift, bitrev, d_out.ptr)
            P.check(rc)
            ref = d_ref.download(np.uint32, (H, w))
            got = d_out.download(np.uint32, (H, w))
            assert np.array_equal(got, ref), (log_h, w, log_b, bitrev, call)
            # and against the oracle's restatement of Radix2Dit::coset_lde_batch directly
            assert np.array_equal(got, O.bb_coset_lde(t, log_b, shift, bitrev)), (log_h, w, log_b, bitrev, call)
            for b in (d_in, d_ref, d_out):
                b.free()


def test_noalloc_leaves_free_device_memory_unchanged():
    """After a first call (which loads the kernels), further calls take no
    device memory: the free byte count is the same before and after."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    log_h, w, log_b = 12, 16, 1
    H = 1 << (log_h + log_b)
    with P.Context(0) as ctx:
        t = rng.integers(0, BB_P, size=(1 << log_h, w), dtype=np.uint32)
        d_in = ctx.to_device(t)
        d_out = ctx.alloc(H * w * 4)
        ctx.sync()
        P.check(_noalloc(ctx, d_in.ptr, log_h, w, log_b, 31, True, d_out.ptr))
        ctx.sync()
        free0 = torch.cuda.mem_get_info(0)[0]
        for _ in range(3):
            P.check(_noalloc(ctx, d_in.ptr, log_h, w, log_b, 31, True, d_out.ptr))
        ctx.sync()
        assert torch.cuda.mem_get_info(0)[0] == free0
        assert np.array_equal(d_out.download(np.uint32, (H, w)), O.bb_coset_lde(t, log_b, 31, True))
        d_in.free()
        d_out.free()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    with P.Context(0) as ctx:
        d = ctx.alloc(64)
        rc = _noalloc(ctx, d.ptr, 20, 256, 1, 31, True, d.ptr)
        assert rc == 1
        buf = C.create_string_buffer(512)
        P.load().p3g_last_error(buf, 512)
        assert b"fixed maximum" in buf.value
        d.free()
