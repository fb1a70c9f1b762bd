"""p3g_ctx_memory: the context pool's statistics follow its allocations."""
import pytest

pytestmark = pytest.mark.gpu


def test_pool_statistics_follow_allocations(gpu_ctx):
    gpu_ctx.sync()
    before = gpu_ctx.memory()
    assert before["reserved"] >= before["used"] >= 0
    buf = gpu_ctx.alloc(64 << 20)
    gpu_ctx.sync()
    during = gpu_ctx.memory()
    assert during["used"] >= before["used"] + (64 << 20)
    assert during["reserved"] >= during["used"]
    assert during["used_high"] >= during["used"] and during["reserved_high"] >= during["reserved"]
    buf.free()
    gpu_ctx.sync()
    after = gpu_ctx.memory()
    assert after["used"] == before["used"]
    assert after["reserved"] >= after["used"]  # the pool keeps what it reserved

