"""ctypes binding of libp3g_gb300.so (the C ABI declared in include/p3g.h).

This is the thin host-side mirror used by the tests, ``__graft_entry__`` and
bench.py: every call goes through the C ABI into the CUDA library.  There is
no CPU fallback -- if the library cannot be loaded or a call fails, an
exception is raised.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libp3g_gb300.so")

BABYBEAR = 0
GOLDILOCKS = 1
BB_P = 0x78000001
GL_P = 0xFFFFFFFF00000001

EXPORTS = [
    "p3g_version", "p3g_status_string", "p3g_last_error", "p3g_kernel_launches", "p3g_ctx_create", "p3g_ctx_destroy",
    "p3g_stream_synchronize", "p3g_malloc", "p3g_free", "p3g_memcpy_h2d", "p3g_memcpy_d2h",
    "p3g_set_poseidon2", "p3g_poseidon2_permute", "p3g_coset_lde", "p3g_dft", "p3g_mmcs_commit",
    "p3g_commit_matrix", "p3g_tree_info", "p3g_tree_layer_ptr", "p3g_tree_leaf_ptr",
    "p3g_mmcs_open_batch", "p3g_tree_free", "p3g_commit_traces", "p3g_commit_traces_host", "p3g_fold_matrix_bb4",
    "p3g_coset_lde_bb_noalloc", "p3g_plan_commit", "p3g_plan_commit_host", "p3g_plan_launch", "p3g_plan_info",
    "p3g_plan_destroy", "p3g_server_create", "p3g_server_submit", "p3g_server_poll",
    "p3g_server_pending", "p3g_server_open", "p3g_server_read_fold", "p3g_server_release", "p3g_server_destroy",
    "p3g_pcs_open_values", "p3g_pcs_reduce", "p3g_bb4_axpy", "p3g_grind", "p3g_fri_rounds", "p3g_fri_prove", "p3g_ctx_memory",
]


# p3g_dft kinds
DFT, IDFT, COSET_DFT, COSET_IDFT = 0, 1, 2, 3


class P3GError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"p3g status {status}: {msg}")
        self.status = status


class FriParams(C.Structure):
    _fields_ = [("log_blowup", C.c_uint32), ("log_final_poly_len", C.c_uint32), ("max_log_arity", C.c_uint32),
                ("num_queries", C.c_uint32), ("commit_proof_of_work_bits", C.c_uint32),
                ("query_proof_of_work_bits", C.c_uint32)]


class Challenger(C.Structure):
    _fields_ = [("sponge_state", C.c_uint32 * 16), ("input", C.c_uint32 * 8), ("output", C.c_uint32 * 8),
                ("n_input", C.c_uint32), ("n_output", C.c_uint32)]


class Matrix(C.Structure):
    _fields_ = [("d_data", C.c_void_p), ("height", C.c_uint64), ("width", C.c_uint32),
                ("reserved", C.c_uint32)]


class FoldJob(C.Structure):
    _fields_ = [("d_in", C.c_void_p), ("d_out", C.c_void_p), ("log_height", C.c_uint32),
                ("log_arity", C.c_uint32), ("beta", C.c_uint32 * 4)]


class Request(C.Structure):
    _fields_ = [("id", C.c_uint64), ("h_trace", C.c_void_p), ("log_h", C.c_uint32), ("width", C.c_uint32),
                ("log_blowup", C.c_uint32), ("reserved", C.c_uint32), ("shift", C.c_uint64),
                ("beta", C.c_uint32 * 4)]


class Result(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("reserved", C.c_uint32),
                ("root", C.c_uint32 * 8), ("fold_head", C.c_uint32 * 4),
                ("t_submit_ns", C.c_uint64), ("t_admit_ns", C.c_uint64), ("t_done_ns", C.c_uint64)]


class Trace(C.Structure):
    _fields_ = [("d_trace", C.c_void_p), ("log_h", C.c_uint32), ("width", C.c_uint32),
                ("log_blowup", C.c_uint32), ("reserved", C.c_uint32), ("shift", C.c_uint64)]


_lib = None


def load(path: str | None = None):
    """Loads the library; raises if it is missing (build it with build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libp3g_gb300.so not built at {p}; run plonky3-gpu_gb300/build.py")
    L = C.CDLL(p)
    vp, sz, i32, u32, u64 = C.c_void_p, C.c_size_t, C.c_int, C.c_uint32, C.c_uint64
    L.p3g_version.restype = i32
    L.p3g_status_string.restype = C.c_char_p
    L.p3g_status_string.argtypes = [i32]
    L.p3g_last_error.argtypes = [C.c_char_p, sz]
    L.p3g_kernel_launches.restype = u64
    L.p3g_kernel_launches.argtypes = []
    L.p3g_ctx_create.argtypes = [i32, C.POINTER(vp)]
    L.p3g_ctx_destroy.argtypes = [vp]
    L.p3g_stream_synchronize.argtypes = [vp, vp]
    L.p3g_malloc.argtypes = [vp, sz, C.POINTER(vp), vp]
    L.p3g_free.argtypes = [vp, vp, vp]
    L.p3g_memcpy_h2d.argtypes = [vp, vp, vp, sz, vp]
    L.p3g_memcpy_d2h.argtypes = [vp, vp, vp, sz, vp]
    L.p3g_set_poseidon2.argtypes = [vp, i32, u32, u32, u32, u32, vp, vp, vp]
    L.p3g_poseidon2_permute.argtypes = [vp, i32, vp, sz, vp]
    L.p3g_coset_lde.argtypes = [vp, i32, vp, u32, u32, u32, u64, i32, vp, vp]
    L.p3g_dft.argtypes = [vp, i32, i32, vp, u32, u32, u64, i32, vp, vp]
    L.p3g_mmcs_commit.argtypes = [vp, i32, C.POINTER(Matrix), sz, u32, C.POINTER(vp), vp, vp]
    L.p3g_commit_matrix.argtypes = [vp, i32, vp, u64, u32, C.POINTER(vp), vp, vp]
    L.p3g_tree_info.argtypes = [vp, C.POINTER(u32), C.POINTER(u64), C.POINTER(u32)]
    L.p3g_tree_layer_ptr.argtypes = [vp, u32, C.POINTER(vp)]
    L.p3g_tree_leaf_ptr.argtypes = [vp, u32, C.POINTER(vp)]
    L.p3g_mmcs_open_batch.argtypes = [vp, vp, vp, sz, vp, vp, vp]
    L.p3g_tree_free.argtypes = [vp, vp, vp]
    L.p3g_commit_traces.argtypes = [vp, i32, C.POINTER(Trace), sz, u32, C.POINTER(vp), vp, vp]
    L.p3g_commit_traces_host.argtypes = [vp, i32, C.POINTER(Trace), sz, u32, C.POINTER(vp), vp, vp]
    L.p3g_fold_matrix_bb4.argtypes = [vp, vp, u32, u32, vp, vp, vp]
    L.p3g_coset_lde_bb_noalloc.argtypes = [vp, u32, u32, u32, u32, i32, vp, vp]
    L.p3g_plan_commit.argtypes = [vp, i32, C.POINTER(Trace), sz, u32, C.POINTER(FoldJob), u32, C.POINTER(vp)]
    L.p3g_plan_commit_host.argtypes = L.p3g_plan_commit.argtypes
    L.p3g_plan_launch.argtypes = [vp, vp, vp]
    L.p3g_plan_info.argtypes = [vp, C.POINTER(vp), C.POINTER(u32), C.POINTER(u64)]
    L.p3g_plan_destroy.argtypes = [vp, vp]
    L.p3g_server_create.argtypes = [vp, u32, u64, C.POINTER(vp)]
    L.p3g_server_submit.argtypes = [vp, C.POINTER(Request)]
    L.p3g_server_poll.argtypes = [vp, C.POINTER(Result), sz, C.POINTER(sz)]
    L.p3g_server_pending.argtypes = [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)]
    L.p3g_server_open.argtypes = [vp, u64, vp, sz, vp, vp]
    L.p3g_server_read_fold.argtypes = [vp, u64, vp, u64]
    L.p3g_server_release.argtypes = [vp, u64]
    L.p3g_server_destroy.argtypes = [vp]
    L.p3g_pcs_open_values.argtypes = [vp, vp, u32, u32, i32, u32, vp, u32, vp, vp]
    L.p3g_bb4_axpy.argtypes = [vp, vp, vp, u64, vp, vp]
    L.p3g_grind.argtypes = [vp, C.c_int, vp, vp, u32, u32, u64, vp, vp]
    L.p3g_fri_rounds.argtypes = [vp, u32, vp, vp, vp]
    L.p3g_ctx_memory.argtypes = [vp, vp, vp, vp, vp]
    L.p3g_fri_prove.argtypes = [vp, vp, vp, u32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.p3g_pcs_reduce.argtypes = [vp, vp, u32, u32, i32, u32, vp, u32, vp, vp, u64, i32, vp, vp]
    for name in EXPORTS:
        if name not in ("p3g_version", "p3g_status_string", "p3g_kernel_launches"):
            getattr(L, name).restype = i32
    _lib = L
    return L


def kernel_launches() -> int:
    return int(load().p3g_kernel_launches())


def check(status: int):
    if status != 0:
        buf = C.create_string_buffer(1024)
        load().p3g_last_error(buf, 1024)
        raise P3GError(status, buf.value.decode(errors="replace"))


def _np_ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ----------------------------------------------------------------- MT19937 (for constants)
def mt19937(seed: int, n: int) -> list[int]:
    """std::mt19937 outputs (the published Mersenne Twister)."""
    mt = [0] * 624
    mt[0] = seed & 0xFFFFFFFF
    for i in range(1, 624):
        mt[i] = (1812433253 * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
    out, idx = [], 624
    for _ in range(n):
        if idx >= 624:
            for i in range(624):
                y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            idx = 0
        y = mt[idx]
        idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        out.append(y & 0xFFFFFFFF)
    return out


def mt19937_64(seed: int, n: int) -> list[int]:
    """std::mt19937_64 outputs."""
    M = 0xFFFFFFFFFFFFFFFF
    mt = [0] * 312
    mt[0] = seed & M
    for i in range(1, 312):
        mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & M
    out, idx = [], 312
    for _ in range(n):
        if idx >= 312:
            for i in range(312):
                y = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
                mt[i] = mt[(i + 156) % 312] ^ (y >> 1) ^ (0xB5026F5AA96619E9 if y & 1 else 0)
            idx = 0
        x = mt[idx]
        idx += 1
        x ^= (x >> 29) & 0x5555555555555555
        x ^= (x << 17) & 0x71D67FFFEDA60000
        x ^= (x << 37) & 0xFFF7EEE000000000
        x ^= x >> 43
        out.append(x & M)
    return out


def seeded_constants_bb16(rounds_p: int = 13):
    """Poseidon2 BabyBear-16 constants drawn from std::mt19937(0xdeadbeef), initial and
    terminal interleaved per (round, lane), then the partial-round constants -- the
    convention of the reference's CUDA Merkle example."""
    raw = mt19937(0xDEADBEEF, 2 * 4 * 16 + rounds_p)
    ini = np.array([raw[2 * k] % BB_P for k in range(64)], np.uint32)
    ter = np.array([raw[2 * k + 1] % BB_P for k in range(64)], np.uint32)
    inr = np.array([raw[128 + r] % BB_P for r in range(rounds_p)], np.uint32)
    return ini, ter, inr


def seeded_constants_gl8(rounds_p: int = 22):
    """Goldilocks-8 constants from std::mt19937_64(12345), same draw order."""
    raw = mt19937_64(12345, 2 * 4 * 8 + rounds_p)
    ini = np.array([raw[2 * k] % GL_P for k in range(32)], np.uint64)
    ter = np.array([raw[2 * k + 1] % GL_P for k in range(32)], np.uint64)
    inr = np.array([raw[64 + r] % GL_P for r in range(rounds_p)], np.uint64)
    return ini, ter, inr


# ----------------------------------------------------------------- device buffers
class DeviceBuffer:
    """A device allocation from the context pool."""

    def __init__(self, ctx: "Context", nbytes: int, stream=None):
        self.ctx = ctx
        self.nbytes = nbytes
        p = C.c_void_p()
        check(load().p3g_malloc(ctx.handle, max(nbytes, 1), C.byref(p), stream))
        self.ptr = p.value

    def upload(self, arr: np.ndarray, stream=None):
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        check(load().p3g_memcpy_h2d(self.ctx.handle, self.ptr, _np_ptr(a), a.nbytes, stream))
        return self

    def download(self, dtype, shape, stream=None) -> np.ndarray:
        out = np.empty(shape, dtype=dtype)
        check(load().p3g_memcpy_d2h(self.ctx.handle, _np_ptr(out), self.ptr, out.nbytes, stream))
        return out

    def free(self, stream=None):
        if self.ptr:
            check(load().p3g_free(self.ctx.handle, self.ptr, stream))
            self.ptr = None


class Tree:
    def __init__(self, ctx: "Context", handle: int, field: int):
        self.ctx, self.handle, self.field = ctx, handle, field

    def info(self):
        n = C.c_uint32()
        sizes = (C.c_uint64 * 64)()
        dig = C.c_uint32()
        check(load().p3g_tree_info(self.handle, C.byref(n), sizes, C.byref(dig)))
        return [int(sizes[i]) for i in range(n.value)], dig.value

    def layers(self):
        sizes, dig = self.info()
        dt = np.uint32 if self.field == BABYBEAR else np.uint64
        out = []
        for i, s in enumerate(sizes):
            p = C.c_void_p()
            check(load().p3g_tree_layer_ptr(self.handle, i, C.byref(p)))
            arr = np.empty((s, dig), dtype=dt)
            check(load().p3g_memcpy_d2h(self.ctx.handle, _np_ptr(arr), p, arr.nbytes, None))
            out.append(arr)
        return out

    def layer_ptr(self, i: int) -> int:
        """Device pointer of digest layer i (0 = leaves; the last is the cap)."""
        p = C.c_void_p()
        check(load().p3g_tree_layer_ptr(self.handle, i, C.byref(p)))
        return p.value

    def leaf_ptr(self, i: int) -> int:
        p = C.c_void_p()
        check(load().p3g_tree_leaf_ptr(self.handle, i, C.byref(p)))
        return p.value

    def open_batch(self, indices, row_elems: int):
        sizes, dig = self.info()
        dt = np.uint32 if self.field == BABYBEAR else np.uint64
        idx = np.ascontiguousarray(indices, dtype=np.uint64)
        rows = np.zeros((idx.size, row_elems), dtype=dt)
        proof = np.zeros((idx.size, len(sizes) - 1, dig), dtype=dt)
        check(load().p3g_mmcs_open_batch(self.ctx.handle, self.handle, _np_ptr(idx), idx.size,
                                         _np_ptr(rows), _np_ptr(proof), None))
        return rows, proof

    def free(self, stream=None):
        if self.handle:
            check(load().p3g_tree_free(self.ctx.handle, self.handle, stream))
            self.handle = None


class Plan:
    """A batched commit captured as one CUDA graph (p3g_plan_*).  With
    host=True the trace pointers and the fold input are pinned host memory
    (p3g_plan_commit_host): every launch copies them in."""

    def __init__(self, ctx: "Context", field: int, traces, cap_height: int = 0, fold=None,
                 n_streams: int = 0, host: bool = False):
        self.ctx, self.field = ctx, field
        arr = (Trace * len(traces))(*[Trace(p, lh, w, lb, 0, s) for (p, lh, w, lb, s) in traces])
        fj = None
        if fold is not None:
            d_in, d_out, lh, la, beta = fold
            fj = FoldJob(d_in, d_out, lh, la, (C.c_uint32 * 4)(*[int(b) for b in beta]))
        h = C.c_void_p()
        fn = load().p3g_plan_commit_host if host else load().p3g_plan_commit
        check(fn(ctx.handle, field, arr, len(traces), cap_height, C.byref(fj) if fj is not None else None,
                 n_streams, C.byref(h)))
        self.handle = h.value
        t = C.c_void_p()
        ns = C.c_uint32()
        kl = C.c_uint64()
        check(load().p3g_plan_info(self.handle, C.byref(t), C.byref(ns), C.byref(kl)))
        self.tree = Tree(ctx, t.value, field)
        self.n_streams = ns.value
        self.kernels_per_launch = kl.value

    def launch(self, stream=None):
        check(load().p3g_plan_launch(self.ctx.handle, self.handle, stream))

    def destroy(self):
        if self.handle:
            check(load().p3g_plan_destroy(self.ctx.handle, self.handle))
            self.handle = None


class Server:
    """Continuous-batching commit+fold service (p3g_server_*)."""

    def __init__(self, ctx: "Context", max_slots: int = 4, mem_budget: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        check(load().p3g_server_create(ctx.handle, max_slots, mem_budget, C.byref(h)))
        self.handle = h.value

    def submit(self, rid: int, h_trace_ptr: int, log_h: int, width: int, log_blowup: int, shift: int, beta):
        r = Request(rid, h_trace_ptr, log_h, width, log_blowup, 0, shift,
                    (C.c_uint32 * 4)(*[int(b) for b in beta]))
        check(load().p3g_server_submit(self.handle, C.byref(r)))

    def poll(self, max_results: int = 256):
        arr = (Result * max_results)()
        n = C.c_size_t()
        check(load().p3g_server_poll(self.handle, arr, max_results, C.byref(n)))
        return [arr[i] for i in range(n.value)]

    def pending(self):
        q, f, r, b = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(load().p3g_server_pending(self.handle, C.byref(q), C.byref(f), C.byref(r), C.byref(b)))
        return q.value, f.value, r.value, b.value

    def open(self, rid: int, indices, width: int, nlayers: int):
        idx = np.ascontiguousarray(indices, dtype=np.uint64)
        rows = np.zeros((idx.size, width), np.uint32)
        proof = np.zeros((idx.size, max(nlayers - 1, 0), 8), np.uint32)
        check(load().p3g_server_open(self.handle, rid, _np_ptr(idx), idx.size, _np_ptr(rows), _np_ptr(proof)))
        return rows, proof

    def read_fold(self, rid: int, lde_height: int) -> np.ndarray:
        """The request's resident fold output: lde_height / 2 BabyBear^4 values."""
        out = np.zeros((lde_height // 2, 4), np.uint32)
        check(load().p3g_server_read_fold(self.handle, rid, _np_ptr(out), lde_height // 2))
        return out

    def release(self, rid: int):
        check(load().p3g_server_release(self.handle, rid))

    def close(self):
        if self.handle:
            check(load().p3g_server_destroy(self.handle))
            self.handle = None


class Context:
    """Owns a p3g_ctx on one device."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(load().p3g_ctx_create(device, C.byref(h)))
        self.handle = h.value

    def close(self):
        if self.handle:
            check(load().p3g_ctx_destroy(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def sync(self, stream=None):
        check(load().p3g_stream_synchronize(self.handle, stream))

    # -- buffers
    def alloc(self, nbytes: int, stream=None) -> DeviceBuffer:
        return DeviceBuffer(self, nbytes, stream)

    def to_device(self, arr: np.ndarray, stream=None) -> DeviceBuffer:
        a = np.ascontiguousarray(arr)
        return DeviceBuffer(self, a.nbytes, stream).upload(a, stream)

    # -- Poseidon2
    def set_poseidon2(self, field: int, width: int, rounds_f: int, rounds_p: int, degree: int,
                      initial, terminal, internal):
        dt = np.uint32 if field == BABYBEAR else np.uint64
        ini = np.ascontiguousarray(initial, dtype=dt).reshape(-1)
        ter = np.ascontiguousarray(terminal, dtype=dt).reshape(-1)
        inr = np.ascontiguousarray(internal, dtype=dt).reshape(-1)
        if inr.size == 0:
            inr = np.zeros(1, dt)
        check(load().p3g_set_poseidon2(self.handle, field, width, rounds_f, rounds_p, degree,
                                       _np_ptr(ini), _np_ptr(ter), _np_ptr(inr)))

    def set_default_poseidon2(self):
        """BabyBear-16 x^7 8+13 and Goldilocks-8 x^7 8+22 with the seeded constants."""
        self.set_poseidon2(BABYBEAR, 16, 8, 13, 7, *seeded_constants_bb16(13))
        self.set_poseidon2(GOLDILOCKS, 8, 8, 22, 7, *seeded_constants_gl8(22))

    def permute(self, field: int, states: np.ndarray) -> np.ndarray:
        dt = np.uint32 if field == BABYBEAR else np.uint64
        s = np.ascontiguousarray(states, dtype=dt)
        d = self.to_device(s)
        check(load().p3g_poseidon2_permute(self.handle, field, d.ptr, s.shape[0], None))
        out = d.download(dt, s.shape)
        d.free()
        return out

    # -- LDE
    def coset_lde_device(self, field: int, d_in: int, log_h: int, width: int, log_blowup: int,
                         shift: int, bitrev: bool, d_out: int, stream=None):
        check(load().p3g_coset_lde(self.handle, field, d_in, log_h, width, log_blowup, shift,
                                   int(bitrev), d_out, stream))

    def coset_lde(self, trace: np.ndarray, log_blowup: int, shift: int | None = None,
                  bitrev: bool = True) -> np.ndarray:
        field = BABYBEAR if trace.dtype == np.uint32 else GOLDILOCKS
        if shift is None:
            shift = 31 if field == BABYBEAR else 7
        h, w = trace.shape
        log_h = h.bit_length() - 1
        assert 1 << log_h == h
        din = self.to_device(trace)
        dout = self.alloc((h << log_blowup) * w * trace.itemsize)
        self.coset_lde_device(field, din.ptr, log_h, w, log_blowup, shift, bitrev, dout.ptr)
        out = dout.download(trace.dtype, (h << log_blowup, w))
        din.free()
        dout.free()
        return out

    # -- dft / idft / coset_dft / coset_idft
    def dft_device(self, field: int, kind: int, d_in: int, log_h: int, width: int, shift: int, bitrev: bool,
                   d_out: int, stream=None):
        check(load().p3g_dft(self.handle, field, kind, d_in, log_h, width, shift, int(bitrev), d_out, stream))

    def dft(self, kind: int, mat: np.ndarray, shift: int = 0, bitrev: bool = False) -> np.ndarray:
        """kind: DFT, IDFT, COSET_DFT or COSET_IDFT; natural order unless bitrev."""
        field = BABYBEAR if mat.dtype == np.uint32 else GOLDILOCKS
        h, w = mat.shape
        log_h = h.bit_length() - 1
        assert 1 << log_h == h
        din = self.to_device(mat)
        dout = self.alloc(max(h * w * mat.itemsize, 1))
        try:
            self.dft_device(field, kind, din.ptr, log_h, w, shift, bitrev, dout.ptr)
            return dout.download(mat.dtype, (h, w))
        finally:
            din.free()
            dout.free()

    # -- MMCS
    def mmcs_commit_device(self, field: int, mats, cap_height: int = 0, stream=None) -> Tree:
        """mats: list of (device_ptr, height, width)."""
        arr = (Matrix * len(mats))(*[Matrix(p, h, w, 0) for (p, h, w) in mats])
        t = C.c_void_p()
        check(load().p3g_mmcs_commit(self.handle, field, arr, len(mats), cap_height, C.byref(t), None, stream))
        return Tree(self, t.value, field)

    def mmcs_commit(self, mats, cap_height: int = 0):
        """Host matrices in; returns (layers, tree, device buffers)."""
        field = BABYBEAR if mats[0].dtype == np.uint32 else GOLDILOCKS
        bufs = [self.to_device(m) for m in mats]
        tree = self.mmcs_commit_device(field, [(b.ptr, m.shape[0], m.shape[1]) for b, m in zip(bufs, mats)],
                                       cap_height)
        return tree, bufs

    def commit_matrix(self, mat: np.ndarray):
        field = BABYBEAR if mat.dtype == np.uint32 else GOLDILOCKS
        buf = self.to_device(mat)
        t = C.c_void_p()
        check(load().p3g_commit_matrix(self.handle, field, buf.ptr, mat.shape[0], mat.shape[1], C.byref(t),
                                       None, None))
        return Tree(self, t.value, field), buf

    def commit_matrix_device(self, field: int, d_flat: int, height: int, width: int, stream=None) -> Tree:
        """Flat MMCS commit_matrix of a device matrix (height x width)."""
        t = C.c_void_p()
        check(load().p3g_commit_matrix(self.handle, field, d_flat, height, width, C.byref(t), None, stream))
        return Tree(self, t.value, field)

    def commit_traces_device(self, field: int, traces, cap_height: int = 0, stream=None,
                             cap_out: np.ndarray | None = None) -> Tree:
        """traces: list of (device_ptr, log_h, width, log_blowup, shift)."""
        arr = (Trace * len(traces))(*[Trace(p, lh, w, lb, 0, s) for (p, lh, w, lb, s) in traces])
        t = C.c_void_p()
        capp = _np_ptr(cap_out) if cap_out is not None else None
        check(load().p3g_commit_traces(self.handle, field, arr, len(traces), cap_height, C.byref(t), capp, stream))
        return Tree(self, t.value, field)

    def commit_traces_host(self, field: int, traces, cap_height: int = 0, stream=None,
                           cap_out: np.ndarray | None = None) -> Tree:
        """traces: list of (host_ptr, log_h, width, log_blowup, shift); host
        memory should be pinned for the copies to overlap the LDEs."""
        arr = (Trace * len(traces))(*[Trace(p, lh, w, lb, 0, s) for (p, lh, w, lb, s) in traces])
        t = C.c_void_p()
        capp = _np_ptr(cap_out) if cap_out is not None else None
        check(load().p3g_commit_traces_host(self.handle, field, arr, len(traces), cap_height, C.byref(t), capp,
                                            stream))
        return Tree(self, t.value, field)

    def bb4_axpy_device(self, d_y: int, d_x: int, n: int, a, stream=None):
        """y += a * x for n BabyBear^4 values on the device."""
        aa = np.ascontiguousarray(a, dtype=np.uint32).reshape(4)
        check(load().p3g_bb4_axpy(self.handle, d_y, d_x, n, _np_ptr(aa), stream))

    # -- memory
    def memory(self) -> dict:
        """The context pool's reserved and used bytes, current and peak."""
        v = [C.c_uint64() for _ in range(4)]
        check(load().p3g_ctx_memory(self.handle, *[C.byref(x) for x in v]))
        return dict(zip(("reserved", "used", "reserved_high", "used_high"), (x.value for x in v)))

    # -- proof of work
    def grind(self, field: int, sponge_state, pending, bits: int, max_witness: int = 0, stream=None) -> int:
        """DuplexChallenger::grind from the challenger's sponge state and
        pending inputs: the smallest passing witness."""
        dt = np.uint32 if field == BABYBEAR else np.uint64
        st = np.ascontiguousarray(sponge_state, dtype=dt)
        inp = np.ascontiguousarray(pending, dtype=dt).reshape(-1)
        w = C.c_uint64()
        check(load().p3g_grind(self.handle, field, _np_ptr(st), _np_ptr(inp) if inp.size else None, inp.size,
                               bits, max_witness, C.byref(w), stream))
        return w.value

    # -- FRI prover with the transcript on the device
    def fri_prove_device(self, inputs, params: dict, state, pending, outputs, stream=None) -> dict:
        """prove_fri over device BabyBear^4 vectors: inputs = [(device ptr,
        log_height)], tallest first; the challenger's sponge state, pending
        inputs and pending outputs.  Returns the proof's parts and the
        challenger afterwards."""
        prm = FriParams(**params)
        lh = (C.c_uint32 * len(inputs))(*[h for _, h in inputs])
        nr = C.c_uint32()
        las = (C.c_uint32 * 32)()
        check(load().p3g_fri_rounds(lh, len(inputs), C.byref(prm), C.byref(nr), las))
        R, nq = nr.value, prm.num_queries
        arities = [las[r] for r in range(R)]
        heights, h = [], inputs[0][1]
        for la in arities:
            heights.append(h)
            h -= la
        ch = Challenger()
        ch.sponge_state[:] = [int(x) for x in state]
        for i, v in enumerate(pending):
            ch.input[i] = int(v)
        for i, v in enumerate(outputs):
            ch.output[i] = int(v)
        ch.n_input, ch.n_output = len(pending), len(outputs)
        commits = np.zeros((R, 8), np.uint32)
        wits = np.zeros(R, np.uint64)
        final = np.zeros((1 << prm.log_final_poly_len, 4), np.uint32)
        qw = C.c_uint64()
        qidx = np.zeros(max(nq, 1), np.uint64)
        rows_w = sum(nq * (4 << la) for la in arities)
        path_w = sum(nq * (hh - la) * 8 for hh, la in zip(heights, arities))
        rows = np.zeros(max(rows_w, 1), np.uint32)
        paths = np.zeros(max(path_w, 1), np.uint32)
        ptrs = (C.c_void_p * len(inputs))(*[p for p, _ in inputs])
        check(load().p3g_fri_prove(self.handle, ptrs, lh, len(inputs), C.byref(prm), C.byref(ch), _np_ptr(commits),
                                   _np_ptr(wits), _np_ptr(final), C.byref(qw), _np_ptr(qidx), _np_ptr(rows),
                                   _np_ptr(paths), stream))
        out_rows, out_paths, ro, po = [], [], 0, 0
        for hh, la in zip(heights, arities):
            out_rows.append(rows[ro:ro + nq * (4 << la)].reshape(nq, 4 << la))
            ro += nq * (4 << la)
            out_paths.append(paths[po:po + nq * (hh - la) * 8].reshape(nq, hh - la, 8))
            po += nq * (hh - la) * 8
        return {"log_arities": arities, "commits": commits, "commit_witnesses": wits, "final_poly": final,
                "query_witness": qw.value, "query_indices": qidx[:nq], "rows": out_rows, "paths": out_paths,
                "state": np.array(ch.sponge_state[:], np.uint32), "pending": list(ch.input[:ch.n_input]),
                "outputs": list(ch.output[:ch.n_output])}

    # -- PCS open
    def pcs_open_values_device(self, d_lde: int, log_n: int, width: int, bitrev_rows: bool, shift: int, points,
                               stream=None) -> np.ndarray:
        """Opened values (n_points x width x 4) of a resident BabyBear LDE."""
        pts = np.ascontiguousarray(points, dtype=np.uint32).reshape(-1, 4)
        out = np.zeros((pts.shape[0], width, 4), dtype=np.uint32)
        check(load().p3g_pcs_open_values(self.handle, d_lde, log_n, width, int(bitrev_rows), shift, _np_ptr(pts),
                                         pts.shape[0], _np_ptr(out), stream))
        return out

    def pcs_reduce_device(self, d_lde: int, log_n: int, width: int, bitrev_rows: bool, shift: int, points, opened,
                          alpha, alpha_pow: int, q_bitrev: bool, d_q: int, stream=None):
        """Adds one matrix's reduced opening into the device vector d_q (2^log_n x 4)."""
        pts = np.ascontiguousarray(points, dtype=np.uint32).reshape(-1, 4)
        ov = np.ascontiguousarray(opened, dtype=np.uint32).reshape(pts.shape[0], width, 4)
        a = np.ascontiguousarray(alpha, dtype=np.uint32).reshape(4)
        check(load().p3g_pcs_reduce(self.handle, d_lde, log_n, width, int(bitrev_rows), shift, _np_ptr(pts),
                                    pts.shape[0], _np_ptr(ov), _np_ptr(a), alpha_pow, int(q_bitrev), d_q, stream))

    # -- FRI
    def fold_matrix_bb4_device(self, d_in: int, log_height: int, log_arity: int, beta, d_out: int,
                               stream=None):
        b = np.ascontiguousarray(beta, dtype=np.uint32).reshape(4)
        check(load().p3g_fold_matrix_bb4(self.handle, d_in, log_height, log_arity, _np_ptr(b), d_out, stream))

    def fold_matrix_bb4(self, values: np.ndarray, log_height: int, log_arity: int, beta) -> np.ndarray:
        v = np.ascontiguousarray(values, dtype=np.uint32).reshape(-1, 4)
        din = self.to_device(v)
        n = (1 << log_height) >> log_arity
        dout = self.alloc(n * 16)
        self.fold_matrix_bb4_device(din.ptr, log_height, log_arity, beta, dout.ptr)
        out = dout.download(np.uint32, (n, 4))
        din.free()
        dout.free()
        return out
