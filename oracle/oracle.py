"""ctypes front end of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, by ``__graft_entry__.smoke()`` as
the checker, and by bench.py's CPU-baseline leg.  The product library never
imports this module.

Every function here wraps one restatement in oracle.c, which cites the
reference routine (dloghin/plonky3-gpu, src/include/...) it follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

BB_P = 0x78000001
GL_P = 0xFFFFFFFF00000001

MAX_HALF_F = 8
MAX_P = 32
MAX_W = 24


class P2Params(C.Structure):
    _fields_ = [
        ("field", C.c_int32),
        ("width", C.c_int32),
        ("rounds_f", C.c_int32),
        ("rounds_p", C.c_int32),
        ("degree", C.c_int32),
        ("rate", C.c_int32),
        ("digest", C.c_int32),
        ("pad_", C.c_int32),
        ("initial_rc", C.c_uint64 * (MAX_HALF_F * MAX_W)),
        ("terminal_rc", C.c_uint64 * (MAX_HALF_F * MAX_W)),
        ("internal_rc", C.c_uint64 * MAX_P),
    ]


_lib = None


def build() -> str:
    """Compile liboracle.so with the committed Makefile (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        u32, u64, sz, vp, i32 = C.c_uint32, C.c_uint64, C.c_size_t, C.c_void_p, C.c_int
        for n in ("orc_bb_add", "orc_bb_sub", "orc_bb_mul"):
            getattr(L, n).restype = u32
            getattr(L, n).argtypes = [u32, u32]
        L.orc_bb_pow.restype = u32
        L.orc_bb_pow.argtypes = [u32, u64]
        L.orc_bb_inv.restype = u32
        L.orc_bb_inv.argtypes = [u32]
        L.orc_bb_two_adic_generator.restype = u32
        L.orc_bb_two_adic_generator.argtypes = [C.c_uint]
        L.orc_pcs_open_values.restype = None
        L.orc_pcs_open_values.argtypes = [vp, C.c_uint, sz, u32, vp, vp, i32]
        L.orc_pcs_reduce.restype = None
        L.orc_pcs_reduce.argtypes = [vp, C.c_uint, sz, u32, vp, sz, vp, vp, u64, vp, i32]
        for n in ("orc_gl_add", "orc_gl_sub", "orc_gl_mul"):
            getattr(L, n).restype = u64
            getattr(L, n).argtypes = [u64, u64]
        L.orc_gl_pow.restype = u64
        L.orc_gl_pow.argtypes = [u64, u64]
        L.orc_gl_inv.restype = u64
        L.orc_gl_inv.argtypes = [u64]
        L.orc_gl_two_adic_generator.restype = u64
        L.orc_gl_two_adic_generator.argtypes = [C.c_uint]
        L.orc_bb4_mul.argtypes = [vp, vp, vp]
        L.orc_bb4_inv.argtypes = [vp, vp]
        L.orc_bb4_dth_root.restype = u32
        L.orc_mt19937.argtypes = [u32, vp, sz]
        L.orc_mt19937_64.argtypes = [u64, vp, sz]
        for n in ("orc_bb_dft_batch", "orc_bb_idft_batch", "orc_bb_reverse_rows",
                  "orc_gl_dft_batch", "orc_gl_idft_batch", "orc_gl_reverse_rows"):
            getattr(L, n).argtypes = [vp, C.c_uint, sz]
        L.orc_bb_coset_dft_batch.argtypes = [vp, C.c_uint, sz, u32]
        L.orc_bb_coset_idft_batch.argtypes = [vp, C.c_uint, sz, u32]
        L.orc_gl_coset_dft_batch.argtypes = [vp, C.c_uint, sz, u64]
        L.orc_bb_coset_lde.restype = i32
        L.orc_bb_coset_lde.argtypes = [vp, C.c_uint, sz, C.c_uint, u32, i32, vp, i32]
        L.orc_gl_coset_lde.restype = i32
        L.orc_gl_coset_lde.argtypes = [vp, C.c_uint, sz, C.c_uint, u64, i32, vp, i32]
        L.orc_p2_permute_bb.argtypes = [vp, vp]
        L.orc_p2_permute_gl.argtypes = [vp, vp]
        L.orc_grind.restype = i32
        L.orc_grind.argtypes = [vp, vp, vp, C.c_uint, C.c_uint, u64, vp]
        L.orc_p2_hash.argtypes = [vp, vp, sz, vp]
        L.orc_p2_compress.argtypes = [vp, vp, vp, vp]
        L.orc_mmcs_commit.restype = i32
        L.orc_mmcs_commit.argtypes = [vp, vp, vp, vp, sz, C.c_uint, vp, sz, vp, sz, i32]
        L.orc_commit_matrix.restype = i32
        L.orc_commit_matrix.argtypes = [vp, vp, sz, sz, vp, sz, vp, sz, i32]
        L.orc_fold_matrix_bb4.restype = i32
        L.orc_fold_matrix_bb4.argtypes = [vp, C.c_uint, C.c_uint, vp, vp, i32]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# ------------------------------------------------------------------ RNG
def mt19937(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint32)
    lib().orc_mt19937(seed & 0xFFFFFFFF, _ptr(out), n)
    return out


def mt19937_64(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint64)
    lib().orc_mt19937_64(seed & 0xFFFFFFFFFFFFFFFF, _ptr(out), n)
    return out


def bb_random_matrix(h: int, w: int, seed: int) -> np.ndarray:
    """``std::mt19937 rng(seed); BabyBear(rng() % p)`` row-major (test_ntt_cuda.cpp:55-62)."""
    return (mt19937(seed, h * w) % np.uint32(BB_P)).astype(np.uint32).reshape(h, w)


def gl_random_matrix(h: int, w: int, seed: int) -> np.ndarray:
    return (mt19937_64(seed, h * w) % np.uint64(GL_P)).astype(np.uint64).reshape(h, w)


# ------------------------------------------------------------------ Poseidon2 params
def p2_params(field: int, width: int, rounds_f: int, rounds_p: int, degree: int, rate: int,
              digest: int, initial, terminal, internal) -> P2Params:
    p = P2Params()
    p.field, p.width, p.rounds_f, p.rounds_p, p.degree = field, width, rounds_f, rounds_p, degree
    p.rate, p.digest = rate, digest
    ini = np.asarray(initial, dtype=np.uint64).reshape(-1)
    ter = np.asarray(terminal, dtype=np.uint64).reshape(-1)
    inr = np.asarray(internal, dtype=np.uint64).reshape(-1)
    for i, v in enumerate(ini):
        p.initial_rc[i] = int(v)
    for i, v in enumerate(ter):
        p.terminal_rc[i] = int(v)
    for i, v in enumerate(inr):
        p.internal_rc[i] = int(v)
    return p


def example_constants_bb16(rounds_f: int = 8, rounds_p: int = 13, width: int = 16):
    """Constants drawn like merkle_tree_cuda_example.cu:53-66 (mt19937(0xdeadbeef))."""
    half = rounds_f // 2
    raw = mt19937(0xDEADBEEF, 2 * half * width + rounds_p)
    ini = np.zeros((half, width), np.uint64)
    ter = np.zeros((half, width), np.uint64)
    k = 0
    for r in range(half):
        for i in range(width):
            ini[r, i] = raw[k] % BB_P
            ter[r, i] = raw[k + 1] % BB_P
            k += 2
    inr = np.array([raw[k + j] % BB_P for j in range(rounds_p)], np.uint64)
    return ini, ter, inr


def example_constants_gl8(rounds_f: int = 8, rounds_p: int = 22, width: int = 8):
    """Constants drawn like goldilocks_poseidon2_cuda.cu:50-66 (mt19937_64(12345))."""
    half = rounds_f // 2
    raw = mt19937_64(12345, 2 * half * width + rounds_p)
    ini = np.zeros((half, width), np.uint64)
    ter = np.zeros((half, width), np.uint64)
    k = 0
    for r in range(half):
        for i in range(width):
            ini[r, i] = raw[k] % np.uint64(GL_P)
            ter[r, i] = raw[k + 1] % np.uint64(GL_P)
            k += 2
    inr = np.array([raw[k + j] % np.uint64(GL_P) for j in range(rounds_p)], np.uint64)
    return ini, ter, inr


def bb16_params() -> P2Params:
    """BabyBear Poseidon2 width 16, 8 full + 13 partial rounds, x^7, rate 8, digest 8."""
    ini, ter, inr = example_constants_bb16()
    return p2_params(0, 16, 8, 13, 7, 8, 8, ini, ter, inr)


def bb16_zero_params() -> P2Params:
    """All-zero constants, RP=22 (fri_test.cpp:57-71, test_merkle_tree.cpp:450-463)."""
    return p2_params(0, 16, 8, 22, 7, 8, 8, np.zeros((4, 16)), np.zeros((4, 16)), np.zeros(22))


def gl8_params() -> P2Params:
    """Goldilocks Poseidon2 width 8, 8 full + 22 partial rounds, x^7, rate 4, digest 4."""
    ini, ter, inr = example_constants_gl8()
    return p2_params(1, 8, 8, 22, 7, 4, 4, ini, ter, inr)


# ------------------------------------------------------------------ LDE
def bb_coset_lde(trace: np.ndarray, log_blowup: int, shift: int = 31, bitrev: bool = True,
                 nthreads: int = 1) -> np.ndarray:
    trace = np.ascontiguousarray(trace, dtype=np.uint32)
    h, w = trace.shape
    log_h = h.bit_length() - 1
    assert 1 << log_h == h
    out = np.empty((h << log_blowup, w), dtype=np.uint32)
    rc = lib().orc_bb_coset_lde(_ptr(trace), log_h, w, log_blowup, shift, int(bitrev), _ptr(out), nthreads)
    assert rc == 0
    return out


def gl_coset_lde(trace: np.ndarray, log_blowup: int, shift: int = 7, bitrev: bool = True,
                 nthreads: int = 1) -> np.ndarray:
    trace = np.ascontiguousarray(trace, dtype=np.uint64)
    h, w = trace.shape
    log_h = h.bit_length() - 1
    assert 1 << log_h == h
    out = np.empty((h << log_blowup, w), dtype=np.uint64)
    rc = lib().orc_gl_coset_lde(_ptr(trace), log_h, w, log_blowup, shift, int(bitrev), _ptr(out), nthreads)
    assert rc == 0
    return out


def bb_dft(kind: str, mat: np.ndarray, shift: int = 31) -> np.ndarray:
    m = np.ascontiguousarray(mat, dtype=np.uint32).copy()
    h, w = m.shape
    log_h = h.bit_length() - 1
    L = lib()
    if kind == "dft":
        L.orc_bb_dft_batch(_ptr(m), log_h, w)
    elif kind == "idft":
        L.orc_bb_idft_batch(_ptr(m), log_h, w)
    elif kind == "coset_dft":
        L.orc_bb_coset_dft_batch(_ptr(m), log_h, w, shift)
    elif kind == "coset_idft":
        L.orc_bb_coset_idft_batch(_ptr(m), log_h, w, shift)
    else:
        raise ValueError(kind)
    return m


# ------------------------------------------------------------------ Poseidon2 / sponge
def permute(p: P2Params, state: np.ndarray) -> np.ndarray:
    if p.field == 0:
        s = np.ascontiguousarray(state, dtype=np.uint32).copy()
        lib().orc_p2_permute_bb(C.byref(p), _ptr(s))
    else:
        s = np.ascontiguousarray(state, dtype=np.uint64).copy()
        lib().orc_p2_permute_gl(C.byref(p), _ptr(s))
    return s


def _dt(p: P2Params):
    return np.uint32 if p.field == 0 else np.uint64


def hash_iter(p: P2Params, data: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(data, dtype=_dt(p)).reshape(-1)
    out = np.zeros(p.digest, dtype=_dt(p))
    lib().orc_p2_hash(C.byref(p), _ptr(d), d.size, _ptr(out))
    return out


def compress(p: P2Params, left: np.ndarray, right: np.ndarray) -> np.ndarray:
    l = np.ascontiguousarray(left, dtype=_dt(p))
    r = np.ascontiguousarray(right, dtype=_dt(p))
    out = np.zeros(p.digest, dtype=_dt(p))
    lib().orc_p2_compress(C.byref(p), _ptr(l), _ptr(r), _ptr(out))
    return out


def mmcs_commit(p: P2Params, mats, cap_height: int = 0, nthreads: int = 1):
    """Mixed-height MerkleTreeMmcs::commit.  Returns the list of digest layers
    (each an array of shape [n, digest]), bottom-up; the last is the cap."""
    dt = _dt(p)
    arrs = [np.ascontiguousarray(m, dtype=dt) for m in mats]
    n = len(arrs)
    ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in arrs])
    hs = (C.c_size_t * n)(*[a.shape[0] for a in arrs])
    ws = (C.c_size_t * n)(*[a.shape[1] for a in arrs])
    max_h = max(a.shape[0] for a in arrs)
    cap = 2 * max_h + 2
    out = np.zeros((cap, p.digest), dtype=dt)
    sizes = (C.c_size_t * 64)()
    nl = lib().orc_mmcs_commit(C.byref(p), ptrs, hs, ws, n, cap_height, _ptr(out), cap, sizes, 64, nthreads)
    assert nl > 0, nl
    layers, off = [], 0
    for i in range(nl):
        layers.append(out[off:off + sizes[i]].copy())
        off += sizes[i]
    return layers


def commit_matrix(p: P2Params, mat: np.ndarray, nthreads: int = 1):
    """Flat p3_merkle::MerkleTreeMmcs::commit_matrix; returns digest layers."""
    dt = _dt(p)
    m = np.ascontiguousarray(mat, dtype=dt)
    h, w = m.shape
    cap = 2 * h + 64
    out = np.zeros((cap, p.digest), dtype=dt)
    sizes = (C.c_size_t * 80)()
    nl = lib().orc_commit_matrix(C.byref(p), _ptr(m), h, w, _ptr(out), cap, sizes, 80, nthreads)
    assert nl > 0, nl
    layers, off = [], 0
    for i in range(nl):
        layers.append(out[off:off + sizes[i]].copy())
        off += sizes[i]
    return layers


def pcs_commit(p: P2Params, traces, log_blowup: int = 1, shift: int = 1):
    """TwoAdicFriPcs::commit (two_adic_fri_pcs.hpp:207-266): natural-order LDE of
    each matrix, rows concatenated with ``r % height``, width zero-padded to a
    power of two, then the flat commit_matrix.  Returns (root, flat matrix)."""
    ldes = [bb_coset_lde(t, log_blowup, shift=shift, bitrev=False) for t in traces]
    max_h = max(l.shape[0] for l in ldes)
    total_w = sum(l.shape[1] for l in ldes)
    padded_w = 1 << (total_w - 1).bit_length() if total_w > 1 else 1
    flat = np.zeros((max_h, padded_w), dtype=np.uint32)
    col = 0
    for l in ldes:
        reps = max_h // l.shape[0]
        flat[:, col:col + l.shape[1]] = np.tile(l, (reps, 1))
        col += l.shape[1]
    layers = commit_matrix(p, flat)
    return layers[-1][0], flat


def mmcs_verify_batch(p: P2Params, cap, heights, widths, index: int, opened_rows, proof) -> bool:
    """MerkleTreeMmcs::verify_batch (merkle_tree_mmcs.hpp:168-254): hash the
    tallest matrices' opened rows, walk the sibling path compressing (left or
    right by the index bit) and injecting the rows of matrices whose height
    equals the new level size, then compare with cap[index >> levels]."""
    n = len(heights)
    order = sorted(range(n), key=lambda i: -heights[i])  # stable: sorted() is stable
    max_h = heights[order[0]]
    cap = np.asarray(cap)
    cap_size = cap.shape[0]
    levels, h = 0, max_h
    while h > cap_size:
        h //= 2
        levels += 1
    if len(proof) != levels:
        return False
    pos = 0

    def collect(hh):
        nonlocal pos
        out = []
        while pos < n and heights[order[pos]] == hh:
            out.append(order[pos])
            pos += 1
        return out

    tall = collect(max_h)
    cur = hash_iter(p, np.concatenate([np.asarray(opened_rows[i]) for i in tall]) if tall else np.zeros(0))
    idx = index
    for step in range(levels):
        sib = np.asarray(proof[step])
        cur = compress(p, cur, sib) if idx % 2 == 0 else compress(p, sib, cur)
        idx >>= 1
        inj = collect(max_h >> (step + 1))
        if inj:
            rh = hash_iter(p, np.concatenate([np.asarray(opened_rows[i]) for i in inj]))
            cur = compress(p, cur, rh)
    if idx >= cap_size:
        return False
    return bool(np.array_equal(cur, cap[idx]))


# ------------------------------------------------------------------ FRI fold
def fold_matrix_bb4(values: np.ndarray, log_height: int, log_arity: int, beta,
                    nthreads: int = 1) -> np.ndarray:
    v = np.ascontiguousarray(values, dtype=np.uint32).reshape(-1, 4)
    assert v.shape[0] == 1 << log_height
    b = np.asarray(beta, dtype=np.uint32).reshape(4)
    out = np.zeros(((1 << log_height) >> log_arity, 4), dtype=np.uint32)
    rc = lib().orc_fold_matrix_bb4(_ptr(v), log_height, log_arity, _ptr(b), _ptr(out), nthreads)
    assert rc == 0
    return out


def bb4_mul(a, b):
    x = np.asarray(a, np.uint32).reshape(4).copy()
    y = np.asarray(b, np.uint32).reshape(4).copy()
    o = np.zeros(4, np.uint32)
    lib().orc_bb4_mul(_ptr(x), _ptr(y), _ptr(o))
    return o


def bb4_inv(a):
    x = np.asarray(a, np.uint32).reshape(4).copy()
    o = np.zeros(4, np.uint32)
    lib().orc_bb4_inv(_ptr(x), _ptr(o))
    return o


# ------------------------------------------------------------------ PCS open
def pcs_open_values(lde: np.ndarray, shift: int, z, nthreads: int = 1) -> np.ndarray:
    """Opened values of an n x w natural-order LDE at BB4 point z (w x 4)."""
    m = np.ascontiguousarray(lde, dtype=np.uint32)
    n, w = m.shape
    zz = np.asarray(z, dtype=np.uint32).reshape(4)
    out = np.zeros((w, 4), dtype=np.uint32)
    lib().orc_pcs_open_values(_ptr(m), n.bit_length() - 1, w, shift, _ptr(zz), _ptr(out), nthreads)
    return out


def pcs_reduce(lde: np.ndarray, shift: int, zs, opened, alpha, ap0: int, q: np.ndarray,
               nthreads: int = 1) -> np.ndarray:
    """Adds one matrix's reduced-opening terms into q (n x 4, natural order)."""
    m = np.ascontiguousarray(lde, dtype=np.uint32)
    n, w = m.shape
    z = np.ascontiguousarray(zs, dtype=np.uint32).reshape(-1, 4)
    ov = np.ascontiguousarray(opened, dtype=np.uint32).reshape(z.shape[0], w, 4)
    a = np.asarray(alpha, dtype=np.uint32).reshape(4)
    assert q.dtype == np.uint32 and q.shape == (n, 4) and q.flags.c_contiguous
    lib().orc_pcs_reduce(_ptr(m), n.bit_length() - 1, w, shift, _ptr(z), z.shape[0], _ptr(ov), _ptr(a), ap0,
                         _ptr(q), nthreads)
    return q


# ------------------------------------------------------------------ transcript
class Transcript:
    """The reference's DuplexChallenger<BabyBear, Perm, 16, 8>
    (duplex_challenger.hpp:43-260) restated over the oracle's Poseidon2-16:
    observations fill an input buffer that overwrites the first RATE state
    words when full (or before a sample), then the state is permuted and its
    first RATE words become the output buffer, sampled from the back.
    TEST INFRASTRUCTURE: it drives the FRI commit phase in the tests."""
    RATE = 8

    def __init__(self, params: P2Params):
        self.p = params
        self.state = np.zeros(16, dtype=np.uint32)
        self.inp: list[int] = []
        self.out: list[int] = []

    def copy(self) -> "Transcript":
        t = Transcript(self.p)
        t.state, t.inp, t.out = self.state.copy(), list(self.inp), list(self.out)
        return t

    def _absorb(self, v: int):
        self.inp.append(int(v) % BB_P)
        if len(self.inp) == self.RATE:
            self._duplex()

    def _duplex(self):
        for i, v in enumerate(self.inp):
            self.state[i] = v
        self.inp = []
        self.state = permute(self.p, self.state)
        self.out = [int(x) for x in self.state[:self.RATE]]

    def observe(self, v: int):
        self.out = []
        self._absorb(v)

    def observe_ext(self, v):
        self.out = []
        for c in v:
            self._absorb(int(c))

    def observe_cap(self, digests):
        if len(digests) == 0:
            return
        self.out = []
        for d in digests:
            for e in d:
                self._absorb(int(e))

    def sample(self) -> int:
        if self.inp or not self.out:
            self._duplex()
        return self.out.pop()

    def sample_ext(self) -> list[int]:
        return [self.sample() for _ in range(4)]

    def _observe_witness(self, w: int):
        self.out = []
        self._absorb(w & 0xFFFFFFFF)
        self._absorb(w >> 32)

    def grind_py(self, bits: int) -> int:
        """grind, searched by replaying this class's own steps per candidate."""
        mask = (1 << bits) - 1
        w = 0
        while True:
            a = self.copy()
            a._observe_witness(w)
            if a.sample() & mask == 0:
                self._observe_witness(w)
                self.sample()
                return w
            w += 1

    def grind(self, bits: int) -> int:
        """grind through the C restatement (orc_grind), then the observe and
        sample that the reference's grind leaves behind."""
        w = grind(self.p, self.state, self.inp, bits)
        self._observe_witness(w)
        self.sample()
        return w

    def sample_bits(self, bits: int) -> int:
        """sample_bits (duplex_challenger.hpp:129-141) for bits <= 31: one sample."""
        assert bits <= 31
        return self.sample() & ((1 << bits) - 1)

    def check_witness(self, bits: int, w: int) -> bool:
        self._observe_witness(w)
        return self.sample() & ((1 << bits) - 1) == 0


def grind(p: P2Params, state, pending, bits: int, limit: int = 1 << 40) -> int:
    """DuplexChallenger::grind from a sponge state and pending inputs (orc_grind)."""
    dt = _dt(p)
    st = np.ascontiguousarray(state, dtype=dt)
    inp = np.ascontiguousarray(list(pending) if len(pending) else [0], dtype=dt)
    w = C.c_uint64()
    if lib().orc_grind(C.byref(p), _ptr(st), _ptr(inp), len(pending), bits, limit, C.byref(w)) != 0:
        raise ValueError("no witness below the limit")
    return w.value


def fri_log_arity(log_height: int, has_next: bool, next_log_height: int, log_final_height: int,
                  max_log_arity: int) -> int:
    """compute_log_arity_for_round (fri_params.hpp:36-57)."""
    target = next_log_height if has_next else log_final_height
    if log_height <= target:
        return 0
    return min(log_height - target, max_log_arity)


def bb4_axpy(y: np.ndarray, a, x: np.ndarray) -> np.ndarray:
    """y + a * x elementwise over BabyBear^4 (n x 4 arrays)."""
    out = np.empty_like(y)
    aa = np.asarray(a, dtype=np.uint32)
    for i in range(y.shape[0]):
        t = bb4_mul(aa, x[i])
        out[i] = [(int(y[i][k]) + int(t[k])) % BB_P for k in range(4)]
    return out


def bb4_pow(a, e: int):
    r, b = np.array([1, 0, 0, 0], np.uint32), np.asarray(a, dtype=np.uint32)
    while e:
        if e & 1:
            r = bb4_mul(r, b)
        b = bb4_mul(b, b)
        e >>= 1
    return r
