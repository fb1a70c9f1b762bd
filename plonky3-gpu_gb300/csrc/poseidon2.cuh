// poseidon2.cuh -- register-resident Poseidon2 permutations.
//
// Same permutation as the reference's Poseidon2Cuda::permute
// (poseidon2_cuda.hpp:57-116): initial MDS-light; RF/2 rounds of
// (+rc, x^D on all lanes, MDS-light); RP rounds of (+rc on lane 0, x^D on lane
// 0, internal layer s_i <- s_i * 2^i + sum(s)) (generic.hpp:148-175); RF/2
// terminal full rounds.  MDS-light applies the circulant [2 3 1 1] to each
// 4-chunk and adds the column sums (external.hpp:67-77, 170-201).
//
// The state is held in registers, round constants come from the
// kernel-parameter struct (constant bank), and BabyBear runs in Montgomery
// form so that x^D is a chain of single Montgomery products.  Each round's
// body is unrolled over the state words, but the rounds themselves stay a
// loop: the fully unrolled permutation (about 5,600 instructions for BabyBear,
// 12,500 for Goldilocks) overflowed the instruction cache, and warps waited
// for instructions more than for the multiplier (ncu: "no instruction" the
// top stall, issue active about 50%).  Rolled, the isolated permutation runs
// 16% (BabyBear) and 21% (Goldilocks) faster.
#pragma once
#include "internal.hpp"

namespace p3g {

// ------------------------------------------------------------------ BabyBear 16
// x^d on a Montgomery-form value in (-p, p) (the signed product accepts
// either sign): the chain of products stays in signed (-p, p) form and is
// brought back to [0, p) once.
__device__ __forceinline__ uint32_t bb_sbox(int32_t xs, int d) {
    const int32_t x2 = bb::smul(xs, xs);
    if (d == 3) return bb::canon(bb::smul(x2, xs));
    const int32_t x4 = bb::smul(x2, x2);
    if (d == 5) return bb::canon(bb::smul(x4, xs));
    const int32_t x3 = bb::smul(x2, xs);
    return bb::canon(bb::smul(x3, x4));  // d == 7: x^2, x^3, x^4, x^7 (field.hpp:105-127)
}

// s + c - p for s, c in [0, p): one instruction, and in (-p, p), which is all
// the S-box's signed product needs (the round-constant addition of a full
// or partial round).
__device__ __forceinline__ int32_t bb_add_rc(uint32_t s, uint32_t c) { return int32_t(s + c - bb::P); }

// The sum of the 16 state words, canonical: pair sums in 32 bits (each below
// 2p < 2^32), a 64-bit total S < 16p < 2^35, then one Barrett step for
// p = 15 * 2^27 + 1: q = floor((S >> 27) / 15) makes S - q p lie in
// [-17, p), and the canonical value follows with one conditional + p.
// (About half the instructions of fifteen modular additions.)
__device__ __forceinline__ uint32_t bb_sum16(const uint32_t* s) {
    uint64_t S = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) S += uint32_t(s[2 * i] + s[2 * i + 1]);
    const uint32_t v = uint32_t(S >> 27);          // < 2^8
    const uint32_t q = __umulhi(v, 286392320u);     // floor(v / 15) for v < 2^8 (286392320 = 4370 * 2^16)
    return bb::canon(int32_t(uint32_t(S) - q * bb::P));
}

// Shoup constants floor(2^(32+i) / p) for the internal diagonal 2^i.
namespace ct {
constexpr uint32_t shoup_pow2(int i) { return uint32_t((uint64_t(1) << (32 + i)) / bb::P); }
}  // namespace ct
#define P3G_SH16 \
    ct::shoup_pow2(0), ct::shoup_pow2(1), ct::shoup_pow2(2), ct::shoup_pow2(3), ct::shoup_pow2(4), \
    ct::shoup_pow2(5), ct::shoup_pow2(6), ct::shoup_pow2(7), ct::shoup_pow2(8), ct::shoup_pow2(9), \
    ct::shoup_pow2(10), ct::shoup_pow2(11), ct::shoup_pow2(12), ct::shoup_pow2(13), ct::shoup_pow2(14), \
    ct::shoup_pow2(15)
static __constant__ uint32_t c_bb_shoup_pow2[16] = {P3G_SH16};

// s * 2^i mod p for s in [0, p), 1 <= i <= 15 (Shoup: q = floor(s w' / 2^32),
// s*2^i - q*p lies in [0, 2p)).  Multiplying the Montgomery representative by
// the plain constant 2^i is the same as multiplying the field element.
// For i <= 2 (s is canonical, so 2s < 2p < 2^32) repeated modular doubling
// does it on the ALU pipe alone: the permutation is bound by the IMAD pipe,
// and this measured 2.3% faster than the Shoup product there (doubling up to
// i = 1 or 3 gained 0.9% and 1.2%; up to i = 6 lost 1.5%).
__device__ __forceinline__ uint32_t bb_mul_pow2(uint32_t s, int i) {
    if (i <= 2) {
#pragma unroll
        for (int j = 0; j < 2; ++j)
            if (j < i) {
                const uint32_t d = s << 1, t = d - bb::P;
                s = d < t ? d : t;
            }
        return s;
    }
    const uint32_t q = __umulhi(s, c_bb_shoup_pow2[i]);
    const uint32_t r = (s << i) - q * bb::P;
    const uint32_t t = r - bb::P;
    return r < t ? r : t;
}

template <class T, T (*ADD)(T, T)>
__device__ __forceinline__ void mat4(T* x) {
    T t01 = ADD(x[0], x[1]);
    T t23 = ADD(x[2], x[3]);
    T t0123 = ADD(t01, t23);
    T t01123 = ADD(t0123, x[1]);
    T t01233 = ADD(t0123, x[3]);
    x[3] = ADD(t01233, ADD(x[0], x[0]));
    x[1] = ADD(t01123, ADD(x[2], x[2]));
    x[0] = ADD(t01123, t01);
    x[2] = ADD(t01233, t23);
}

template <class T, int W, T (*ADD)(T, T)>
__device__ __forceinline__ void mds_light(T* s) {
#pragma unroll
    for (int i = 0; i < W; i += 4) mat4<T, ADD>(s + i);
    T sums[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        sums[k] = s[k];
#pragma unroll
        for (int j = k + 4; j < W; j += 4) sums[k] = ADD(sums[k], s[j]);
    }
#pragma unroll
    for (int i = 0; i < W; ++i) s[i] = ADD(s[i], sums[i % 4]);
}

__device__ __forceinline__ uint32_t bbadd(uint32_t a, uint32_t b) { return bb::add(a, b); }

// Calls f(r) for r = 0 .. N-1, as a loop (ROLL) or unrolled.
template <bool ROLL, int N, class Fn>
__device__ __forceinline__ void rounds(const Fn& f) {
    if constexpr (ROLL) {
#pragma unroll 1
        for (int r = 0; r < N; ++r) f(r);
    } else {
#pragma unroll
        for (int r = 0; r < N; ++r) f(r);
    }
}

// State in Montgomery form.  ROLL: the round loops stay loops (the default;
// the proof-of-work search, whose candidate loop wraps the permutation, ran
// faster unrolled when measured).
template <int D, int RF, int RP, bool ROLL = true>
__device__ __forceinline__ void p2_bb16(uint32_t* s, const P2BB16& p) {
    mds_light<uint32_t, 16, bbadd>(s);
    rounds<ROLL, RF / 2>([&](int r) {
#pragma unroll
        for (int i = 0; i < 16; ++i) s[i] = bb_sbox(bb_add_rc(s[i], p.initial[r][i]), D);
        mds_light<uint32_t, 16, bbadd>(s);
    });
    rounds<ROLL, RP>([&](int r) {
        s[0] = bb_sbox(bb_add_rc(s[0], p.internal[r]), D);
        const uint32_t sum = bb_sum16(s);
        s[0] = bb::add(s[0], sum);  // diag[0] = 1
#pragma unroll
        for (int i = 1; i < 16; ++i) s[i] = bb::add(bb_mul_pow2(s[i], i), sum);
    });
    rounds<ROLL, RF / 2>([&](int r) {
#pragma unroll
        for (int i = 0; i < 16; ++i) s[i] = bb_sbox(bb_add_rc(s[i], p.terminal[r][i]), D);
        mds_light<uint32_t, 16, bbadd>(s);
    });
}

// ------------------------------------------------------------------ BabyBear 16, one lane per word
// The same permutation on 16 lanes of a warp (lanes 16g..16g+15 hold the
// state of permutation g, one word each): for the latency-bound callers --
// the small top levels of a tree and the transcript -- where one thread per
// permutation waits on a long chain of dependent products.  Every lane runs
// the same field operations as p2_bb16 on its word; MDS-light gathers the
// lane's 4-chunk by shuffles and adds the column sums by an xor-reduction
// over the chunks; a partial round reduces the 16 words the same way.
// All 32 lanes of the warp must call it together.
struct CoopConsts {  // this lane's constants
    uint32_t ini[4], ter[4];
    uint32_t shoup;  // floor(2^(32+i) / p) for the diagonal 2^i, i = lane
};
__device__ __forceinline__ CoopConsts coop_consts(const P2BB16& p, int i) {
    CoopConsts c;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        c.ini[r] = p.initial[r][i];
        c.ter[r] = p.terminal[r][i];
    }
    c.shoup = c_bb_shoup_pow2[i];
    return c;
}

__device__ __forceinline__ uint32_t coop_mds_light(uint32_t x, int i) {
    const int base = i & ~3, pos = i & 3;
    const uint32_t x0 = __shfl_sync(0xffffffffu, x, base, 16), x1 = __shfl_sync(0xffffffffu, x, base + 1, 16);
    const uint32_t x2 = __shfl_sync(0xffffffffu, x, base + 2, 16), x3 = __shfl_sync(0xffffffffu, x, base + 3, 16);
    const uint32_t t01 = bb::add(x0, x1), t23 = bb::add(x2, x3), t0123 = bb::add(t01, t23);
    const uint32_t t01123 = bb::add(t0123, x1), t01233 = bb::add(t0123, x3);
    uint32_t y;  // mat4 [2 3 1 1] row pos (external.hpp:67-77)
    if (pos == 0) y = bb::add(t01123, t01);
    else if (pos == 1) y = bb::add(t01123, bb::add(x2, x2));
    else if (pos == 2) y = bb::add(t01233, t23);
    else y = bb::add(t01233, bb::add(x0, x0));
    uint32_t col = bb::add(y, __shfl_xor_sync(0xffffffffu, y, 4, 16));
    col = bb::add(col, __shfl_xor_sync(0xffffffffu, col, 8, 16));
    return bb::add(y, col);
}

template <int D, int RF, int RP>
__device__ __forceinline__ uint32_t p2_bb16_coop(uint32_t x, const P2BB16& p, const CoopConsts& c, int i) {
    x = coop_mds_light(x, i);
#pragma unroll
    for (int r = 0; r < RF / 2; ++r) x = coop_mds_light(bb_sbox(bb_add_rc(x, c.ini[r]), D), i);
#pragma unroll 1
    for (int r = 0; r < RP; ++r) {
        if (i == 0) x = bb_sbox(bb_add_rc(x, p.internal[r]), D);
        uint32_t sum = bb::add(x, __shfl_xor_sync(0xffffffffu, x, 1, 16));
        sum = bb::add(sum, __shfl_xor_sync(0xffffffffu, sum, 2, 16));
        sum = bb::add(sum, __shfl_xor_sync(0xffffffffu, sum, 4, 16));
        sum = bb::add(sum, __shfl_xor_sync(0xffffffffu, sum, 8, 16));
        uint32_t d = x;  // x * 2^i (diag[0] = 1)
        if (i > 0) {
            const uint32_t q = __umulhi(x, c.shoup);
            const uint32_t r0 = (x << i) - q * bb::P, r1 = r0 - bb::P;
            d = r0 < r1 ? r0 : r1;
        }
        x = bb::add(d, sum);
    }
#pragma unroll
    for (int r = 0; r < RF / 2; ++r) x = coop_mds_light(bb_sbox(bb_add_rc(x, c.ter[r]), D), i);
    return x;
}

// ------------------------------------------------------------------ Goldilocks 8
// The state words are kept below 2^64 but not reduced mod p inside the
// permutation (every product and linear layer accepts any u64 operands);
// squeezing makes them canonical.  x^d with every product left unreduced.
__device__ __forceinline__ uint64_t gl_sbox(uint64_t x, int d) {
    uint64_t x2 = gl::mul_lazy(x, x);
    if (d == 3) return gl::mul_lazy(x2, x);
    if (d == 5) return gl::mul_lazy(gl::mul_lazy(x2, x2), x);
    uint64_t x3 = gl::mul_lazy(x2, x), x4 = gl::mul_lazy(x2, x2);
    return gl::mul_lazy(x3, x4);
}
// Goldilocks linear layers on unreduced sums: a G2 is lo + hi * 2^64 with a
// small hi (a carry count), added with one three-limb carry chain and
// reduced once per output (2^64 = 2^32 - 1 mod p), instead of a canonical
// reduction after every addition.
struct G2 {
    uint64_t lo;
    uint32_t hi;
};
__device__ __forceinline__ G2 g2(uint64_t x) { return {x, 0u}; }
__device__ __forceinline__ G2 g2add(G2 a, G2 b) {
    uint32_t l0, l1, h;
    asm("{\n\t"
        "add.cc.u32 %0, %3, %6;\n\t"
        "addc.cc.u32 %1, %4, %7;\n\t"
        "addc.u32 %2, %5, %8;\n\t"
        "}"
        : "=&r"(l0), "=&r"(l1), "=&r"(h)
        : "r"(uint32_t(a.lo)), "r"(uint32_t(a.lo >> 32)), "r"(a.hi), "r"(uint32_t(b.lo)),
          "r"(uint32_t(b.lo >> 32)), "r"(b.hi));
    return {(uint64_t(l1) << 32) | l0, h};
}
// a value below 2^64 congruent to a G2 (hi < 2^32)
__device__ __forceinline__ uint64_t g2red(G2 a) {
    const uint64_t t = (uint64_t(a.hi) << 32) - a.hi;  // hi * (2^32 - 1) <= (2^32 - 1)^2
    uint64_t s = a.lo + t;
    if (s < t) s += gl::EPS;  // wrapped: + 2^64 = + EPS; s < t keeps this below 2^64
    return s;
}
// x * 2^k as a G2, 1 <= k < 32
__device__ __forceinline__ G2 g2shl(uint64_t x, int k) { return {x << k, uint32_t(x >> (64 - k))}; }

// MDS-light for width 8 (external.hpp:67-77, 170-201): [2 3 1 1] on each
// 4-chunk, then the column sums; every output is a sum of at most 21 inputs
// below 2^64, so its carry count stays below 2^5.
__device__ __forceinline__ void mds_light_gl8(uint64_t* s) {
    G2 y[8];
#pragma unroll
    for (int c = 0; c < 8; c += 4) {
        const G2 x0 = g2(s[c]), x1 = g2(s[c + 1]), x2 = g2(s[c + 2]), x3 = g2(s[c + 3]);
        const G2 t01 = g2add(x0, x1), t23 = g2add(x2, x3);
        const G2 t0123 = g2add(t01, t23);
        const G2 t01123 = g2add(t0123, x1), t01233 = g2add(t0123, x3);
        y[c + 3] = g2add(t01233, g2add(x0, x0));
        y[c + 1] = g2add(t01123, g2add(x2, x2));
        y[c + 0] = g2add(t01123, t01);
        y[c + 2] = g2add(t01233, t23);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const G2 col = g2add(y[k], y[k + 4]);
        s[k] = g2red(g2add(y[k], col));
        s[k + 4] = g2red(g2add(y[k + 4], col));
    }
}
// s + c for any s < 2^64 and canonical c; the result is below 2^64 but
// possibly >= p (an S-box input: products accept any u64)
__device__ __forceinline__ uint64_t gl_add_lazy(uint64_t a, uint64_t c) {
    uint64_t t = a + c;
    if (t < c) t += gl::EPS;  // a + c - 2^64 < 2^64 - 2^33 leaves room for EPS
    return t;
}

template <int D, int RF, int RP, bool ROLL = true>
__device__ __forceinline__ void p2_gl8(uint64_t* s, const P2GL8& p) {
    mds_light_gl8(s);
    rounds<ROLL, RF / 2>([&](int r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) s[i] = gl_sbox(gl_add_lazy(s[i], p.initial[r][i]), D);
        mds_light_gl8(s);
    });
    rounds<ROLL, RP>([&](int r) {
        // internal layer (generic.hpp:148-175): s_i <- s_i * 2^i + sum(s)
        s[0] = gl_sbox(gl_add_lazy(s[0], p.internal[r]), D);
        G2 sum = g2(s[0]);  // carry count below 8, left unreduced
#pragma unroll
        for (int i = 1; i < 8; ++i) sum = g2add(sum, g2(s[i]));
        s[0] = g2red(g2add(g2(s[0]), sum));
#pragma unroll
        for (int i = 1; i < 8; ++i) s[i] = g2red(g2add(g2shl(s[i], i), sum));
    });
    rounds<ROLL, RF / 2>([&](int r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) s[i] = gl_sbox(gl_add_lazy(s[i], p.terminal[r][i]), D);
        mds_light_gl8(s);
    });
}

// ------------------------------------------------------------------ field-generic sponge glue
struct HBB {
    using T = uint32_t;
    using Params = P2BB16;
    static constexpr int W = 16, RATE = 8, DIG = 8;
    static __host__ __device__ __forceinline__ T absorb(T canonical) { return bb::mmul(canonical, bb::R2); }
    static __device__ __forceinline__ T squeeze(T m) { return bb::canon(bb::smul(int32_t(m), 1)); }
    // BabyBear(uint32_t) reduces its argument (baby_bear.hpp:51)
    static __device__ __forceinline__ T from_u32(uint32_t x) { return x % bb::P; }
    template <int D, int RF, int RP, bool ROLL = true>
    static __device__ __forceinline__ void perm(T* s, const Params& p) { p2_bb16<D, RF, RP, ROLL>(s, p); }
};
struct HGL {
    using T = uint64_t;
    using Params = P2GL8;
    static constexpr int W = 8, RATE = 4, DIG = 4;
    static __host__ __device__ __forceinline__ T absorb(T canonical) { return canonical; }
    // the permutation leaves words below 2^64, not necessarily below p
    static __device__ __forceinline__ T squeeze(T v) { return v >= gl::P ? v - gl::P : v; }
    static __device__ __forceinline__ T from_u32(uint32_t x) { return x; }  // goldilocks.hpp:34
    template <int D, int RF, int RP, bool ROLL = true>
    static __device__ __forceinline__ void perm(T* s, const Params& p) { p2_gl8<D, RF, RP, ROLL>(s, p); }
};

}  // namespace p3g
