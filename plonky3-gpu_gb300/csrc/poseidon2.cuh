// poseidon2.cuh -- register-resident Poseidon2 permutations.
//
// Same permutation as the reference's Poseidon2Cuda::permute
// (poseidon2_cuda.hpp:57-116): initial MDS-light; RF/2 rounds of
// (+rc, x^D on all lanes, MDS-light); RP rounds of (+rc on lane 0, x^D on lane
// 0, internal layer s_i <- s_i * 2^i + sum(s)) (generic.hpp:148-175); RF/2
// terminal full rounds.  MDS-light applies the circulant [2 3 1 1] to each
// 4-chunk and adds the column sums (external.hpp:67-77, 170-201).
//
// The state is held in registers (fully unrolled), round constants come from
// the kernel-parameter struct (constant bank), and BabyBear runs in
// Montgomery form so that x^D is a chain of single Montgomery products.
#pragma once
#include "internal.hpp"

namespace p3g {

// ------------------------------------------------------------------ BabyBear 16
// x^d on a Montgomery-form value in [0, p): the chain of products stays in
// signed (-p, p) form and is brought back to [0, p) once.
__device__ __forceinline__ uint32_t bb_sbox(uint32_t x, int d) {
    const int32_t xs = int32_t(x);
    const int32_t x2 = bb::smul(xs, xs);
    if (d == 3) return bb::canon(bb::smul(x2, xs));
    const int32_t x4 = bb::smul(x2, x2);
    if (d == 5) return bb::canon(bb::smul(x4, xs));
    const int32_t x3 = bb::smul(x2, xs);
    return bb::canon(bb::smul(x3, x4));  // d == 7: x^2, x^3, x^4, x^7 (field.hpp:105-127)
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
__device__ __forceinline__ uint32_t bb_mul_pow2(uint32_t s, int i) {
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
__device__ __forceinline__ uint64_t gladd(uint64_t a, uint64_t b) { return gl::add(a, b); }

// State in Montgomery form.
template <int D, int RF, int RP>
__device__ __forceinline__ void p2_bb16(uint32_t* s, const P2BB16& p) {
    mds_light<uint32_t, 16, bbadd>(s);
#pragma unroll
    for (int r = 0; r < RF / 2; ++r) {
#pragma unroll
        for (int i = 0; i < 16; ++i) s[i] = bb_sbox(bb::add(s[i], p.initial[r][i]), D);
        mds_light<uint32_t, 16, bbadd>(s);
    }
#pragma unroll
    for (int r = 0; r < RP; ++r) {
        s[0] = bb_sbox(bb::add(s[0], p.internal[r]), D);
        uint32_t sum = s[0];
#pragma unroll
        for (int i = 1; i < 16; ++i) sum = bb::add(sum, s[i]);
        s[0] = bb::add(s[0], sum);  // diag[0] = 1
#pragma unroll
        for (int i = 1; i < 16; ++i) s[i] = bb::add(bb_mul_pow2(s[i], i), sum);
    }
#pragma unroll
    for (int r = 0; r < RF / 2; ++r) {
#pragma unroll
        for (int i = 0; i < 16; ++i) s[i] = bb_sbox(bb::add(s[i], p.terminal[r][i]), D);
        mds_light<uint32_t, 16, bbadd>(s);
    }
}

// ------------------------------------------------------------------ Goldilocks 8
// x^d with the intermediate powers left below 2^64 but unreduced mod p
// (a product accepts any u64 operands); only the result is canonical.
__device__ __forceinline__ uint64_t gl_sbox(uint64_t x, int d) {
    uint64_t x2 = gl::mul_lazy(x, x);
    if (d == 3) return gl::mul(x2, x);
    if (d == 5) return gl::mul(gl::mul_lazy(x2, x2), x);
    uint64_t x3 = gl::mul_lazy(x2, x), x4 = gl::mul_lazy(x2, x2);
    return gl::mul(x3, x4);
}
// x * 2^k for 1 <= k < 64, canonical in/out.
__device__ __forceinline__ uint64_t gl_mul_pow2(uint64_t x, int k) {
    return gl::reduce128(x << k, x >> (64 - k));
}

template <int D, int RF, int RP>
__device__ __forceinline__ void p2_gl8(uint64_t* s, const P2GL8& p) {
    mds_light<uint64_t, 8, gladd>(s);
#pragma unroll
    for (int r = 0; r < RF / 2; ++r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) s[i] = gl_sbox(gl::add(s[i], p.initial[r][i]), D);
        mds_light<uint64_t, 8, gladd>(s);
    }
#pragma unroll
    for (int r = 0; r < RP; ++r) {
        s[0] = gl_sbox(gl::add(s[0], p.internal[r]), D);
        uint64_t sum = s[0];
#pragma unroll
        for (int i = 1; i < 8; ++i) sum = gl::add(sum, s[i]);
        s[0] = gl::add(s[0], sum);
#pragma unroll
        for (int i = 1; i < 8; ++i) s[i] = gl::add(gl_mul_pow2(s[i], i), sum);
    }
#pragma unroll
    for (int r = 0; r < RF / 2; ++r) {
#pragma unroll
        for (int i = 0; i < 8; ++i) s[i] = gl_sbox(gl::add(s[i], p.terminal[r][i]), D);
        mds_light<uint64_t, 8, gladd>(s);
    }
}

// ------------------------------------------------------------------ field-generic sponge glue
struct HBB {
    using T = uint32_t;
    using Params = P2BB16;
    static constexpr int W = 16, RATE = 8, DIG = 8;
    static __device__ __forceinline__ T absorb(T canonical) { return bb::mmul(canonical, bb::R2); }
    static __device__ __forceinline__ T squeeze(T m) { return bb::canon(bb::smul(int32_t(m), 1)); }
    template <int D, int RF, int RP>
    static __device__ __forceinline__ void perm(T* s, const Params& p) { p2_bb16<D, RF, RP>(s, p); }
};
struct HGL {
    using T = uint64_t;
    using Params = P2GL8;
    static constexpr int W = 8, RATE = 4, DIG = 4;
    static __device__ __forceinline__ T absorb(T canonical) { return canonical; }
    static __device__ __forceinline__ T squeeze(T v) { return v; }
    template <int D, int RF, int RP>
    static __device__ __forceinline__ void perm(T* s, const Params& p) { p2_gl8<D, RF, RP>(s, p); }
};

}  // namespace p3g
