// ntt.cuh -- column-batched radix-2^r DFT inside one CTA.
//
// A CTA owns a tile of N = 2^LOGN rows x C columns of a row-major matrix in
// shared memory (element (row i, column c) at i*C + c).  Each column is an
// independent polynomial, so the C columns share every twiddle factor; warp
// lanes run across columns, which keeps global accesses coalesced (C
// consecutive words of a row) and shared-memory accesses bank-conflict free.
//
// The size-N transform is a decimation-in-frequency network split into
// "super-stages" of radix R = 2^r <= 32: each thread loads R elements at
// stride M = S/R of its current sub-block (size S), runs a radix-2 DIF of size
// R in registers with compile-time twiddles (constant-bank operands), scales
// slot s by omega_S^(i_lo * bitrev_r(s)) and stores slot s at position
// i_lo + M*s.  After all super-stages, position p holds X[bitrev_N(p)] -- the
// standard natural-in / bit-reversed-out DIF order, which the callers fold
// into their global row addressing.  This is the same transform as the
// reference's Radix2Dit::dft_batch (radix2_dit.hpp:82-121); only the
// evaluation order of the butterflies differs, and field arithmetic is exact.
#pragma once
#include "fields.cuh"

namespace p3g {

// --------------------------------------------------- compile-time root tables
namespace ct {
constexpr uint32_t bb_mulmod(uint32_t a, uint32_t b) { return uint32_t(uint64_t(a) * b % bb::P); }
constexpr uint32_t bb_powmod(uint32_t a, uint64_t e) {
    uint32_t r = 1;
    while (e) {
        if (e & 1) r = bb_mulmod(r, a);
        a = bb_mulmod(a, a);
        e >>= 1;
    }
    return r;
}
constexpr uint32_t bb_w32_m(int j, bool inv) {
    uint32_t w = bb_powmod(440564289u, uint64_t(1) << (27 - 5));
    if (inv) w = bb_powmod(w, bb::P - 2);
    return uint32_t((uint64_t(bb_powmod(w, uint64_t(j))) << 32) % bb::P);
}
constexpr uint64_t gl_mulmod(uint64_t a, uint64_t b) {
    return uint64_t((unsigned __int128)a * b % gl::P);
}
constexpr uint64_t gl_powmod(uint64_t a, uint64_t e) {
    uint64_t r = 1;
    while (e) {
        if (e & 1) r = gl_mulmod(r, a);
        a = gl_mulmod(a, a);
        e >>= 1;
    }
    return r;
}
constexpr uint64_t gl_w32(int j, bool inv) {
    uint64_t w = gl_powmod(7, (gl::P - 1) >> 5);
    if (inv) w = gl_powmod(w, gl::P - 2);
    return gl_powmod(w, uint64_t(j));
}
}  // namespace ct

#define P3G_W16(F, INV) \
    F(0, INV), F(1, INV), F(2, INV), F(3, INV), F(4, INV), F(5, INV), F(6, INV), F(7, INV), F(8, INV), \
    F(9, INV), F(10, INV), F(11, INV), F(12, INV), F(13, INV), F(14, INV), F(15, INV)

// omega_32^(+-j), j < 16, in each field's constant form.
static __constant__ uint32_t c_bb_w32[2][16] = {{P3G_W16(ct::bb_w32_m, false)}, {P3G_W16(ct::bb_w32_m, true)}};
static __constant__ uint64_t c_gl_w32[2][16] = {{P3G_W16(ct::gl_w32, false)}, {P3G_W16(ct::gl_w32, true)}};

template <class F>
__device__ __forceinline__ typename F::T w32(int inv, int j);
template <>
__device__ __forceinline__ uint32_t w32<FBB>(int inv, int j) { return c_bb_w32[inv][j]; }
template <>
__device__ __forceinline__ uint64_t w32<FGL>(int inv, int j) { return c_gl_w32[inv][j]; }

__host__ __device__ constexpr unsigned bitrev_ct(unsigned x, int bits) {
    unsigned r = 0;
    for (int i = 0; i < bits; ++i) {
        r = (r << 1) | (x & 1);
        x >>= 1;
    }
    return r;
}
__device__ __forceinline__ unsigned bitrev_dev(unsigned x, int bits) {
    return bits == 0 ? 0u : (__brev(x) >> (32 - bits));
}

// In-register radix-2 DIF of size 2^LR (natural in, bit-reversed out).
template <class F, int LR, int INV>
__device__ __forceinline__ void reg_dif(typename F::T* x) {
    constexpr int R = 1 << LR;
#pragma unroll
    for (int l = 0; l < LR; ++l) {
        const int half = R >> (l + 1);
#pragma unroll
        for (int blk = 0; blk < R; blk += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; ++j) {
                typename F::T a = x[blk + j], b = x[blk + j + half];
                x[blk + j] = F::add(a, b);
                typename F::T d = F::sub(a, b);
                if (j == 0) {
                    x[blk + j + half] = d;
                } else {
                    x[blk + j + half] = F::mulc(d, w32<F>(INV, j * (32 / (2 * half))));
                }
            }
        }
    }
}

// Super-stage split of LOGN into radices <= 5.
__host__ __device__ constexpr int ss_count(int logn) { return logn == 0 ? 0 : (logn + 4) / 5; }
__host__ __device__ constexpr int ss_radix(int logn, int j) {
    // ceil-balanced split: first (logn % cnt) parts get one more bit
    return logn / ss_count(logn) + (j < logn % ss_count(logn) ? 1 : 0);
}
__host__ __device__ constexpr int ss_max_radix(int logn) { return logn == 0 ? 0 : ss_radix(logn, 0); }

// Threads per column for an N = 2^LOGN tile: one group of the largest radix
// per thread, capped so that the CTA has at most MAXT threads.
template <int LOGN, int C, int MAXT>
struct DftShape {
    static constexpr int N = 1 << LOGN;
    static constexpr int TPC0 = N >> ss_max_radix(LOGN);
    static constexpr int TPC = TPC0 * C > MAXT ? MAXT / C : TPC0;
    static constexpr int THREADS = TPC * C;
};

// One super-stage on the smem tile: sub-blocks of size 2^LS, radix 2^LR.
// tw[e] = omega_N^e (const form), e < N.  Thread (t, c) with t in [0, TPC).
template <class F, int LOGN, int LS, int LR, int C, int TPC, int INV>
__device__ __forceinline__ void super_stage(typename F::T* tile, const typename F::T* tw, int t, int c) {
    using T = typename F::T;
    constexpr int N = 1 << LOGN;
    constexpr int R = 1 << LR;
    constexpr int M = (1 << LS) >> LR;   // stride inside a sub-block
    constexpr int GROUPS = N >> LR;      // groups per column
    static_assert(GROUPS % TPC == 0, "groups per thread");
    constexpr int TWS = LOGN - LS;       // omega_S = omega_N^(2^TWS)
#pragma unroll 1
    for (int g = t; g < GROUPS; g += TPC) {
        const int blk = g / M, i_lo = g % M;
        const int base = blk * (1 << LS) + i_lo;
        T x[R];
#pragma unroll
        for (int k = 0; k < R; ++k) x[k] = tile[(base + M * k) * C + c];
        reg_dif<F, LR, INV>(x);
        if (M > 1) {
#pragma unroll
            for (int s = 1; s < R; ++s) {
                const int e = (i_lo * int(bitrev_ct(unsigned(s), LR))) << TWS;
                x[s] = F::mulc(x[s], tw[e]);
            }
        }
#pragma unroll
        for (int k = 0; k < R; ++k) tile[(base + M * k) * C + c] = x[k];
    }
}

__host__ __device__ constexpr int ss_consumed(int logn, int j) {
    int s = 0;
    for (int i = 0; i < j; ++i) s += ss_radix(logn, i);
    return s;
}

template <class F, int LOGN, int C, int TPC, int INV, int J>
struct SSChain {
    static __device__ __forceinline__ void run(typename F::T* tile, const typename F::T* tw, int t, int c) {
        if constexpr (J < ss_count(LOGN)) {
            constexpr int LR = ss_radix(LOGN, J);
            constexpr int LS = LOGN - ss_consumed(LOGN, J);  // sub-block size before this stage
            super_stage<F, LOGN, LS, LR, C, TPC, INV>(tile, tw, t, c);
            __syncthreads();
            SSChain<F, LOGN, C, TPC, INV, J + 1>::run(tile, tw, t, c);
        }
    }
};

// Full in-CTA DIF: tile natural order in, bit-reversed out.  Requires a
// __syncthreads() before the call (tile filled) and ends with one.
template <class F, int LOGN, int C, int TPC, int INV>
__device__ __forceinline__ void cta_dif(typename F::T* tile, const typename F::T* tw, int t, int c) {
    if constexpr (LOGN > 0) SSChain<F, LOGN, C, TPC, INV, 0>::run(tile, tw, t, c);
}

}  // namespace p3g
