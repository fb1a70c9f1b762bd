// ntt.cuh -- column-batched radix-2^r DFT inside one CTA.
//
// A CTA owns a tile of N = 2^LOGN rows x C columns of a row-major matrix.
// Each column is an independent polynomial, so the C columns share every
// twiddle factor; warp lanes run across columns, so global accesses are
// coalesced C-word row segments.
//
// The size-N transform is a decimation-in-frequency network split into
// "super-stages" of radix R = 2^r <= 32.  Super-stage j: each thread takes R
// elements at stride M = S/R of its sub-block (size S), runs a radix-2 DIF of
// size R in registers with compile-time twiddles (constant-bank operands),
// scales slot s by omega_S^(i_lo * bitrev_r(s)) and leaves slot s at position
// i_lo + M*s.  The first super-stage reads its elements through a caller
// supplied `load(row)` (global memory, or a permuted shared-memory tile) and
// the last hands its results to `store(pos, value)` (global memory, or a
// tile): only the exchanges between super-stages go through shared memory.
// Loads and stores work on whole groups (`group<R, M>(base, x)`: rows
// base + M*k; `group<LR>(base, x)`: positions base + k) so that global
// accesses walk one strided pointer instead of materialising R addresses.
// After all super-stages, position p holds X[bitrev_N(p)] -- natural-in /
// bit-reversed-out, which the callers fold into their global row addressing.
// Same transform as Radix2Dit::dft_batch (radix2_dit.hpp:82-121); only the
// order of the (exact) butterflies differs.
//
// Shared-memory layout: 128-byte lines; a line holds L = 128 / (C * sizeof(T))
// row segments.  Row `row` lives in line row >> log2(L) at sub-slot
// (row ^ hash(row)) mod L, where hash mixes the row bits that differ between
// the rows one warp touches at once (consecutive groups, the last
// super-stage's groups, the bit-reversed read), so those rows land on
// distinct banks.
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
constexpr uint32_t bb_w32(int j, bool inv) {
    uint32_t w = bb_powmod(440564289u, uint64_t(1) << (27 - 5));
    if (inv) w = bb_powmod(w, bb::P - 2);
    return bb_powmod(w, uint64_t(j));
}
constexpr uint32_t bb_w32_c(int j, bool inv) {  // Shoup companion floor(w * 2^32 / p)
    return uint32_t((uint64_t(bb_w32(j, inv)) << 32) / bb::P);
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

// omega_32^(+-j), j < 16: BabyBear as Shoup pairs (value, companion),
// Goldilocks canonical.
static __constant__ uint32_t c_bb_w32[2][16] = {{P3G_W16(ct::bb_w32, false)}, {P3G_W16(ct::bb_w32, true)}};
static __constant__ uint32_t c_bb_w32c[2][16] = {{P3G_W16(ct::bb_w32_c, false)}, {P3G_W16(ct::bb_w32_c, true)}};
static __constant__ uint64_t c_gl_w32[2][16] = {{P3G_W16(ct::gl_w32, false)}, {P3G_W16(ct::gl_w32, true)}};

template <class F>
__device__ __forceinline__ typename F::TW w32(int inv, int j);
template <>
__device__ __forceinline__ uint2 w32<FBB>(int inv, int j) { return make_uint2(c_bb_w32[inv][j], c_bb_w32c[inv][j]); }
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
                if (j == 0) {
                    x[blk + j + half] = F::sub(a, b);
                } else {
                    x[blk + j + half] = F::mul_tw(F::sub_lazy(a, b), w32<F>(INV, j * (32 / (2 * half))));
                }
            }
        }
    }
}

// Super-stage split of LOGN into radices of at most 2^mlr.  mlr is 5 for
// 4-byte elements and 4 for 8-byte ones: a radix-32 group of u64 values
// takes 64 registers per thread before any temporaries, which held the
// Goldilocks passes to a few warps per SM.
// (Both limits can be set at build time, -DP3G_SS_MLR4= / -DP3G_SS_MLR8=, to
// compare splits.)
#ifndef P3G_SS_MLR4
#define P3G_SS_MLR4 5
#endif
#ifndef P3G_SS_MLR8
#define P3G_SS_MLR8 4
#endif
template <class T>
__host__ __device__ constexpr int ss_max_lr() { return sizeof(T) == 8 ? P3G_SS_MLR8 : P3G_SS_MLR4; }
// Groups of a super-stage a thread's loop unrolls (1: the loop stays rolled;
// settable at build time to compare).
#ifndef P3G_SS_GROUP_UNROLL
#define P3G_SS_GROUP_UNROLL 1
#endif
constexpr int SS_GROUP_UNROLL = P3G_SS_GROUP_UNROLL;
__host__ __device__ constexpr int ss_count(int logn, int mlr) { return logn == 0 ? 0 : (logn + mlr - 1) / mlr; }
__host__ __device__ constexpr int ss_radix(int logn, int j, int mlr) {
    // ceil-balanced split: the first (logn % cnt) parts get one more bit
    return logn / ss_count(logn, mlr) + (j < logn % ss_count(logn, mlr) ? 1 : 0);
}
__host__ __device__ constexpr int ss_max_radix(int logn, int mlr) { return logn == 0 ? 0 : ss_radix(logn, 0, mlr); }
__host__ __device__ constexpr int ss_consumed(int logn, int j, int mlr) {
    int s = 0;
    for (int i = 0; i < j; ++i) s += ss_radix(logn, i, mlr);
    return s;
}
// Inter-super-stage twiddles in stage order.  Super-stage J (every one but
// the last) multiplies slot s of group i_lo by omega_N^((i_lo * bitrev(s)) <<
// TWS_J); the table holds that value at ss_tw_off(J) + i_lo * R_J + s, so a
// group's R_J twiddles sit at one base address plus compile-time offsets
// (one address per group instead of a product per twiddle).  Stage J's block
// has 2^LS_J entries (s = 0 included, unused); the whole table
// ss_tw_size(LOGN) entries (LOGN at LOGN <= 2 * radix, more above).
__host__ __device__ constexpr int ss_tw_off(int logn, int j, int mlr) {
    int o = 0;
    for (int i = 0; i < j; ++i) o += 1 << (logn - ss_consumed(logn, i, mlr));
    return o;
}
__host__ __device__ constexpr int ss_tw_size(int logn, int mlr) {
    return ss_count(logn, mlr) <= 1 ? 0 : ss_tw_off(logn, ss_count(logn, mlr) - 1, mlr);
}
// e such that entry idx of the stage-ordered table is omega_N^e (e < N)
__host__ __device__ inline uint32_t ss_tw_exp(int logn, int mlr, int idx) {
    int j = 0;
    while (j + 2 < ss_count(logn, mlr) && idx >= ss_tw_off(logn, j + 1, mlr)) ++j;
    const int lr = ss_radix(logn, j, mlr);
    const unsigned local = unsigned(idx - ss_tw_off(logn, j, mlr));
    const unsigned i_lo = local >> lr, s = local & ((1u << lr) - 1u);
    return (i_lo * bitrev_ct(s, lr)) << ss_consumed(logn, j, mlr);
}
__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x >> 1); }

// Tile geometry: N = 2^LOGN rows x C columns, at most MAXT threads.
template <class T, int LOGN, int C, int MAXT>
struct DftShape {
    static constexpr int N = 1 << LOGN;
    static constexpr int MLR = ss_max_lr<T>();
    static constexpr int TPC0 = N >> ss_max_radix(LOGN, MLR);
    static constexpr int TPC = TPC0 * C > MAXT ? MAXT / C : TPC0;  // threads per column
    static constexpr int THREADS = TPC * C;
    // swizzled shared-memory layout
    static constexpr int LINE = 128 / int(sizeof(T));   // elements per 128-byte line
    static constexpr int RPL = LINE / C >= 1 ? LINE / C : 1;  // row segments per line
    static constexpr int LG = ilog2(RPL);
    static constexpr int RL = ss_count(LOGN, MLR) ? ss_radix(LOGN, ss_count(LOGN, MLR) - 1, MLR) : 0;
    static constexpr int SH1 = cmax(RL, LG);
    static constexpr int SH2 = cmax(LOGN - LG, LG);
    static constexpr int TILE = N * C;  // elements
    // stage-ordered twiddle table: entries, and the size a kernel allots
    static constexpr int TWN = ss_tw_size(LOGN, MLR);
    static constexpr int TWA = TWN > N ? TWN : N;
    static __host__ __device__ __forceinline__ int swz(int row) { return (row ^ (row >> SH1) ^ (row >> SH2)) & (RPL - 1); }
    static __host__ __device__ __forceinline__ int addr(int row, int c) {
        if constexpr (RPL == 1) {
            return row * C + c;
        } else {
            return (row >> LG) * LINE + swz(row) * C + c;
        }
    }
    // The rows one thread touches in a group are base + mk with base and mk
    // sharing no set bit, mk a compile-time offset.  The swizzle is linear
    // over XOR and the line index over such a sum, so row0(base, c) is
    // computed once per group and at(r0, mk) == addr(base + mk, c) costs an
    // XOR and an add per element (mk's terms fold into constants).
    struct Row0 {
        int line;  // (base >> LG) * LINE, or base * C + c without a swizzle
        int sub;   // swz(base) * C + c
    };
    static __host__ __device__ __forceinline__ Row0 row0(int base, int c) {
        if constexpr (RPL == 1) return {base * C + c, 0};
        else return {(base >> LG) * LINE, swz(base) * C + c};
    }
    static __host__ __device__ __forceinline__ int at(const Row0& r, int mk) {
        if constexpr (RPL == 1) return r.line + mk * C;
        else return r.line + (mk >> LG) * LINE + (r.sub ^ (swz(mk) * C));
    }
};

// One super-stage J.  tw: the stage-ordered twiddle table (prepared twiddles).
template <class F, class SH, int LOGN, int J, int C, int INV, class Load, class Store>
__device__ __forceinline__ void super_stage(typename F::T* tile, const typename F::TW* tw, int t, int c,
                                            Load& load, Store& store) {
    using T = typename F::T;
    constexpr int MLR = ss_max_lr<T>();
    constexpr int CNT = ss_count(LOGN, MLR);
    constexpr int LR = ss_radix(LOGN, J, MLR);
    constexpr int LS = LOGN - ss_consumed(LOGN, J, MLR);
    constexpr int R = 1 << LR;
    constexpr int M = (1 << LS) >> LR;
    constexpr int GROUPS = (1 << LOGN) >> LR;
    constexpr bool FIRST = J == 0, LAST = J == CNT - 1;
    static_assert(GROUPS % SH::TPC == 0, "groups per thread");
#pragma unroll SS_GROUP_UNROLL
    for (int g = t; g < GROUPS; g += SH::TPC) {
        const int blk = g / M, i_lo = g % M;
        const int base = blk * (1 << LS) + i_lo;  // i_lo < M: disjoint from M*k
        T x[R];
        if constexpr (FIRST) {
            load.template group<R, M>(base, x);  // rows base + M*k
        } else {
            const auto r0 = SH::row0(base, c);
#pragma unroll
            for (int k = 0; k < R; ++k) x[k] = tile[SH::at(r0, M * k)];
        }
        reg_dif<F, LR, INV>(x);
        if constexpr (LAST) {
            store.template group<LR>(base, x);  // positions base + k (M == 1)
        } else {
            const typename F::TW* twg = tw + ss_tw_off(LOGN, J, MLR) + i_lo * R;
#pragma unroll
            for (int s = 1; s < R; ++s) x[s] = F::mul_tw(x[s], twg[s]);
            const auto r0 = SH::row0(base, c);
#pragma unroll
            for (int k = 0; k < R; ++k) tile[SH::at(r0, M * k)] = x[k];
        }
    }
}

template <class F, class SH, int LOGN, int C, int INV, int J>
struct SSChain {
    template <class Load, class Store>
    static __device__ __forceinline__ void run(typename F::T* tile, const typename F::TW* tw, int t, int c,
                                               Load& load, Store& store) {
        constexpr int CNT = ss_count(LOGN, ss_max_lr<typename F::T>());
        if constexpr (J < CNT) {
            super_stage<F, SH, LOGN, J, C, INV>(tile, tw, t, c, load, store);
            if constexpr (J + 1 < CNT) __syncthreads();
            SSChain<F, SH, LOGN, C, INV, J + 1>::run(tile, tw, t, c, load, store);
        }
    }
};

// Full in-CTA DIF on one column per thread group: element at natural row i
// comes from the load functor; the store functor receives X[bitrev_N(p)] for
// position p.  `tile` is the
// exchange buffer (SH::TILE elements).  Callers synchronise around it.
template <class F, class SH, int LOGN, int C, int INV, class Load, class Store>
__device__ __forceinline__ void cta_dif(typename F::T* tile, const typename F::TW* tw, int t, int c, Load& load,
                                        Store& store) {
    SSChain<F, SH, LOGN, C, INV, 0>::run(tile, tw, t, c, load, store);
}

}  // namespace p3g
