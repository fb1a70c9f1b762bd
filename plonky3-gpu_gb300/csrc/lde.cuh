// lde.cuh -- batched coset low-degree extension (BabyBear, Goldilocks).
// Templates; lde_bb.cu and lde_gl.cu instantiate one field each.
//
// Computes, for a row-major h x w matrix of evaluations on the subgroup of
// order h, the coset LDE of height H = h * 2^b exactly as the reference's
// Radix2Dit::coset_lde_batch (radix2_dit.hpp:221-233: idft_batch, zero-pad,
// coset_dft_batch) followed, when bitrev_out is set, by
// p3_matrix::reverse_matrix_index_bits (util.hpp:33-45).
//
// Algebra used (exact field arithmetic, so results are bit-identical):
//   c_k = (1/h) sum_i e_i w_h^(-ik)                 (coefficients)
//   out[t*h + r] = LDE[bitrev_H(t*h + r)] = Y_t[bitrev_h(r)],
//   Y_t = DFT_h(c_k * g_t^k),  g_t = shift * w_H^(bitrev_b(t)),
// i.e. the bit-reversed LDE is 2^b independent size-h coset DFTs, each
// produced in bit-reversed order by a DIF network, so the zero padding is
// never materialised.
//
// h <= 2^10: one kernel; each CTA keeps a whole column tile on chip
// (read the trace once, write the LDE once).
// 2^10 < h <= 2^21: three passes of a four-step split h = N1 * N2:
//   pass 1: size-N2 inverse DFTs over rows i1 + N1*i2 (stride N1), twiddle
//           w_h^(-i1 k2), write scratch row i1 + N1*k2;
//   pass 2: size-N1 inverse DFT over contiguous rows, then per coset t the
//           scale c_k * g_t^k, size-N1 forward DFT and twiddle
//           g_t^(k2) w_h^(k2 m1), write out row t*h + bitrev(m1)*N2 + k2;
//   pass 3: size-N2 forward DFT over contiguous N2-row blocks, in place.
// 2^21 < h <= 2^26: the coefficients and each coset's transform through the
// split transform of dft.cuh (lde_big_run), same output layout.
// Every pass reads its tile straight from global memory into the registers
// of the first radix-32 super-stage and writes the last super-stage's
// registers straight back; shared memory only carries the exchange between
// super-stages (and, in pass 2, the coefficients between the inverse and the
// forward transforms).
#pragma once
#include <array>
#include <type_traits>
#include <vector>

#include "internal.hpp"
#include "ntt.cuh"

namespace p3g {

template <class F>
struct LdeCfg;
#ifndef P3G_LDE_BB_C13
#define P3G_LDE_BB_C13 16
#endif
#ifndef P3G_LDE_BB_C2
#define P3G_LDE_BB_C2 8
#endif
template <>
struct LdeCfg<FBB> {
    static constexpr int C13 = P3G_LDE_BB_C13;  // columns per tile, passes 1/3 and single (64-byte rows)
    static constexpr int C2 = P3G_LDE_BB_C2;    // pass 2 keeps two tiles: 32-byte rows, two CTAs per SM
    static constexpr int MAXT = 256;
    static constexpr uint32_t ONE_C = bb::R1;
};
template <>
struct LdeCfg<FGL> {
    static constexpr int C13 = 8;
    static constexpr int C2 = 4;
    static constexpr int MAXT = 256;
    static constexpr uint64_t ONE_C = 1;
};

// Minimum resident CTAs per SM of passes 1/3 and of pass 2 (launch bounds;
// settable at build time to compare register budgets).
#ifndef P3G_LDE_MINB13
#define P3G_LDE_MINB13 2
#endif
#ifndef P3G_LDE_MINB2
#define P3G_LDE_MINB2 2
#endif

// Resident CTAs per SM that pass 2's launch bounds ask for: at least
// P3G_LDE_MINB2 and enough for 16 warps, so a 128-thread tile (2^9 rows and
// fewer) gets the 128-register budget of the 256-thread one instead of
// 173 registers and 12% of the warps (measured at 2^18 x 128).
// (At most 16: tiny tiles of a few threads would ask for more CTAs than an
// SM holds.)
constexpr int lde_minb2(int threads) {
    return 512 / threads > P3G_LDE_MINB2 ? (512 / threads < 16 ? 512 / threads : 16) : P3G_LDE_MINB2;
}

constexpr int LDE_SINGLE_MAX = 10;  // single-kernel LDE up to h = 2^10
constexpr int LDE_PASS_MAX = 21;    // three-pass LDE up to h = 2^21
// above it, one more split h = 2^21 * B with B <= 32 (dft.cuh, big_run; B is
// bounded by the in-register roots, which go up to omega_32)
constexpr int LDE_BIG_MAX = LDE_PASS_MAX + 5;

// Prepared in-tile DFT twiddles (one table per context and field): for every
// LOGN in 1..DFT_TW_MAXLOG the stage-ordered table of the size-2^LOGN
// transform (ntt.cuh: ss_tw_size entries) as F::TW; the forward tables
// first, then the inverse ones.  Kernels copy their LOGN's table into shared
// memory instead of deriving every entry from the two-level root table (two
// loads, two products and, for BabyBear, a 64-bit Shoup quotient per entry
// and CTA).
constexpr int DFT_TW_MAXLOG = 11;
template <class T>
constexpr size_t dft_tw_block() {  // entries of one direction, LOGN = 1..11
    size_t n = 0;
    for (int L = 1; L <= DFT_TW_MAXLOG; ++L) n += size_t(ss_tw_size(L, ss_max_lr<T>()));
    return n;
}
template <class T>
constexpr size_t dft_tw_offset(int logn, bool inv) {
    size_t o = inv ? dft_tw_block<T>() : 0;
    for (int L = 1; L < logn; ++L) o += size_t(ss_tw_size(L, ss_max_lr<T>()));
    return o;
}
template <class F>
std::vector<typename F::TW> build_dft_tw() {
    using T = typename F::T;
    constexpr int MLR = ss_max_lr<T>();
    std::vector<typename F::TW> v(2 * dft_tw_block<T>());
    for (int L = 1; L <= DFT_TW_MAXLOG; ++L) {
        const uint64_t wf = F::root(unsigned(L)), wi = F::h_inv(wf);
        std::vector<uint64_t> pf(size_t(1) << L), pi(size_t(1) << L);
        uint64_t a = 1, b = 1;
        for (size_t e = 0; e < pf.size(); ++e) {
            pf[e] = a;
            pi[e] = b;
            a = F::h_mul(a, wf);
            b = F::h_mul(b, wi);
        }
        for (int i = 0; i < ss_tw_size(L, MLR); ++i) {
            const uint32_t e = ss_tw_exp(L, MLR, i);
            v[dft_tw_offset<T>(L, false) + size_t(i)] = F::h_tw(pf[e]);
            v[dft_tw_offset<T>(L, true) + size_t(i)] = F::h_tw(pi[e]);
        }
    }
    return v;
}
// Entry i of the stage-ordered table of the size-2^LOGN transform, from the
// root table (kernels without a prepared table).
template <class F, int LOGN>
__device__ __forceinline__ typename F::TW stage_tw(RootTab<F> roots, int i, bool inv) {
    const uint32_t e = ss_tw_exp(LOGN, ss_max_lr<typename F::T>(), i);
    return F::tw_from_const(inv ? roots.omega_inv(LOGN, e) : roots.omega(LOGN, e));
}

// out[i] = scale * base^i, all in const form.
template <class F>
__global__ void k_pow_table(typename F::T* out, typename F::T base, typename F::T scale, int n) {
    using T = typename F::T;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T r = LdeCfg<F>::ONE_C, b = base;
    unsigned e = unsigned(i);
    while (e) {
        if (e & 1) r = F::cmul(r, b);
        b = F::cmul(b, b);
        e >>= 1;
    }
    out[i] = F::cmul(r, scale);
}

// Prepared coset twists of every coset t < 2^log_b, shared by all CTAs:
// out[t*N + k] = s[k] * omega_H^(bitrev_b(t) * stride * k)   (N = 2^logn).
template <class F>
__global__ void k_pre_table(typename F::TW* out, const typename F::T* s, int logn, int log_b, int logH,
                            uint64_t stride, RootTab<F> roots) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= (int64_t(1) << (logn + log_b))) return;
    const int tc = int(i >> logn);
    const uint64_t k = uint64_t(i) & ((uint64_t(1) << logn) - 1);
    const uint64_t u = bitrev_dev(unsigned(tc), log_b);
    out[i] = F::tw_from_const(F::cmul(s[k], roots.omega(logH, u * stride * k)));
}

// h = 1: the LDE of a constant polynomial is constant.
template <class F>
__global__ void k_broadcast_row(const typename F::T* in, typename F::T* out, int w, int rows) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= int64_t(rows) * w) return;
    out[i] = in[i % w];
}

template <class F, int LOGN, int C>
struct Tile : DftShape<typename F::T, LOGN, C, LdeCfg<F>::MAXT> {};

// Grids of row blocks x column tiles are one-dimensional, the column tile
// varying fastest: the CTAs in flight together cover whole row spans, so
// every 128-byte line they touch is read or written in full while it is in
// L2, and the column-tile count has no 65535 limit (grid.y).
struct TileCoord {
    int64_t blk;  // row block
    int ct;       // column tile
};
template <int C>
__device__ __forceinline__ TileCoord tile_coord(int w) {
    const unsigned nct = unsigned(w + C - 1) / unsigned(C);
    const unsigned b = blockIdx.x;
    return {int64_t(b / nct), int(b % nct)};
}
inline dim3 tile_grid(int64_t nblk, int w, int C) {
    const int64_t n = nblk * ((int64_t(w) + C - 1) / C);
    if (n >= (int64_t(1) << 31)) throw Error(P3G_EUNSUPPORTED, "transform: grid of 2^31 or more CTAs");
    return dim3(unsigned(n));
}

// ---- group loads (first super-stage) and stores (last super-stage)
// Global rows i -> p0[i * s] (p0 already offset to this thread's column).
template <class T>
struct GLoad {
    const T* p0;
    int64_t s;
    bool ok;
    template <int R, int M>
    __device__ __forceinline__ void group(int base, T* x) const {
        const T* q = p0 + base * s;
        const int64_t st = int64_t(M) * s;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            x[k] = ok ? __ldg(q) : T(0);
            q += st;
        }
    }
};
// Shared tile row bitrev(i), times pre[i] (coefficients -> twisted coefficients).
// base < M (the first super-stage), so bitrev(base + M*k) is
// bitrev(base) + bitrev(M*k) with no common bit.
template <class F, class SH, int LOGN>
struct PermLoad {
    using T = typename F::T;
    const T* A;
    const typename F::TW* pre;
    int c;
    template <int R, int M>
    __device__ __forceinline__ void group(int base, T* x) const {
        const auto r0 = SH::row0(int(bitrev_dev(unsigned(base), LOGN)), c);
#pragma unroll
        for (int k = 0; k < R; ++k)
            x[k] = F::mul_tw(A[SH::at(r0, int(bitrev_ct(unsigned(M * k), LOGN)))], pre[base + M * k]);
    }
};
// Shared tile, natural positions (base is a multiple of 2^LR).
template <class T, class SH>
struct TileStore {
    T* A;
    int c;
    template <int LR>
    __device__ __forceinline__ void group(int base, const T* x) const {
        const auto r0 = SH::row0(base, c);
#pragma unroll
        for (int k = 0; k < (1 << LR); ++k) A[SH::at(r0, k)] = x[k];
    }
};
// x * c for a prepared twiddle (F::TW) or a const-form value (F::T); for
// Goldilocks both are the canonical value and the product is the same.
template <class F, class P>
__device__ __forceinline__ typename F::T post_mul(typename F::T x, P c) {
    if constexpr (std::is_same<P, typename F::TW>::value) return F::mul_tw(x, c);
    else return F::mulc(x, c);
}

// Global position p -> p0[p * s] (optionally times post[p]; post holds
// prepared twiddles or, with P = F::T, const-form values).
template <class F, bool POST, class P = typename F::TW>
struct GStore {
    using T = typename F::T;
    T* p0;
    int64_t s;
    const P* post;
    bool ok;
    template <int LR>
    __device__ __forceinline__ void group(int base, const T* x) const {
        if (!ok) return;
        T* q = p0 + base * s;
#pragma unroll
        for (int k = 0; k < (1 << LR); ++k) {
            *q = POST ? post_mul<F>(x[k], post[base + k]) : x[k];
            q += s;
        }
    }
};
// Global position p -> p0[bitrev_N(p) * s] * post[p] (pass 1: scratch rows
// i1 + N1*k2; post in const form).  With p = g*R + k, bitrev_N(p) =
// bitrev_r(k) * 2^(N-r) + bitrev_(N-r)(g): walk k in bit-reversed order so
// the pointer only advances.
template <class F, int LOGN>
struct BitrevStore {
    using T = typename F::T;
    T* p0;
    int64_t s;
    const T* post;
    bool ok;
    template <int LR>
    __device__ __forceinline__ void group(int base, const T* x) const {
        if (!ok) return;
        const int g = base >> LR;
        T* q = p0 + int64_t(bitrev_dev(unsigned(g), LOGN - LR)) * s;
        const int64_t st = s << (LOGN - LR);
#pragma unroll
        for (int j = 0; j < (1 << LR); ++j) {
            const int k = int(bitrev_ct(unsigned(j), LR));
            *q = F::mulc(x[k], post[base + k]);
            q += st;
        }
    }
};
// Global LDE rows for the final pass: bit-reversed order is contiguous;
// natural order scatters each position to bitrev_H(row).
template <class T>
struct OutStore {
    T* out;     // column-offset base
    int64_t w;
    int64_t row0;
    int logH;
    bool bitrev;
    bool ok;
    template <int LR>
    __device__ __forceinline__ void group(int base, const T* x) const {
        if (!ok) return;
        if (bitrev) {
            T* q = out + (row0 + base) * w;
#pragma unroll
            for (int k = 0; k < (1 << LR); ++k) {
                *q = x[k];
                q += w;
            }
        } else {
#pragma unroll
            for (int k = 0; k < (1 << LR); ++k)
                out[int64_t(bitrev_dev(unsigned(row0 + base + k), logH)) * w] = x[k];
        }
    }
};

// ------------------------------------------------------------ batches
// Every launch runs a batch of LDEs of one shape (log_h, log_b, shift): one
// trace for a single call, a whole height group for a batched commit.  The
// grids of the traces are laid end to end; a CTA finds its trace from the
// first CTA of each trace in the pass.  The batch is a kernel parameter
// (constant bank); larger batches take several launches.
constexpr int LDE_MAXJ = 64;
template <class T>
struct LdeJob {
    const T* in;  // h x w trace
    T* scr;       // pass-1 output, tiled by pass-2 column tiles (unused by the single kernel)
    T* mid;       // pass-2 output (the LDE itself when rows are bit-reversed)
    T* out;       // H x w LDE
    uint32_t w;
    uint32_t cta0[3];  // first CTA of this trace in pass 1 (or the single kernel), 2 and 3
};
template <class T>
struct LdeJobs {
    int n;
    LdeJob<T> job[LDE_MAXJ];
};
// This CTA's trace in pass `ps`, and the CTA's index within that trace's grid.
template <class T>
__device__ __forceinline__ const LdeJob<T>& lde_job(const LdeJobs<T>& J, int ps, unsigned& local) {
    int j = 0;
#pragma unroll 1
    while (j + 1 < J.n && J.job[j + 1].cta0[ps] <= blockIdx.x) ++j;
    local = blockIdx.x - J.job[j].cta0[ps];
    return J.job[j];
}
template <int C>
__device__ __forceinline__ TileCoord local_tile(unsigned local, int w) {
    const unsigned nct = unsigned(w + C - 1) / unsigned(C);
    return {int64_t(local / nct), int(local % nct)};
}

// ------------------------------------------------------------ single kernel
template <class F, int LOGN>
__global__ void __launch_bounds__(Tile<F, LOGN, LdeCfg<F>::C13>::THREADS)
k_lde_single(const LdeJobs<typename F::T> J, int log_b, int bitrev_out, const typename F::T* __restrict__ sq,
             RootTab<F> roots, const typename F::TW* __restrict__ gtwi, const typename F::TW* __restrict__ gtwf,
             const typename F::TW* __restrict__ gpre) {
    constexpr int C = LdeCfg<F>::C13;
    using SH = Tile<F, LOGN, C>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    T* B = A + SH::TILE;
    TW* twi = reinterpret_cast<TW*>(B + SH::TILE);
    TW* twf = twi + SH::TWA;
    TW* pre = twf + SH::TWA;
    unsigned local;
    const LdeJob<T>& jb = lde_job(J, 0, local);
    const int w = int(jb.w);
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const int col = int(local) * C + c;
    const bool ok = col < w;
    const int logH = LOGN + log_b;

    for (int e = tid; e < SH::TWN; e += NT) {
        twi[e] = gtwi ? gtwi[e] : stage_tw<F, LOGN>(roots, e, true);
        twf[e] = gtwf ? gtwf[e] : stage_tw<F, LOGN>(roots, e, false);
    }
    __syncthreads();
    {
        GLoad<T> ld{jb.in + col, w, ok};
        TileStore<T, SH> st{A, c};
        cta_dif<F, SH, LOGN, C, 1>(A, twi, t, c, ld, st);
    }
    for (int tc = 0; tc < (1 << log_b); ++tc) {
        const uint64_t u = bitrev_dev(unsigned(tc), log_b);
        for (int k = tid; k < N; k += NT)
            pre[k] = gpre ? gpre[tc * N + k] : F::tw_from_const(F::cmul(sq[k], roots.omega(logH, u * k)));
        __syncthreads();  // pre ready; A complete (first round) or B free (later rounds)
        PermLoad<F, SH, LOGN> ld{A, pre, c};
        OutStore<T> st{jb.out + col, w, int64_t(tc) * N, logH, bitrev_out != 0, ok};
        cta_dif<F, SH, LOGN, C, 0>(B, twf, t, c, ld, st);
        __syncthreads();  // pre and B reused by the next coset
    }
}

// ------------------------------------------------------------ pass 1 (LOGN = n2)
template <class F, int LOGN>
__global__ void __launch_bounds__(Tile<F, LOGN, LdeCfg<F>::C13>::THREADS, P3G_LDE_MINB13)
k_lde_pass1(const LdeJobs<typename F::T> J, int n1, RootTab<F> roots, const typename F::TW* __restrict__ gtwi) {
    constexpr int C = LdeCfg<F>::C13;
    using SH = Tile<F, LOGN, C>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    TW* tw = reinterpret_cast<TW*>(A + SH::TILE);
    T* post = reinterpret_cast<T*>(tw + SH::TWA);  // const form
    unsigned local;
    const LdeJob<T>& jb = lde_job(J, 0, local);
    const int w = int(jb.w);
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const TileCoord tc_ = local_tile<C>(local, w);
    const int col = tc_.ct * C + c;
    const bool ok = col < w;
    const int64_t i1 = tc_.blk;
    const int64_t N1 = int64_t(1) << n1;
    const int n = n1 + LOGN;

    for (int e = tid; e < SH::TWN; e += NT) tw[e] = gtwi ? gtwi[e] : stage_tw<F, LOGN>(roots, e, true);
    for (int e = tid; e < N; e += NT) post[e] = roots.omega_inv(n, uint64_t(i1) * bitrev_dev(e, LOGN));
    __syncthreads();
    // scratch is tiled by pass 2's column tiles: element (row r, column col)
    // at ((col / C2) * h + r) * C2 + col % C2, so that each pass-2 CTA reads
    // one contiguous block
    constexpr int C2 = LdeCfg<F>::C2;
    const int64_t h = int64_t(1) << n;
    T* dst = ok ? jb.scr + ((int64_t(col / C2) * h + i1) * C2 + col % C2) : jb.scr;
    GLoad<T> ld{jb.in + i1 * w + col, N1 * w, ok};
    BitrevStore<F, LOGN> st{dst, N1 * C2, post, ok};
    cta_dif<F, SH, LOGN, C, 1>(A, tw, t, c, ld, st);
}

// ------------------------------------------------------------ pass 2 (LOGN = n1)
template <class F, int LOGN>
__global__ void __launch_bounds__(Tile<F, LOGN, LdeCfg<F>::C2>::THREADS,
                                  lde_minb2(Tile<F, LOGN, LdeCfg<F>::C2>::THREADS))
k_lde_pass2(const LdeJobs<typename F::T> J, int n2, int log_b, const typename F::T* __restrict__ sp,
            const typename F::T* __restrict__ sq, RootTab<F> roots, const typename F::TW* __restrict__ gtwi,
            const typename F::TW* __restrict__ gtwf, const typename F::TW* __restrict__ gpre) {
    constexpr int C = LdeCfg<F>::C2;
    using SH = Tile<F, LOGN, C>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    T* B = A + SH::TILE;
    TW* twi = reinterpret_cast<TW*>(B + SH::TILE);
    TW* twf = twi + SH::TWA;
    TW* pre = twf + SH::TWA;
    T* post = reinterpret_cast<T*>(pre + N);  // const form
    unsigned local;
    const LdeJob<T>& jb = lde_job(J, 1, local);
    const int w = int(jb.w);
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const TileCoord tc_ = local_tile<C>(local, w);
    const int col = tc_.ct * C + c;
    const bool ok = col < w;
    const int64_t k2 = tc_.blk;
    const int64_t N2 = int64_t(1) << n2;
    const int n = LOGN + n2;
    const int64_t h = int64_t(1) << n;
    const int logH = n + log_b;

    for (int e = tid; e < SH::TWN; e += NT) {
        twi[e] = gtwi ? gtwi[e] : stage_tw<F, LOGN>(roots, e, true);
        twf[e] = gtwf ? gtwf[e] : stage_tw<F, LOGN>(roots, e, false);
    }
    __syncthreads();
    {
        GLoad<T> ld{jb.scr + (int64_t(tc_.ct) * h + int64_t(N) * k2) * C + c, C, ok};
        TileStore<T, SH> st{A, c};
        cta_dif<F, SH, LOGN, C, 1>(A, twi, t, c, ld, st);
    }
    const T sqk2 = sq[k2];
    uint64_t u_prev = 0;
    for (int tc = 0; tc < (1 << log_b); ++tc) {
        const uint64_t u = bitrev_dev(unsigned(tc), log_b);
        // post[k] = sq[k2] * omega_H^(k2 * (u + bitrev(k) * 2^b)): built from
        // the root table for the first coset, then moved on to the next coset
        // by one product with omega_H^(k2 * (u - u_prev)) (each thread owns
        // the entries it updates; the barrier after the last coset's
        // transform ended every read)
        const T step = tc ? roots.omega(logH, uint64_t(k2) * u - uint64_t(k2) * u_prev) : T(0);
        for (int k = tid; k < N; k += NT) {
            pre[k] = gpre ? gpre[tc * N + k]
                          : F::tw_from_const(F::cmul(sp[k], roots.omega(logH, u * uint64_t(N2) * k)));
            post[k] = tc ? F::cmul(post[k], step)
                         : F::cmul(sqk2, roots.omega(logH, uint64_t(k2) * (uint64_t(bitrev_dev(k, LOGN)) << log_b)));
        }
        u_prev = u;
        __syncthreads();
        PermLoad<F, SH, LOGN> ld{A, pre, c};
        GStore<F, true, T> st{jb.mid + (tc * h + k2) * w + col, N2 * w, post, ok};
        cta_dif<F, SH, LOGN, C, 0>(B, twf, t, c, ld, st);
        __syncthreads();
    }
}

// ------------------------------------------------------------ pass 3 (LOGN = n2)
template <class F, int LOGN>
__global__ void __launch_bounds__(Tile<F, LOGN, LdeCfg<F>::C13>::THREADS, P3G_LDE_MINB13)
k_lde_pass3(const LdeJobs<typename F::T> J, int n1, int log_b, int bitrev_out, RootTab<F> roots,
            const typename F::TW* __restrict__ gtwf) {
    constexpr int C = LdeCfg<F>::C13;
    using SH = Tile<F, LOGN, C>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    TW* tw = reinterpret_cast<TW*>(A + SH::TILE);
    unsigned local;
    const LdeJob<T>& jb = lde_job(J, 2, local);
    const int w = int(jb.w);
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const TileCoord tc_ = local_tile<C>(local, w);
    const int col = tc_.ct * C + c;
    const bool ok = col < w;
    const int64_t blk = tc_.blk;
    const int n = n1 + LOGN;
    const int logH = n + log_b;
    const int64_t base = blk * N;  // = t*h + s1*N2

    for (int e = tid; e < SH::TWN; e += NT) tw[e] = gtwf ? gtwf[e] : stage_tw<F, LOGN>(roots, e, false);
    __syncthreads();
    GLoad<T> ld{jb.mid + base * w + col, w, ok};
    OutStore<T> st{jb.out + col, w, base, logH, bitrev_out != 0, ok};
    cta_dif<F, SH, LOGN, C, 0>(A, tw, t, c, ld, st);
}

// ------------------------------------------------------------ host side
template <class Kern>
static void set_smem(Kern k, size_t bytes) {
    P3G_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

// The in-tile twiddle table of size 2^logn (nullptr when there is no table:
// the kernels then derive it from the root table).
template <class F>
static const typename F::TW* tw_table(const typename F::TW* dft_tw, int logn, bool inv) {
    return dft_tw && logn <= DFT_TW_MAXLOG ? dft_tw + dft_tw_offset<typename F::T>(logn, inv) : nullptr;
}

template <class F, int LOGN>
static void launch_single(const LdeJobs<typename F::T>& J, unsigned ctas, int log_b, int br, const typename F::T* sq,
                          const typename F::TW* pre, RootTab<F> roots, const typename F::TW* dft_tw,
                          cudaStream_t st) {
    using SH = Tile<F, LOGN, LdeCfg<F>::C13>;
    size_t smem = 2 * SH::TILE * sizeof(typename F::T) + (2 * SH::TWA + SH::N) * sizeof(typename F::TW);
    auto k = k_lde_single<F, LOGN>;
    set_smem(k, smem);
    k<<<ctas, SH::THREADS, smem, st>>>(J, log_b, br, sq, roots, tw_table<F>(dft_tw, LOGN, true),
                                       tw_table<F>(dft_tw, LOGN, false), pre);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F, int LOGN>
static void launch_pass1(const LdeJobs<typename F::T>& J, unsigned ctas, int n1, RootTab<F> roots,
                         const typename F::TW* dft_tw, cudaStream_t st) {
    using SH = Tile<F, LOGN, LdeCfg<F>::C13>;
    size_t smem = SH::TILE * sizeof(typename F::T) + SH::TWA * sizeof(typename F::TW) + SH::N * sizeof(typename F::T);
    auto k = k_lde_pass1<F, LOGN>;
    set_smem(k, smem);
    k<<<ctas, SH::THREADS, smem, st>>>(J, n1, roots, tw_table<F>(dft_tw, LOGN, true));
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F, int LOGN>
static void launch_pass2(const LdeJobs<typename F::T>& J, unsigned ctas, int n2, int log_b, const typename F::T* sp,
                         const typename F::T* sq, const typename F::TW* pre, RootTab<F> roots,
                         const typename F::TW* dft_tw, cudaStream_t st) {
    using SH = Tile<F, LOGN, LdeCfg<F>::C2>;
    size_t smem = 2 * SH::TILE * sizeof(typename F::T) + (2 * SH::TWA + SH::N) * sizeof(typename F::TW) +
                  SH::N * sizeof(typename F::T);
    auto k = k_lde_pass2<F, LOGN>;
    set_smem(k, smem);
    k<<<ctas, SH::THREADS, smem, st>>>(J, n2, log_b, sp, sq, roots, tw_table<F>(dft_tw, LOGN, true),
                                       tw_table<F>(dft_tw, LOGN, false), pre);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F, int LOGN>
static void launch_pass3(const LdeJobs<typename F::T>& J, unsigned ctas, int n1, int log_b, int br, RootTab<F> roots,
                         const typename F::TW* dft_tw, cudaStream_t st) {
    using SH = Tile<F, LOGN, LdeCfg<F>::C13>;
    size_t smem = SH::TILE * sizeof(typename F::T) + SH::TWA * sizeof(typename F::TW);
    auto k = k_lde_pass3<F, LOGN>;
    set_smem(k, smem);
    k<<<ctas, SH::THREADS, smem, st>>>(J, n1, log_b, br, roots, tw_table<F>(dft_tw, LOGN, false));
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

#define P3G_CASES_1_11(M) M(1) M(2) M(3) M(4) M(5) M(6) M(7) M(8) M(9) M(10) M(11)

template <class F>
static void pow_table(typename F::T* out, uint64_t base, uint64_t scale, int n, cudaStream_t st) {
    k_pow_table<F><<<ceil_div(n, 256), 256, 0, st>>>(out, F::to_const(base), F::to_const(scale), n);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F>
static void pre_table(typename F::TW* out, const typename F::T* s, int logn, int log_b, int logH, uint64_t stride,
                      RootTab<F> roots, cudaStream_t st) {
    const int64_t n = int64_t(1) << (logn + log_b);
    k_pre_table<F><<<unsigned(ceil_div(n, 256)), 256, 0, st>>>(out, s, logn, log_b, logH, stride, roots);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

// The four-step split of the three-pass LDE: h = 2^n1 * 2^n2.
inline int lde_n2(int log_h) { return (log_h + 1) / 2; }

// Tables of one LDE shape (log_h, log_b, shift), shared by every trace of
// that shape: [0] the first power table, [1] the second, [2] the prepared
// coset twists.  Sizes in bytes (0 = unused).
template <class F>
std::array<size_t, 3> lde_table_bytes(int log_h, int log_b) {
    using T = typename F::T;
    using TW = typename F::TW;
    if (log_h == 0) return {0, 0, 0};
    if (log_h <= LDE_SINGLE_MAX) return {sizeof(T) << log_h, 0, sizeof(TW) << (log_h + log_b)};
    const int n2 = lde_n2(log_h), n1 = log_h - n2;
    return {sizeof(T) << n1, sizeof(T) << n2, sizeof(TW) << (n1 + log_b)};
}
// Fills the shape's tables (three small kernels on `st`).
template <class F>
void lde_tables(int log_h, int log_b, uint64_t shift, void* const* tab, RootTab<F> roots, cudaStream_t st) {
    using T = typename F::T;
    using TW = typename F::TW;
    if (log_h == 0) return;
    const int64_t h = int64_t(1) << log_h;
    const uint64_t inv_h = F::h_inv(uint64_t(h) % F::P);
    if (log_h <= LDE_SINGLE_MAX) {
        pow_table<F>(static_cast<T*>(tab[0]), shift, inv_h, int(h), st);
        pre_table<F>(static_cast<TW*>(tab[2]), static_cast<const T*>(tab[0]), log_h, log_b, log_h + log_b, 1, roots,
                     st);
        return;
    }
    const int n2 = lde_n2(log_h), n1 = log_h - n2;
    const int64_t N2 = int64_t(1) << n2;
    pow_table<F>(static_cast<T*>(tab[0]), F::h_pow(shift, uint64_t(N2)), inv_h, int(int64_t(1) << n1), st);
    pow_table<F>(static_cast<T*>(tab[1]), shift, 1, int(N2), st);
    pre_table<F>(static_cast<TW*>(tab[2]), static_cast<const T*>(tab[0]), n1, log_b, log_h + log_b, uint64_t(N2),
                 roots, st);
}
// Pass-1 scratch of one trace of the three-pass LDE (elements).
template <class F>
size_t lde_scr_elems(int log_h, int w) {
    if (log_h <= LDE_SINGLE_MAX || w == 0) return 0;
    constexpr int C2 = LdeCfg<F>::C2;
    return size_t(ceil_div(w, C2)) * C2 << log_h;
}

// Launches the LDEs of a batch of traces of one shape (2^1 <= h <= 2^21)
// whose tables are filled: jobs[i] gives trace i's input, pass-1 scratch,
// pass-2 output (the output itself with bit-reversed rows) and output.  Every
// pass covers the whole batch (in launches of at most LDE_MAXJ traces).
template <class F>
void lde_batch(const std::vector<LdeJob<typename F::T>>& jobs, int log_h, int log_b, int bitrev_out,
               void* const* tab, RootTab<F> roots, const typename F::TW* dft_tw, cudaStream_t st) {
    using T = typename F::T;
    using TW = typename F::TW;
    const bool single = log_h <= LDE_SINGLE_MAX;
    const int n2 = lde_n2(log_h), n1 = log_h - n2;
    for (size_t j0 = 0; j0 < jobs.size(); j0 += LDE_MAXJ) {
        LdeJobs<T> J{};
        int64_t ctas[3] = {0, 0, 0};
        for (size_t j = j0; j < jobs.size() && j < j0 + LDE_MAXJ; ++j) {
            if (jobs[j].w == 0) continue;
            LdeJob<T> jb = jobs[j];
            const int64_t per[3] = {
                single ? ceil_div(jb.w, LdeCfg<F>::C13) : int64_t(tile_grid(int64_t(1) << n1, int(jb.w), LdeCfg<F>::C13).x),
                single ? 0 : int64_t(tile_grid(int64_t(1) << n2, int(jb.w), LdeCfg<F>::C2).x),
                single ? 0 : int64_t(tile_grid(int64_t(1) << (n1 + log_b), int(jb.w), LdeCfg<F>::C13).x)};
            for (int q = 0; q < 3; ++q) {
                jb.cta0[q] = uint32_t(ctas[q]);
                ctas[q] += per[q];
                if (ctas[q] >= (int64_t(1) << 31)) throw Error(P3G_EUNSUPPORTED, "coset_lde: batch grid too large");
            }
            J.job[J.n++] = jb;
        }
        if (J.n == 0) continue;
        if (single) {
            const T* sq = static_cast<const T*>(tab[0]);
            const TW* pre = static_cast<const TW*>(tab[2]);
            switch (log_h) {
#define C_(L) case L: launch_single<F, L>(J, unsigned(ctas[0]), log_b, bitrev_out, sq, pre, roots, dft_tw, st); break;
                C_(1) C_(2) C_(3) C_(4) C_(5) C_(6) C_(7) C_(8) C_(9) C_(10)
#undef C_
            }
            continue;
        }
        const T* sp = static_cast<const T*>(tab[0]);
        const T* sq = static_cast<const T*>(tab[1]);
        const TW* pre = static_cast<const TW*>(tab[2]);
        switch (n2) {
#define C_(L) case L: launch_pass1<F, L>(J, unsigned(ctas[0]), n1, roots, dft_tw, st); break;
            P3G_CASES_1_11(C_)
#undef C_
            default: throw Error(P3G_EUNSUPPORTED, "coset_lde: pass-1 size");
        }
        switch (n1) {
#define C_(L) case L: launch_pass2<F, L>(J, unsigned(ctas[1]), n2, log_b, sp, sq, pre, roots, dft_tw, st); break;
            P3G_CASES_1_11(C_)
#undef C_
            default: throw Error(P3G_EUNSUPPORTED, "coset_lde: pass-2 size");
        }
        switch (n2) {
#define C_(L) case L: launch_pass3<F, L>(J, unsigned(ctas[2]), n1, log_b, bitrev_out, roots, dft_tw, st); break;
            P3G_CASES_1_11(C_)
#undef C_
            default: throw Error(P3G_EUNSUPPORTED, "coset_lde: pass-3 size");
        }
    }
}

// Scratch buffers of one LDE call: [0] first power table, [1] second power
// table, [2] prepared coset twists, [3] pass-1 output (tiled by pass-2
// column tiles), [4] natural-order staging.  Sizes in bytes (0 = unused).
struct LdeScratch {
    size_t bytes[5] = {0, 0, 0, 0, 0};
    static size_t round(size_t b) { return (b + 255) / 256 * 256; }
    size_t total() const {
        size_t t = 0;
        for (size_t b : bytes) t += round(b);
        return t;
    }
};
template <class F>
LdeScratch lde_scratch(int log_h, int w, int log_b, int bitrev_out) {
    using T = typename F::T;
    LdeScratch s;
    if (log_h == 0 || w == 0) return s;
    const auto tb = lde_table_bytes<F>(log_h, log_b);
    for (int i = 0; i < 3; ++i) s.bytes[i] = tb[i];
    if (log_h <= LDE_SINGLE_MAX) return s;
    s.bytes[3] = sizeof(T) * lde_scr_elems<F>(log_h, w);
    s.bytes[4] = bitrev_out ? 0 : sizeof(T) * (size_t(w) << (log_h + log_b));
    return s;
}

// The LDE of one trace, on validated arguments (log_h <= LDE_PASS_MAX, shift
// canonical and non-zero) and scratch buffers sized by lde_scratch.
template <class F>
void lde_run(const typename F::T* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
             typename F::T* out, cudaStream_t st, RootTab<F> roots, const typename F::TW* dft_tw,
             void* const* buf) {
    using T = typename F::T;
    if (w == 0) return;
    if (log_h == 0) {
        int64_t total = (int64_t(1) << log_b) * w;
        k_broadcast_row<F><<<ceil_div(total, 256), 256, 0, st>>>(in, out, w, int(1 << log_b));
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
        return;
    }
    lde_tables<F>(log_h, log_b, shift, buf, roots, st);
    T* mid = bitrev_out || log_h <= LDE_SINGLE_MAX ? out : static_cast<T*>(buf[4]);
    const std::vector<LdeJob<T>> jobs{LdeJob<T>{in, static_cast<T*>(buf[3]), mid, out, uint32_t(w), {0, 0, 0}}};
    lde_batch<F>(jobs, log_h, log_b, bitrev_out, buf, roots, dft_tw, st);
}

// Bit-reversed LDEs of n traces of one shape (1 <= log_h <= 21) as one batch,
// with the shape's tables already filled (lde_tables) and each trace's pass-1
// scratch given (lde_scr_elems elements; null for the single kernel).
template <class F>
void lde_group_t(int log_h, int log_b, const void* const* in, void* const* scr, void* const* out, const uint32_t* w,
                 size_t n, void* const* tab, RootTab<F> roots, const typename F::TW* dft_tw, cudaStream_t st) {
    using T = typename F::T;
    std::vector<LdeJob<T>> jobs;
    jobs.reserve(n);
    for (size_t i = 0; i < n; ++i)
        jobs.push_back(LdeJob<T>{static_cast<const T*>(in[i]), static_cast<T*>(scr[i]), static_cast<T*>(out[i]),
                                 static_cast<T*>(out[i]), w[i], {0, 0, 0}});
    lde_batch<F>(jobs, log_h, log_b, 1, tab, roots, dft_tw, st);
}

// Context entry: validates, takes the scratch from the context's pool.
template <class F>
static void lde_impl(p3g_ctx* ctx, const typename F::T* in, int log_h, int w, int log_b, uint64_t shift,
                     int bitrev_out, typename F::T* out, cudaStream_t st, RootTab<F> roots,
                     const typename F::TW* dft_tw) {
    P3G_REQUIRE(log_h >= 0 && log_b >= 0, "coset_lde: negative size");
    P3G_REQUIRE(log_h + log_b <= int(F::TWO_ADICITY), "coset_lde: log_h + log_blowup exceeds two-adicity");
    if (log_h > LDE_BIG_MAX) throw Error(P3G_EUNSUPPORTED, "coset_lde: log_h > 26 is not supported");
    P3G_REQUIRE(shift % F::P != 0, "coset_lde: shift must be non-zero");
    if (w == 0) return;
    shift %= F::P;
    if (log_h > LDE_PASS_MAX) {
        lde_big(ctx, in, log_h, w, log_b, shift, bitrev_out, out, st);
        return;
    }
    const LdeScratch need = lde_scratch<F>(log_h, w, log_b, bitrev_out);
    void* buf[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    auto release = [&] {
        for (int i = 0; i < 5; ++i)
            if (buf[i]) ctx->release(buf[i], st);
    };
    try {
        for (int i = 0; i < 5; ++i)
            if (need.bytes[i]) buf[i] = ctx->alloc(need.bytes[i], st);
        lde_run<F>(in, log_h, w, log_b, shift, bitrev_out, out, st, roots, dft_tw, buf);
    } catch (...) {
        release();
        throw;
    }
    release();
}

}  // namespace p3g
