// dft.cuh -- the Dft interface's other members on a batch of columns:
// dft_batch, idft_batch, coset_dft_batch, coset_idft_batch
// (radix2_dit.hpp:82-210; NttCuda's GPU twins, ntt_cuda.hpp:310-356).
// Templates; dft_bb.cu and dft_gl.cu instantiate one field each.
//
// All four are one transform
//     out[m] = alpha^m * sum_k (beta0 * sigma^k * x_k) * w^(+-k m)
//   dft:        sigma = 1,     beta0 = 1,   alpha = 1,          w^(+km)
//   idft:       sigma = 1,     beta0 = 1/h, alpha = 1,          w^(-km)
//   coset_dft:  sigma = shift, beta0 = 1,   alpha = 1,          w^(+km)
//   coset_idft: sigma = 1,     beta0 = 1/h, alpha = shift^-1,   w^(-km)
// (idft_batch's "DFT, reverse rows 1..h-1, scale 1/h" is the inverse-root
// transform scaled by 1/h; coset_idft_batch then scales row i by shift^-i).
//
// h <= 2^10: one kernel, a CTA per column tile (read once, write once).
// Larger h: two passes of the four-step split h = N1 * N2 used by the LDE,
// k = k2 + N2*k1, m = m1 + N1*m2:
//   pass A: for each k2, the size-N1 DIF over rows k2 + N2*k1 (stride N2),
//           inputs twisted by beta0 * sigma^(N2 k1), outputs by
//           sigma^k2 * w_h^(+-k2 m1) * alpha^m1, written to row p*N2 + k2
//           (p the DIF position of m1 = bitrev(p));
//   pass B: size-N2 DIF over each contiguous N2-row block, outputs scaled by
//           alpha^(N1 m2), rows in bit-reversed order (in place) or
//           scattered to natural order.
// 2^21 < h <= 2^26: those two passes as the inner transforms of one more
// split, plus an outer pass (big_run below).
#pragma once
#include "lde.cuh"

namespace p3g {

enum DftKind { DFT_FWD = 0, DFT_INV = 1, DFT_COSET = 2, DFT_COSET_INV = 3 };

// Global rows i -> p0[i * s], times the prepared twist pre[i] (shared memory).
template <class F>
struct GLoadTw {
    using T = typename F::T;
    const T* p0;
    int64_t s;
    const typename F::TW* pre;
    bool ok;
    template <int R, int M>
    __device__ __forceinline__ void group(int base, T* x) const {
        const T* q = p0 + base * s;
        const int64_t st = int64_t(M) * s;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            x[k] = ok ? F::mul_tw(__ldg(q), pre[base + M * k]) : T(0);
            q += st;
        }
    }
};
// OutStore with an optional per-position scale post[p] (shared memory).
template <class F>
struct ScaledOutStore {
    using T = typename F::T;
    T* out;  // column-offset base
    int64_t w;
    int64_t row0;
    int logH;
    bool bitrev;
    bool ok;
    const typename F::TW* post;  // nullptr: no scale
    template <int LR>
    __device__ __forceinline__ void group(int base, const T* x) const {
        if (!ok) return;
#pragma unroll
        for (int k = 0; k < (1 << LR); ++k) {
            const T v = post ? F::mul_tw(x[k], post[base + k]) : x[k];
            const int64_t row = row0 + base + k;
            out[(bitrev ? row : int64_t(bitrev_dev(unsigned(row), logH))) * w] = v;
        }
    }
};

// out[q] = base^(bitrev_logn(q)) as prepared twiddles (base in const form).
template <class F>
__global__ void k_bitrev_pow_tw(typename F::TW* out, typename F::T base, int logn) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (1 << logn)) return;
    unsigned e = bitrev_dev(unsigned(q), logn);
    typename F::T r = LdeCfg<F>::ONE_C, b = base;
    while (e) {
        if (e & 1) r = F::cmul(r, b);
        b = F::cmul(b, b);
        e >>= 1;
    }
    out[q] = F::tw_from_const(r);
}

template <class F, int LOGN>
using DftTile = Tile<F, LOGN, LdeCfg<F>::C13>;

// ------------------------------------------------------------ single kernel
template <class F, int LOGN, int INV>
__global__ void __launch_bounds__(DftTile<F, LOGN>::THREADS)
k_dft_single(const typename F::T* __restrict__ in, typename F::T* __restrict__ out, int w, int bitrev_out,
             const typename F::TW* __restrict__ gpre, const typename F::TW* __restrict__ gpost,
             const typename F::TW* __restrict__ gtw, RootTab<F> roots) {
    constexpr int C = LdeCfg<F>::C13;
    using SH = DftTile<F, LOGN>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    TW* tw = reinterpret_cast<TW*>(A + SH::TILE);
    TW* pre = tw + SH::TWA;
    TW* post = pre + N;
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const int col = tile_coord<C>(w).ct * C + c;
    const bool ok = col < w;
    for (int e = tid; e < SH::TWN; e += NT) tw[e] = gtw ? gtw[e] : stage_tw<F, LOGN>(roots, e, INV != 0);
    for (int e = tid; e < N; e += NT) {
        pre[e] = gpre[e];
        if (gpost) post[e] = gpost[e];
    }
    __syncthreads();
    GLoadTw<F> ld{in + col, w, pre, ok};
    ScaledOutStore<F> st{out + col, w, 0, LOGN, bitrev_out != 0, ok, gpost ? post : nullptr};
    cta_dif<F, SH, LOGN, C, INV>(A, tw, t, c, ld, st);
}

// ------------------------------------------------------------ pass A (LOGN = n1)
template <class F, int LOGN, int INV>
__global__ void __launch_bounds__(DftTile<F, LOGN>::THREADS, 2)
k_dft_pass_a(const typename F::T* __restrict__ in, typename F::T* __restrict__ mid, int w, int n2,
             const typename F::TW* __restrict__ gpre, const typename F::T* __restrict__ sq,
             const typename F::T* __restrict__ a1, const typename F::TW* __restrict__ gtw, RootTab<F> roots) {
    constexpr int C = LdeCfg<F>::C13;
    using SH = DftTile<F, LOGN>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    TW* tw = reinterpret_cast<TW*>(A + SH::TILE);
    TW* pre = tw + SH::TWA;
    TW* post = pre + N;
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const TileCoord tc_ = tile_coord<C>(w);
    const int col = tc_.ct * C + c;
    const bool ok = col < w;
    const int64_t k2 = tc_.blk;
    const int64_t N2 = int64_t(1) << n2;
    const int n = LOGN + n2;
    const T sk2 = sq[k2];
    for (int e = tid; e < SH::TWN; e += NT) tw[e] = gtw ? gtw[e] : stage_tw<F, LOGN>(roots, e, INV != 0);
    for (int e = tid; e < N; e += NT) {
        pre[e] = gpre[e];
        const unsigned m1 = bitrev_dev(unsigned(e), LOGN);
        const uint64_t ex = uint64_t(k2) * m1;
        T v = F::cmul(sk2, INV ? roots.omega_inv(n, ex) : roots.omega(n, ex));
        if (a1) v = F::cmul(v, a1[m1]);
        post[e] = F::tw_from_const(v);
    }
    __syncthreads();
    GLoadTw<F> ld{in + k2 * w + col, N2 * w, pre, ok};
    GStore<F, true> st{mid + k2 * w + col, N2 * w, post, ok};
    cta_dif<F, SH, LOGN, C, INV>(A, tw, t, c, ld, st);
}

// ------------------------------------------------------------ pass B (LOGN = n2)
template <class F, int LOGN, int INV>
__global__ void __launch_bounds__(DftTile<F, LOGN>::THREADS, 2)
k_dft_pass_b(const typename F::T* src, typename F::T* out, int w, int n1, int bitrev_out,
             const typename F::TW* __restrict__ gpost, const typename F::TW* __restrict__ gtw, RootTab<F> roots) {
    constexpr int C = LdeCfg<F>::C13;
    using SH = DftTile<F, LOGN>;
    using T = typename F::T;
    using TW = typename F::TW;
    constexpr int N = SH::N, NT = SH::THREADS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    TW* tw = reinterpret_cast<TW*>(A + SH::TILE);
    TW* post = tw + SH::TWA;
    const int tid = threadIdx.x, c = tid % C, t = tid / C;
    const TileCoord tc_ = tile_coord<C>(w);
    const int col = tc_.ct * C + c;
    const bool ok = col < w;
    const int64_t base = tc_.blk * N;
    for (int e = tid; e < SH::TWN; e += NT) tw[e] = gtw ? gtw[e] : stage_tw<F, LOGN>(roots, e, INV != 0);
    if (gpost)
        for (int e = tid; e < N; e += NT) post[e] = gpost[e];
    __syncthreads();
    GLoad<T> ld{src + base * w + col, w, ok};
    ScaledOutStore<F> st{out + col, w, base, n1 + LOGN, bitrev_out != 0, ok, gpost ? post : nullptr};
    cta_dif<F, SH, LOGN, C, INV>(A, tw, t, c, ld, st);
}

// ------------------------------------------------------------ host side
template <class F, int LOGN, int INV>
static void launch_dft_single(const typename F::T* in, typename F::T* out, int w, int br, const typename F::TW* pre,
                              const typename F::TW* post, const typename F::TW* dft_tw, RootTab<F> roots,
                              cudaStream_t st) {
    using SH = DftTile<F, LOGN>;
    const size_t smem = SH::TILE * sizeof(typename F::T) + (SH::TWA + 2 * SH::N) * sizeof(typename F::TW);
    auto k = k_dft_single<F, LOGN, INV>;
    set_smem(k, smem);
    const dim3 grid = tile_grid(1, w, LdeCfg<F>::C13);
    k<<<grid, SH::THREADS, smem, st>>>(in, out, w, br, pre, post, tw_table<F>(dft_tw, LOGN, INV != 0), roots);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F, int LOGN, int INV>
static void launch_dft_pass_a(const typename F::T* in, typename F::T* mid, int w, int n2, const typename F::TW* pre,
                              const typename F::T* sq, const typename F::T* a1, const typename F::TW* dft_tw,
                              RootTab<F> roots, cudaStream_t st) {
    using SH = DftTile<F, LOGN>;
    const size_t smem = SH::TILE * sizeof(typename F::T) + (SH::TWA + 2 * SH::N) * sizeof(typename F::TW);
    auto k = k_dft_pass_a<F, LOGN, INV>;
    set_smem(k, smem);
    const dim3 grid = tile_grid(int64_t(1) << n2, w, LdeCfg<F>::C13);
    k<<<grid, SH::THREADS, smem, st>>>(in, mid, w, n2, pre, sq, a1, tw_table<F>(dft_tw, LOGN, INV != 0), roots);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F, int LOGN, int INV>
static void launch_dft_pass_b(const typename F::T* mid, typename F::T* out, int w, int n1, int br,
                              const typename F::TW* post, const typename F::TW* dft_tw, RootTab<F> roots,
                              cudaStream_t st) {
    using SH = DftTile<F, LOGN>;
    const size_t smem = SH::TILE * sizeof(typename F::T) + (SH::TWA + SH::N) * sizeof(typename F::TW);
    auto k = k_dft_pass_b<F, LOGN, INV>;
    set_smem(k, smem);
    const dim3 grid = tile_grid(int64_t(1) << n1, w, LdeCfg<F>::C13);
    k<<<grid, SH::THREADS, smem, st>>>(mid, out, w, n1, br, post, tw_table<F>(dft_tw, LOGN, INV != 0), roots);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class F>
static void bitrev_pow_tw(typename F::TW* out, uint64_t base, int logn, cudaStream_t st) {
    k_bitrev_pow_tw<F><<<unsigned(ceil_div(int64_t(1) << logn, 256)), 256, 0, st>>>(out, F::to_const(base), logn);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

template <class F, int INV>
static void dft_run(const typename F::T* in, int log_h, int w, uint64_t sigma, uint64_t beta0, uint64_t alpha,
                    int bitrev_out, typename F::T* out, cudaStream_t st, RootTab<F> roots,
                    const typename F::TW* dft_tw, p3g_ctx* ctx) {
    using T = typename F::T;
    using TW = typename F::TW;
    const int64_t h = int64_t(1) << log_h;
    const bool scale_out = alpha != 1;
    std::vector<void*> bufs;
    auto take = [&](size_t bytes) {
        bufs.push_back(ctx->alloc(bytes, st));
        return bufs.back();
    };
    try {
        if (log_h <= LDE_SINGLE_MAX) {
            T* s = static_cast<T*>(take(sizeof(T) * h));
            TW* pre = static_cast<TW*>(take(sizeof(TW) * h));
            TW* post = scale_out ? static_cast<TW*>(take(sizeof(TW) * h)) : nullptr;
            pow_table<F>(s, sigma, beta0, int(h), st);
            pre_table<F>(pre, s, log_h, 0, log_h, 1, roots, st);
            if (post) bitrev_pow_tw<F>(post, alpha, log_h, st);
            switch (log_h) {
#define C_(L) case L: launch_dft_single<F, L, INV>(in, out, w, bitrev_out, pre, post, dft_tw, roots, st); break;
                C_(1) C_(2) C_(3) C_(4) C_(5) C_(6) C_(7) C_(8) C_(9) C_(10)
#undef C_
            }
        } else {
            const int n2 = (log_h + 1) / 2, n1 = log_h - n2;
            const int64_t N1 = int64_t(1) << n1, N2 = int64_t(1) << n2;
            T* sp = static_cast<T*>(take(sizeof(T) * N1));
            T* sq = static_cast<T*>(take(sizeof(T) * N2));
            TW* pre = static_cast<TW*>(take(sizeof(TW) * N1));
            T* a1 = scale_out ? static_cast<T*>(take(sizeof(T) * N1)) : nullptr;
            TW* post = scale_out ? static_cast<TW*>(take(sizeof(TW) * N2)) : nullptr;
            T* mid = bitrev_out ? out : static_cast<T*>(take(sizeof(T) * size_t(h) * w));
            pow_table<F>(sp, F::h_pow(sigma, uint64_t(N2)), beta0, int(N1), st);
            pre_table<F>(pre, sp, n1, 0, n1, 1, roots, st);
            pow_table<F>(sq, sigma, 1, int(N2), st);
            if (scale_out) {
                pow_table<F>(a1, alpha, 1, int(N1), st);
                bitrev_pow_tw<F>(post, F::h_pow(alpha, uint64_t(N1)), n2, st);
            }
            switch (n1) {
#define C_(L) case L: launch_dft_pass_a<F, L, INV>(in, mid, w, n2, pre, sq, a1, dft_tw, roots, st); break;
                P3G_CASES_1_11(C_)
#undef C_
                default: throw Error(P3G_EUNSUPPORTED, "dft: pass-A size");
            }
            switch (n2) {
#define C_(L) case L: launch_dft_pass_b<F, L, INV>(mid, out, w, n1, bitrev_out, post, dft_tw, roots, st); break;
                P3G_CASES_1_11(C_)
#undef C_
                default: throw Error(P3G_EUNSUPPORTED, "dft: pass-B size");
            }
        }
    } catch (...) {
        for (void* b : bufs) ctx->release(b, st);
        throw;
    }
    for (void* b : bufs) ctx->release(b, st);
}

// ------------------------------------------------------------ h > 2^21
// Above the two-pass limit the transform splits once more, h = A * B with
// A = 2^LDE_PASS_MAX and B = h / A <= 32 (h <= 2^LDE_BIG_MAX).  With input row
// k = B*k1 + k2 and output m = m1 + A*m2 (omega_h^(A*B) = 1):
//   out[m] = alpha^m * sum_k2 omega_B^(+-k2 m2) * (sigma * omega_h^(+-m1))^k2
//            * Z_k2[m1],
//   Z_k2[m1] = sum_k1 beta0 * (sigma^B)^k1 * x[B*k1 + k2] * omega_A^(+-k1 m1),
// so the inner transforms are one dft_run of size A over the A x (B*w) view of
// the matrix (row k1 holds rows B*k1 .. B*k1 + B - 1), and the outer step is,
// per inner output row and column, a twist and a size-B DIF in registers
// (position p holds m2 = bitrev_B(p)).
//   Bit-reversed output: the inner transforms write `out` in bit-reversed row
//   order, row j holding m1 = bitrev_A(j); output position B*j + p then holds
//   m = m1 + A*bitrev_B(p) = bitrev_h(B*j + p), so the outer step runs in
//   place on the B*w elements of row j.
//   Natural output: the inner output goes to a scratch matrix in natural
//   order (row j = m1) and the outer step writes output m to out row
//   row0 + m * rs (rs > 1 interleaves several transforms, as the LDE's cosets).
template <class F, int Q, int INV>
__global__ void __launch_bounds__(256)
k_big_outer(const typename F::T* z, typename F::T* out, int64_t w, int log_a, int log_h,
            typename F::T sigma_c, int inplace, int64_t row0, int64_t rs, const typename F::T* __restrict__ a1,
            const typename F::T* __restrict__ aB, RootTab<F> roots) {
    using T = typename F::T;
    constexpr int B = 1 << Q;
    const int64_t A = int64_t(1) << log_a;
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A * w) return;
    const int64_t j = i / w, c = i - j * w;
    const uint64_t m1 = inplace ? bitrev_dev(unsigned(j), log_a) : uint64_t(j);
    const T* zp = z + j * B * w + c;
    T v[B];
    const T f = F::cmul(INV ? roots.omega_inv(log_h, m1) : roots.omega(log_h, m1), sigma_c);
    T cur = f;
    v[0] = zp[0];
#pragma unroll
    for (int k2 = 1; k2 < B; ++k2) {
        v[k2] = F::mulc(zp[k2 * w], cur);
        if (k2 + 1 < B) cur = F::cmul(cur, f);
    }
    reg_dif<F, Q, INV>(v);
#pragma unroll
    for (int p = 0; p < B; ++p) {
        const int m2 = int(bitrev_ct(unsigned(p), Q));
        T y = v[p];
        if (a1) y = F::mulc(y, F::cmul(a1[m1], aB[m2]));
        if (inplace)
            out[(j * B + p) * w + c] = y;
        else
            out[(row0 + int64_t(m1 + uint64_t(A) * m2) * rs) * w + c] = y;
    }
}

template <class F, int Q, int INV>
static void launch_big_outer(const typename F::T* z, typename F::T* out, int64_t w, int log_a, int log_h,
                             typename F::T sigma_c, int inplace, int64_t row0, int64_t rs, const typename F::T* a1,
                             const typename F::T* aB, RootTab<F> roots, cudaStream_t st) {
    const int64_t n = (int64_t(1) << log_a) * w;
    k_big_outer<F, Q, INV><<<unsigned(ceil_div(n, 256)), 256, 0, st>>>(z, out, w, log_a, log_h, sigma_c, inplace,
                                                                      row0, rs, a1, aB, roots);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

// dft_run's transform for LDE_PASS_MAX < log_h <= LDE_BIG_MAX; natural-order
// output goes to rows row0 + m * rs of `out` (bit-reversed output: row0 = 0,
// rs = 1).  in and out must not overlap.
template <class F, int INV>
static void big_run(const typename F::T* in, int log_h, int w, uint64_t sigma, uint64_t beta0, uint64_t alpha,
                    int bitrev_out, typename F::T* out, int64_t row0, int64_t rs, cudaStream_t st, RootTab<F> roots,
                    const typename F::TW* dft_tw, p3g_ctx* ctx) {
    using T = typename F::T;
    const int la = LDE_PASS_MAX, q = log_h - la;
    const int64_t A = int64_t(1) << la, B = int64_t(1) << q, h = int64_t(1) << log_h;
    P3G_REQUIRE(w <= (1 << 17), "dft: width above 2^17 at log_h > 21");  // keeps A * w / 256 CTAs below 2^31
    std::vector<void*> bufs;
    auto take = [&](size_t bytes) {
        bufs.push_back(ctx->alloc(bytes, st));
        return bufs.back();
    };
    try {
        T* z = bitrev_out ? out : static_cast<T*>(take(sizeof(T) * size_t(h) * size_t(w)));
        dft_run<F, INV>(in, la, int(w * B), F::h_pow(sigma, uint64_t(B)), beta0, 1, bitrev_out, z, st, roots, dft_tw,
                        ctx);
        T* a1 = nullptr;
        T* aB = nullptr;
        if (alpha != 1) {
            a1 = static_cast<T*>(take(sizeof(T) * size_t(A)));
            aB = static_cast<T*>(take(sizeof(T) * size_t(B)));
            pow_table<F>(a1, alpha, 1, int(A), st);
            pow_table<F>(aB, F::h_pow(alpha, uint64_t(A)), 1, int(B), st);
        }
        const T sc = F::to_const(sigma);
        switch (q) {
#define C_(Q) case Q: launch_big_outer<F, Q, INV>(z, out, w, la, log_h, sc, bitrev_out, row0, rs, a1, aB, roots, st); break;
            C_(1) C_(2) C_(3) C_(4) C_(5)
#undef C_
            default: throw Error(P3G_EUNSUPPORTED, "dft: outer split size");
        }
    } catch (...) {
        for (void* b : bufs) ctx->release(b, st);
        throw;
    }
    for (void* b : bufs) ctx->release(b, st);
}

// The coset LDE above the three-pass limit (LDE_PASS_MAX < log_h <=
// LDE_BIG_MAX, arguments validated by lde_impl): the coefficients
// (1/h) IDFT_h(e) into a scratch matrix, then per coset t the size-h
// transform with sigma = g_t = shift * omega_H^(bitrev_b(t)):
//   bit-reversed LDE: block t (rows t*h .. t*h + h - 1) in bit-reversed order,
//   which is where the three-pass LDE puts coset t;
//   natural LDE: coset t's output m is LDE row bitrev_b(t) + 2^b * m.
template <class F>
static void lde_big_run(p3g_ctx* ctx, const typename F::T* in, int log_h, int w, int log_b, uint64_t shift,
                        int bitrev_out, typename F::T* out, cudaStream_t st, RootTab<F> roots,
                        const typename F::TW* dft_tw) {
    using T = typename F::T;
    const int64_t h = int64_t(1) << log_h;
    P3G_REQUIRE(w <= (1 << 17), "coset_lde: width above 2^17 at log_h > 21");  // big_run's limit, checked first
    T* coeffs = static_cast<T*>(ctx->alloc(sizeof(T) * size_t(h) * size_t(w), st));
    try {
        big_run<F, 1>(in, log_h, w, 1, F::h_inv(uint64_t(h) % F::P), 1, 0, coeffs, 0, 1, st, roots, dft_tw, ctx);
        const uint64_t wH = F::root(unsigned(log_h + log_b));
        for (int t = 0; t < (1 << log_b); ++t) {
            const unsigned u = bitrev_ct(unsigned(t), log_b);
            const uint64_t g = F::h_mul(shift, F::h_pow(wH, u));
            if (bitrev_out)
                big_run<F, 0>(coeffs, log_h, w, g, 1, 1, 1, out + size_t(t) * size_t(h) * size_t(w), 0, 1, st, roots,
                              dft_tw, ctx);
            else
                big_run<F, 0>(coeffs, log_h, w, g, 1, 1, 0, out, int64_t(u), int64_t(1) << log_b, st, roots, dft_tw,
                              ctx);
        }
    } catch (...) {
        ctx->release(coeffs, st);
        throw;
    }
    ctx->release(coeffs, st);
}

// Context entry: validates and dispatches one of the four kinds.
template <class F>
static void dft_impl(p3g_ctx* ctx, int kind, const typename F::T* in, int log_h, int w, uint64_t shift,
                     int bitrev_out, typename F::T* out, cudaStream_t st, RootTab<F> roots,
                     const typename F::TW* dft_tw) {
    P3G_REQUIRE(kind >= DFT_FWD && kind <= DFT_COSET_INV, "dft: unknown kind");
    P3G_REQUIRE(log_h >= 0 && log_h <= int(F::TWO_ADICITY), "dft: log_h exceeds two-adicity");
    if (log_h > LDE_BIG_MAX) throw Error(P3G_EUNSUPPORTED, "dft: log_h > 26 is not supported");
    const bool coset = kind == DFT_COSET || kind == DFT_COSET_INV;
    if (coset) P3G_REQUIRE(shift % F::P != 0, "dft: shift must be non-zero");
    if (w == 0) return;
    const int64_t h = int64_t(1) << log_h;
    if (log_h == 0) {  // every kind is the identity on one row
        P3G_CUDA(cudaMemcpyAsync(out, in, sizeof(typename F::T) * size_t(w), cudaMemcpyDeviceToDevice, st));
        return;
    }
    const bool inv = kind == DFT_INV || kind == DFT_COSET_INV;
    const uint64_t sigma = kind == DFT_COSET ? shift % F::P : 1;
    const uint64_t beta0 = inv ? F::h_inv(uint64_t(h) % F::P) : 1;
    const uint64_t alpha = kind == DFT_COSET_INV ? F::h_inv(shift % F::P) : 1;
    if (log_h > LDE_PASS_MAX) {
        if (inv)
            big_run<F, 1>(in, log_h, w, sigma, beta0, alpha, bitrev_out, out, 0, 1, st, roots, dft_tw, ctx);
        else
            big_run<F, 0>(in, log_h, w, sigma, beta0, alpha, bitrev_out, out, 0, 1, st, roots, dft_tw, ctx);
    } else if (inv) {
        dft_run<F, 1>(in, log_h, w, sigma, beta0, alpha, bitrev_out, out, st, roots, dft_tw, ctx);
    } else {
        dft_run<F, 0>(in, log_h, w, sigma, beta0, alpha, bitrev_out, out, st, roots, dft_tw, ctx);
    }
}

}  // namespace p3g
