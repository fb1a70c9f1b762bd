// fold.cu -- FRI fold_matrix over BabyBear^4.
//
// Reference: TwoAdicFriFolding<BabyBear, BabyBear4>::fold_matrix and fold_row
// (fri_folding.hpp:74-222).  Output i interpolates the arity values
// in[i*a .. i*a+a) at beta over the nodes t_j = x * w^bitrev(j), with
// x = omega_{2^log_height}^bitrev(i, log_height - log_arity).
//
// Arity 2 uses the closed form (e0 + e1)/2 + beta (e0 - e1) / (2x), which is
// the same field element as the reference's Lagrange sum (and also covers its
// beta == t_j early return).  x^-1 comes from the context's root table, not a
// per-thread exponentiation.  Arity 4 and 8 evaluate the reference's weights
// L_i = N * a^-1 / ((beta - t_i) x^(a-1) w^-(i)), N = prod_j (beta - t_j),
// as the same field elements without an inversion: N / (beta - t_i) is the
// product of the other factors, and 1 / (x^(a-1) w^-i) = x^-(a-1) w^i.  Its
// early return when beta equals a node is kept.
#include "internal.hpp"
#include "ntt.cuh"

namespace p3g {

__device__ __forceinline__ bb4 bb4_mul(const bb4& a, const bb4& b) { return bb4_mul_cm(a, bb4_to_mont(b)); }

// beta_dev, when given, holds beta (canonical) in device memory -- written by
// the device transcript -- and replaces the by-value argument.
__global__ void k_fold2(const bb4* __restrict__ in, bb4* __restrict__ out, uint64_t n, int log_height,
                        bb4 beta_m, const bb4* beta_dev, uint32_t inv2_m, RootTab<FBB> roots) {
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (beta_dev) beta_m = bb4_to_mont(*beta_dev);
    const int log_folded = log_height - 1;
    const uint32_t xinv_m = roots.omega_inv(log_height, bitrev_dev(unsigned(i), log_folded));
    const uint32_t inv2x_m = bb::mmul(xinv_m, inv2_m);
    const bb4 e0 = in[2 * i], e1 = in[2 * i + 1];
    const bb4 s = bb4_scale_m(bb4_add(e0, e1), inv2_m);
    const bb4 d = bb4_scale_m(bb4_sub(e0, e1), inv2x_m);
    out[i] = bb4_add(s, bb4_mul_cm(d, beta_m));
}

template <int LA>
__global__ void k_fold_general(const bb4* __restrict__ in, bb4* __restrict__ out, uint64_t n, int log_height,
                               bb4 beta, const bb4* beta_dev, uint32_t w_c, uint32_t winv_c, uint32_t arity_inv_c,
                               RootTab<FBB> roots) {
    constexpr int A = 1 << LA;
    uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (beta_dev) beta = *beta_dev;
    const int log_folded = log_height - LA;
    const uint32_t x_m = roots.omega(log_height, bitrev_dev(unsigned(i), log_folded));
    const uint32_t x = bb::mmul(x_m, 1u);
    // nodes t_j = x * w^j, then bit-reversed (fri_folding.hpp:109-125)
    uint32_t tn[A];
    uint32_t wp = x;
#pragma unroll
    for (int j = 0; j < A; ++j) {
        tn[j] = wp;
        wp = bb::mmul(wp, w_c);
    }
    uint32_t t[A];
#pragma unroll
    for (int j = 0; j < A; ++j) t[j] = tn[bitrev_ct(unsigned(j), LA)];
    bb4 ev[A];
#pragma unroll
    for (int j = 0; j < A; ++j) ev[j] = in[i * A + j];
    const bool beta_base = beta.c[1] == 0 && beta.c[2] == 0 && beta.c[3] == 0;
    if (beta_base) {
#pragma unroll
        for (int j = 0; j < A; ++j)
            if (beta.c[0] == t[j]) {
                out[i] = ev[j];
                return;
            }
    }
    // L_j = N a^-1 / ((beta - t_j) x^(a-1) w^-j) with N = prod_k (beta - t_k):
    // N / (beta - t_j) is the product of the other factors, so
    // L_j = a^-1 x^-(a-1) w^j prod_{k != j} (beta - t_k) -- the same field
    // element with no inversion (prefix products, then a running suffix).
    bb4 bmt[A];
#pragma unroll
    for (int j = 0; j < A; ++j) {
        bmt[j] = beta;
        bmt[j].c[0] = bb::sub(beta.c[0], t[j]);
    }
    bb4 pre[A];
    pre[0] = {{1, 0, 0, 0}};
#pragma unroll
    for (int j = 1; j < A; ++j) pre[j] = bb4_mul(pre[j - 1], bmt[j - 1]);
    const uint32_t xinv_m = roots.omega_inv(log_height, bitrev_dev(unsigned(i), log_folded));
    uint32_t s_m = arity_inv_c;  // a^-1 x^-(a-1) w^(A-1), Montgomery
#pragma unroll
    for (int k = 0; k < A - 1; ++k) s_m = bb::mmul(bb::mmul(s_m, xinv_m), w_c);
    bb4 suf = {{1, 0, 0, 0}}, res = {{0, 0, 0, 0}};
#pragma unroll
    for (int j = A - 1; j >= 0; --j) {
        const bb4 L = bb4_scale_m(bb4_mul(pre[j], suf), s_m);
        res = bb4_add(res, bb4_mul(ev[j], L));
        suf = bb4_mul(suf, bmt[j]);
        s_m = bb::mmul(s_m, winv_c);
    }
    out[i] = res;
}

void fold_bb4(p3g_ctx* ctx, const uint32_t* in, int log_height, int log_arity, const uint32_t beta[4],
              uint32_t* out, cudaStream_t st, const uint32_t* d_beta) {
    P3G_REQUIRE(log_arity >= 1 && log_arity <= 3, "fold_matrix: log_arity must be 1, 2 or 3");
    P3G_REQUIRE(log_arity <= log_height && log_height <= 27, "fold_matrix: bad log_height");
    if (!d_beta)
        for (int k = 0; k < 4; ++k) P3G_REQUIRE(beta[k] < bb::P, "fold_matrix: beta must be canonical");
    const uint64_t n = (uint64_t(1) << log_height) >> log_arity;
    const bb4* din = reinterpret_cast<const bb4*>(in);
    bb4* dout = reinterpret_cast<bb4*>(out);
    const bb4* bdev = reinterpret_cast<const bb4*>(d_beta);
    bb4 b = {{0, 0, 0, 0}};
    if (!d_beta) b = {{beta[0], beta[1], beta[2], beta[3]}};
    const unsigned grid = unsigned((n + 255) / 256);
    if (log_arity == 1) {
        bb4 bm = {{bb::to_mont(b.c[0]), bb::to_mont(b.c[1]), bb::to_mont(b.c[2]), bb::to_mont(b.c[3])}};
        k_fold2<<<grid, 256, 0, st>>>(din, dout, n, log_height, bm, bdev, bb::to_mont(bb::h_inv(2)), ctx->bb_roots());
        P3G_LAUNCHED();
    } else {
        const uint32_t w = bb::two_adic_generator(unsigned(log_arity));
        const uint32_t winv = bb::h_pow(w, (uint64_t(1) << log_arity) - 1);
        const uint32_t ainv = bb::h_pow(bb::h_inv(2), uint64_t(log_arity));
        if (log_arity == 2) {
            k_fold_general<2><<<grid, 256, 0, st>>>(din, dout, n, log_height, b, bdev, bb::to_mont(w),
                                                   bb::to_mont(winv), bb::to_mont(ainv), ctx->bb_roots());
        } else {
            k_fold_general<3><<<grid, 256, 0, st>>>(din, dout, n, log_height, b, bdev, bb::to_mont(w),
                                                   bb::to_mont(winv), bb::to_mont(ainv), ctx->bb_roots());
        }
        P3G_LAUNCHED();
    }
    P3G_CUDA(cudaGetLastError());
}

// y[i] += a * x[i] over BabyBear^4 (a in Montgomery form): prove_fri's mix-in of
// the next reduced opening, current[k] += beta^arity * next[k] (fri_prover.hpp:127-138).
__global__ void k_bb4_axpy(bb4* __restrict__ y, const bb4* __restrict__ x, uint64_t n, bb4 am, const bb4* a_dev) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (a_dev) am = bb4_to_mont(*a_dev);
    y[i] = bb4_add(y[i], bb4_mul_cm(x[i], am));
}

void bb4_axpy(p3g_ctx*, uint32_t* y, const uint32_t* x, uint64_t n, const uint32_t* a, cudaStream_t st,
              const uint32_t* d_a) {
    P3G_REQUIRE((n == 0 || (y && x)) && (a || d_a), "bb4_axpy: null argument");
    if (!d_a)
        for (int k = 0; k < 4; ++k) P3G_REQUIRE(a[k] < bb::P, "bb4_axpy: a must be canonical");
    if (n == 0) return;
    bb4 am = {{0, 0, 0, 0}};
    if (!d_a) am = {{bb::to_mont(a[0]), bb::to_mont(a[1]), bb::to_mont(a[2]), bb::to_mont(a[3])}};
    k_bb4_axpy<<<unsigned((n + 255) / 256), 256, 0, st>>>(reinterpret_cast<bb4*>(y), reinterpret_cast<const bb4*>(x),
                                                         n, am, reinterpret_cast<const bb4*>(d_a));
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

}  // namespace p3g
