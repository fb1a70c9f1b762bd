// open.cu -- TwoAdicFriPcs::open's two passes over a resident BabyBear LDE
// (two_adic_fri_pcs.hpp:271-410):
//
//  * opened values, by barycentric interpolation on the LDE's coset
//    (compute_diff_invs + interpolate_coset_with_precomputation,
//    interpolation.hpp:93-180):
//        f_c(z) = (z^n - g^n) * sum_i W_i(z) f_c(g h_i),
//        W_i(z) = d_i / (z - g h_i),  d_i = h_i / (n g^(n-1)),  h_i = omega_n^i;
//  * the reduced opening (the FRI input) of the same rows:
//        q[k] += sum_p sum_c alpha^(a0 + p w + c) (f_c(z_p) - f_c(x_k)) / (z_p - x_k)
//              = sum_p (C_p - D_p[k]) / (z_p - x_k),
//        C_p = sum_c alpha_pc f_c(z_p),  D_p[k] = sum_c alpha_pc f_c(x_k),  x_k = g h_k.
//
// Both read the n x w LDE once, row-major with the columns across the threads
// of a warp (coalesced).  The opened values reduce down the rows: each CTA
// weights 2048 rows (the per-row inverses computed once per 256-row tile into
// shared memory) and writes per-CTA partial sums that a second kernel adds
// and scales by the vanishing factor.  The reduced opening reduces along each
// row: a warp owns 32 rows, each lane first inverts z_p - x_k for one of them,
// then the warp forms the 32 row dot products with the alpha powers (shared
// memory) and a shuffle reduction.  Rows may be stored in natural or
// bit-reversed order; q may be written in either order (bit-reversed is what
// prove_fri takes, two_adic_fri_pcs.hpp:412-419).
#include "internal.hpp"
#include "ntt.cuh"

namespace p3g {
namespace {

constexpr int OPEN_THREADS = 256;  // columns per CTA (partial pass) / 8 warps (reduce pass)
constexpr int OPEN_TILES = 8;      // 256-row tiles per CTA in the partial pass
constexpr int OPEN_MAXP = 4;       // points per call

__device__ __forceinline__ bb4 bb4_zero() { return {{0u, 0u, 0u, 0u}}; }
__device__ __forceinline__ bb4 bb4_fma_base(bb4 acc, uint32_t f, const bb4& wm) {  // acc + f*w, w Montgomery
#pragma unroll
    for (int k = 0; k < 4; ++k) acc.c[k] = bb::add(acc.c[k], bb::mmul(f, wm.c[k]));
    return acc;
}

// Partial sums over this CTA's rows: part[(blockIdx.x * m + p) * w + c] = sum_i W_i(z_p) f_c(i).
__global__ void __launch_bounds__(OPEN_THREADS)
k_open_partial(const uint32_t* __restrict__ lde, int log_n, int w, int bitrev_rows, int m,
               const bb4* __restrict__ z, uint32_t g, uint32_t cinv, RootTab<FBB> roots, bb4* __restrict__ part) {
    __shared__ bb4 W[OPEN_MAXP][OPEN_THREADS];
    const int64_t n = int64_t(1) << log_n;
    const int tid = threadIdx.x;
    const int c = blockIdx.y * OPEN_THREADS + tid;
    const int64_t row0 = int64_t(blockIdx.x) * OPEN_THREADS * OPEN_TILES;
    bb4 acc[OPEN_MAXP];
#pragma unroll
    for (int p = 0; p < OPEN_MAXP; ++p) acc[p] = bb4_zero();
    for (int t = 0; t < OPEN_TILES; ++t) {
        const int64_t tile0 = row0 + int64_t(t) * OPEN_THREADS;
        if (tile0 >= n) break;
        __syncthreads();  // the previous tile's weights are consumed
        {
            const int64_t r = tile0 + tid;
            if (r < n) {
                const uint64_t i = bitrev_rows ? bitrev_dev(unsigned(r), log_n) : uint64_t(r);
                const uint32_t hm = roots.omega(log_n, i);  // h_i, Montgomery form
                const uint32_t gh = bb::mmul(g, hm);        // g h_i
                const uint32_t dm = bb::mmul(bb::mmul(cinv, hm), bb::R2);  // d_i, Montgomery form
                for (int p = 0; p < m; ++p) {
                    bb4 diff = z[p];
                    diff.c[0] = bb::sub(diff.c[0], gh);
                    W[p][tid] = bb4_to_mont(bb4_scale_m(bb4_inv(diff), dm));
                }
            }
        }
        __syncthreads();
        if (c < w) {
            const int rows = int(n - tile0 < OPEN_THREADS ? n - tile0 : OPEN_THREADS);
            const uint32_t* src = lde + tile0 * w + c;
            for (int k = 0; k < rows; ++k) {
                const uint32_t f = __ldg(src + int64_t(k) * w);
#pragma unroll
                for (int p = 0; p < OPEN_MAXP; ++p)
                    if (p < m) acc[p] = bb4_fma_base(acc[p], f, W[p][k]);
            }
        }
    }
    if (c < w)
        for (int p = 0; p < m; ++p) part[(int64_t(blockIdx.x) * m + p) * w + c] = acc[p];
}

// out[p][c] = van_p * sum_b part[b][p][c]   (van in Montgomery form)
__global__ void k_open_finish(const bb4* __restrict__ part, int nb, int m, int w, const bb4* __restrict__ van_m,
                              bb4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m * w) return;
    const int p = i / w;
    bb4 s = bb4_zero();
    for (int b = 0; b < nb; ++b) s = bb4_add(s, part[int64_t(b) * m * w + i]);
    out[i] = bb4_mul_cm(s, van_m[p]);
}

__device__ __forceinline__ bb4 shfl_bb4(const bb4& v, int src) {
    bb4 r;
#pragma unroll
    for (int k = 0; k < 4; ++k) r.c[k] = __shfl_sync(0xffffffffu, v.c[k], src);
    return r;
}

// q[idx(k)] += sum_p (C_p - D_p[k]) / (z_p - x_k) for the CTA's 256 rows.
__global__ void __launch_bounds__(OPEN_THREADS)
k_pcs_reduce(const uint32_t* __restrict__ lde, int log_n, int w, int bitrev_rows, int m, const bb4* __restrict__ z,
             uint32_t g, const bb4* __restrict__ alpha_m, const bb4* __restrict__ cp, RootTab<FBB> roots,
             int q_bitrev, bb4* __restrict__ q) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bb4* A = reinterpret_cast<bb4*>(smem_raw);  // m * w alpha powers, Montgomery form
    for (int i = threadIdx.x; i < m * w; i += blockDim.x) A[i] = alpha_m[i];
    __syncthreads();
    const int64_t n = int64_t(1) << log_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = int64_t(blockIdx.x) * OPEN_THREADS + int64_t(warp) * 32;
    if (base >= n) return;
    // each lane inverts z_p - x_k for row base + lane
    bb4 inv[OPEN_MAXP];
    {
        const int64_t r = base + lane;
        const uint64_t k = r < n ? (bitrev_rows ? bitrev_dev(unsigned(r), log_n) : uint64_t(r)) : 0;
        const uint32_t xk = bb::mmul(g, roots.omega(log_n, k));
#pragma unroll
        for (int p = 0; p < OPEN_MAXP; ++p) {
            if (p < m) {
                bb4 diff = z[p];
                diff.c[0] = bb::sub(diff.c[0], xk);
                inv[p] = bb4_inv(diff);
            } else {
                inv[p] = bb4_zero();
            }
        }
    }
    const int rows = int(n - base < 32 ? n - base : 32);
    for (int j = 0; j < rows; ++j) {
        const int64_t r = base + j;
        const uint32_t* row = lde + r * w;
        bb4 d[OPEN_MAXP];
#pragma unroll
        for (int p = 0; p < OPEN_MAXP; ++p) d[p] = bb4_zero();
        for (int c = lane; c < w; c += 32) {
            const uint32_t f = __ldg(row + c);
#pragma unroll
            for (int p = 0; p < OPEN_MAXP; ++p)
                if (p < m) d[p] = bb4_fma_base(d[p], f, A[p * w + c]);
        }
        bb4 acc = bb4_zero();
#pragma unroll
        for (int p = 0; p < OPEN_MAXP; ++p) {
            if (p >= m) break;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                bb4 o = shfl_bb4(d[p], (lane + off) & 31);
                d[p] = bb4_add(d[p], o);  // every lane ends with the full sum
            }
            const bb4 ip = shfl_bb4(inv[p], j);
            acc = bb4_add(acc, bb4_mul_cm(bb4_sub(cp[p], d[p]), bb4_to_mont(ip)));
        }
        if (lane == 0) {
            const uint64_t k = bitrev_rows ? bitrev_dev(unsigned(r), log_n) : uint64_t(r);
            const uint64_t at = q_bitrev ? bitrev_dev(unsigned(k), log_n) : k;
            q[at] = bb4_add(q[at], acc);
        }
    }
}

// ---- host BabyBear^4 helpers (canonical in/out)
bb4 h_mul4(const bb4& a, const bb4& b) { return bb4_mul_cm(a, bb4_to_mont(b)); }
bb4 h_pow4(bb4 a, uint64_t e) {
    bb4 r = {{1u, 0u, 0u, 0u}};
    while (e) {
        if (e & 1) r = h_mul4(r, a);
        a = h_mul4(a, a);
        e >>= 1;
    }
    return r;
}

void check_open_args(const void* lde, uint32_t log_n, uint32_t w, uint32_t shift, const uint32_t* pts, uint32_t m) {
    P3G_REQUIRE(lde && pts, "pcs_open: null argument");
    P3G_REQUIRE(log_n <= 27, "pcs_open: log_n exceeds two-adicity");
    P3G_REQUIRE(w > 0 && w <= (1u << 20), "pcs_open: bad width");
    P3G_REQUIRE(m >= 1 && m <= uint32_t(OPEN_MAXP), "pcs_open: 1 to 4 points per call");
    P3G_REQUIRE(shift % bb::P != 0 && shift < bb::P, "pcs_open: shift must be canonical and non-zero");
    for (uint32_t i = 0; i < 4 * m; ++i) P3G_REQUIRE(pts[i] < bb::P, "pcs_open: point not canonical");
}

}  // namespace

void pcs_open_values(p3g_ctx* ctx, const uint32_t* lde, int log_n, int w, int bitrev_rows, uint32_t shift,
                     const uint32_t* h_points, int m, uint32_t* h_out, cudaStream_t st) {
    check_open_args(lde, uint32_t(log_n), uint32_t(w), shift, h_points, uint32_t(m));
    const uint64_t n = uint64_t(1) << log_n;
    // d_i = h_i * cinv, cinv = 1 / (n g^(n-1)) (interpolation.hpp compute_diff_invs)
    const uint32_t cinv = bb::h_inv(bb::h_mul(uint32_t(n % bb::P), bb::h_pow(shift, n - 1)));
    std::vector<bb4> z(m), van(m);
    for (int p = 0; p < m; ++p) {
        z[p] = {{h_points[4 * p], h_points[4 * p + 1], h_points[4 * p + 2], h_points[4 * p + 3]}};
        bb4 v = h_pow4(z[p], n);  // z^n - g^n
        v.c[0] = bb::sub(v.c[0], bb::h_pow(shift, n));
        van[p] = bb4_to_mont(v);
    }
    const int rows_per_cta = OPEN_THREADS * OPEN_TILES;
    const int nb = int((n + rows_per_cta - 1) / rows_per_cta);
    const size_t zbytes = sizeof(bb4) * m;
    bb4* dz = static_cast<bb4*>(ctx->alloc(zbytes * 2, st));
    bb4* part = static_cast<bb4*>(ctx->alloc(sizeof(bb4) * size_t(nb) * m * w, st));
    bb4* dout = static_cast<bb4*>(ctx->alloc(sizeof(bb4) * size_t(m) * w, st));
    try {
        P3G_CUDA(cudaMemcpyAsync(dz, z.data(), zbytes, cudaMemcpyHostToDevice, st));
        P3G_CUDA(cudaMemcpyAsync(dz + m, van.data(), zbytes, cudaMemcpyHostToDevice, st));
        dim3 grid(unsigned(nb), unsigned(ceil_div(w, OPEN_THREADS)));
        k_open_partial<<<grid, OPEN_THREADS, 0, st>>>(lde, log_n, w, bitrev_rows, m, dz, shift, cinv,
                                                      ctx->bb_roots(), part);
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
        k_open_finish<<<ceil_div(int64_t(m) * w, 256), 256, 0, st>>>(part, nb, m, w, dz + m, dout);
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
        P3G_CUDA(cudaMemcpyAsync(h_out, dout, sizeof(bb4) * size_t(m) * w, cudaMemcpyDeviceToHost, st));
        P3G_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
        ctx->release(dz, st);
        ctx->release(part, st);
        ctx->release(dout, st);
        throw;
    }
    ctx->release(dz, st);
    ctx->release(part, st);
    ctx->release(dout, st);
}

void pcs_reduce(p3g_ctx* ctx, const uint32_t* lde, int log_n, int w, int bitrev_rows, uint32_t shift,
                const uint32_t* h_points, int m, const uint32_t* h_opened, const uint32_t* h_alpha, uint64_t alpha_pow,
                int q_bitrev, uint32_t* q, cudaStream_t st) {
    check_open_args(lde, uint32_t(log_n), uint32_t(w), shift, h_points, uint32_t(m));
    P3G_REQUIRE(h_opened && h_alpha && q, "pcs_reduce: null argument");
    const size_t mw = size_t(m) * w;
    P3G_REQUIRE(mw * sizeof(bb4) <= 160 * 1024, "pcs_reduce: points x width above 10240");
    const bb4 alpha = {{h_alpha[0], h_alpha[1], h_alpha[2], h_alpha[3]}};
    std::vector<bb4> host(2 * size_t(m) + mw);  // z, C, alpha powers (Montgomery)
    bb4 a = h_pow4(alpha, alpha_pow);
    for (int p = 0; p < m; ++p) {
        host[p] = {{h_points[4 * p], h_points[4 * p + 1], h_points[4 * p + 2], h_points[4 * p + 3]}};
        bb4 cpv = {{0u, 0u, 0u, 0u}};
        for (int c = 0; c < w; ++c) {
            const uint32_t* o = h_opened + 4 * (size_t(p) * w + c);
            cpv = bb4_add(cpv, h_mul4(a, bb4{{o[0], o[1], o[2], o[3]}}));
            host[2 * m + size_t(p) * w + c] = bb4_to_mont(a);
            a = h_mul4(a, alpha);
        }
        host[m + p] = cpv;
    }
    bb4* dev = static_cast<bb4*>(ctx->alloc(sizeof(bb4) * host.size(), st));
    try {
        P3G_CUDA(cudaMemcpyAsync(dev, host.data(), sizeof(bb4) * host.size(), cudaMemcpyHostToDevice, st));
        const size_t smem = sizeof(bb4) * mw;
        P3G_CUDA(cudaFuncSetAttribute(k_pcs_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        const int64_t n = int64_t(1) << log_n;
        k_pcs_reduce<<<unsigned(ceil_div(n, OPEN_THREADS)), OPEN_THREADS, smem, st>>>(
            lde, log_n, w, bitrev_rows, m, dev, shift, dev + 2 * m, dev + m, ctx->bb_roots(), q_bitrev,
            reinterpret_cast<bb4*>(q));
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
    } catch (...) {
        ctx->release(dev, st);
        throw;
    }
    ctx->release(dev, st);
}

}  // namespace p3g
