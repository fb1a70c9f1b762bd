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
// A first kernel inverts z_p - x_k for every row and point (Montgomery's
// batch trick, four rows per thread) and stores the inverses and the weights
// W_k(z_p) = d_k / (z_p - x_k), n x points BabyBear^4 each.  Both passes then
// stream the n x w LDE once, row-major with the columns across the lanes:
// the opened values reduce down the rows (each CTA sums 2048 rows into
// per-CTA partials, which a last kernel adds and scales by the vanishing
// factor); the reduced opening reduces along each row (groups of 8 lanes take
// 4 rows at a time, 32-byte row segments per lane group, three shuffles).
// Products are summed unreduced in 64 bits and reduced once per four.  Rows
// may be stored in natural or bit-reversed order; q may be written in either
// order (bit-reversed is what prove_fri takes, two_adic_fri_pcs.hpp:412-419).
#include "internal.hpp"
#include "ntt.cuh"

namespace p3g {
namespace {

constexpr int OPEN_THREADS = 256;  // 8 warps per CTA
constexpr int OPEN_MAXP = 4;       // points per call

__device__ __forceinline__ bb4 bb4_zero() { return {{0u, 0u, 0u, 0u}}; }

// Sums of products f * w (f, w canonical, each product below p^2 < 2^61.9)
// are kept in 64 bits and folded every four products with 2^32 = R1 (mod p):
// x = hi 2^32 + lo = hi R1 + lo < 2^60 + 2^32, so four more products still fit.
// One 64-bit multiply-add per product and one per fold replace a modular
// product per product; the accumulator is reduced to [0, p) once at the end.
__device__ __forceinline__ uint64_t fold64(uint64_t x) {
    return (x >> 32) * uint64_t(bb::R1) + (x & 0xffffffffull);
}
__device__ __forceinline__ uint32_t reduce64(uint64_t x) {  // x mod p for any x < 2^64
    const uint32_t q = uint32_t(x) * bb::PINV;
    const uint32_t qh = __umulhi(q, bb::P);
    const uint32_t hi = uint32_t(x >> 32);
    uint32_t r = hi - qh;  // x / 2^32 mod p, in (-p, 2^32 - 1]
    if (hi < qh) r += bb::P;
    if (r >= bb::P) r -= bb::P;
    if (r >= bb::P) r -= bb::P;
    return bb::mmul(r, bb::R2);  // times 2^32
}

constexpr int OPEN_SLAB = 512;    // rows per CTA in the opened-values pass
constexpr int OPEN_BATCH = 4;     // rows per thread in the inversion kernel

// inv[p][r] = 1 / (z_p - x_k) (Montgomery form) and, if wgt, wgt[p][r] =
// d_k / (z_p - x_k) (canonical), for storage rows r (k = the row's natural index).
__global__ void __launch_bounds__(OPEN_THREADS)
k_open_weights(int log_n, int bitrev_rows, int m, const bb4* __restrict__ z, uint32_t g, uint32_t cinv,
               RootTab<FBB> roots, bb4* __restrict__ inv, bb4* __restrict__ wgt) {
    const int64_t n = int64_t(1) << log_n;
    const int64_t r0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * OPEN_BATCH;
    if (r0 >= n) return;
    const int cnt = int(n - r0 < OPEN_BATCH ? n - r0 : OPEN_BATCH);
    uint32_t xk[OPEN_BATCH], dm[OPEN_BATCH];
#pragma unroll
    for (int i = 0; i < OPEN_BATCH; ++i) {
        const int64_t r = r0 + (i < cnt ? i : 0);
        const uint64_t k = bitrev_rows ? bitrev_dev(unsigned(r), log_n) : uint64_t(r);
        const uint32_t hm = roots.omega(log_n, k);      // h_k, Montgomery form
        xk[i] = bb::mmul(g, hm);                         // x_k = g h_k
        dm[i] = bb::mmul(bb::mmul(cinv, hm), bb::R2);   // d_k, Montgomery form
    }
    for (int p = 0; p < m; ++p) {
        bb4 a[OPEN_BATCH], pre[OPEN_BATCH];
#pragma unroll
        for (int i = 0; i < OPEN_BATCH; ++i) {
            a[i] = z[p];
            a[i].c[0] = bb::sub(a[i].c[0], xk[i]);
            pre[i] = i == 0 ? a[0] : bb4_mul_cm(pre[i - 1], bb4_to_mont(a[i]));
        }
        bb4 t = bb4_inv(pre[OPEN_BATCH - 1]);  // 1 / (a_0 ... a_3)
#pragma unroll
        for (int i = OPEN_BATCH - 1; i >= 0; --i) {
            const bb4 ai = i == 0 ? t : bb4_mul_cm(t, bb4_to_mont(pre[i - 1]));  // 1 / a_i
            if (i > 0) t = bb4_mul_cm(t, bb4_to_mont(a[i]));
            if (i < cnt) {
                inv[int64_t(p) * n + r0 + i] = bb4_to_mont(ai);
                if (wgt) wgt[int64_t(p) * n + r0 + i] = bb4_scale_m(ai, dm[i]);
            }
        }
    }
}

// Opened-value partial sums.  Warp (cg, rs) of a CTA covers 32 columns of
// column group cg and rows [slab0 + rs * span, + span); partial index
// (blockIdx.x * rsplit + rs) holds sum_i W_i(z_p) f_c(i) over those rows.
// The next sixteen rows' loads are issued before the current sixteen rows'
// products so that enough bytes are in flight per SM to cover the latency.
template <int M>
__global__ void __launch_bounds__(OPEN_THREADS)
k_open_partial(const uint32_t* __restrict__ lde, int log_n, int w, int cgs, int rsplit,
               const bb4* __restrict__ wgt, bb4* __restrict__ part) {
    constexpr int U = 16;
    const int64_t n = int64_t(1) << log_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp >= cgs * rsplit) return;
    const int cg = warp % cgs, rs = warp / cgs;
    const int c = (blockIdx.y * cgs + cg) * 32 + lane;
    const int64_t span = OPEN_SLAB / rsplit;
    const int64_t r_begin = int64_t(blockIdx.x) * OPEN_SLAB + rs * span;
    const int64_t r_end = r_begin + span < n ? r_begin + span : n;
    uint64_t acc[M][4];
#pragma unroll
    for (int p = 0; p < M; ++p)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[p][j] = 0;
    const bool ok = c < w;
    const uint32_t* col = lde + (ok ? c : 0);
    // software pipeline: the next U rows are loaded while the current ones are multiplied
    uint32_t f[U], g[U];
#pragma unroll
    for (int k = 0; k < U; ++k) f[k] = (ok && r_begin + k < r_end) ? __ldg(col + (r_begin + k) * w) : 0u;
    for (int64_t r0 = r_begin; r0 < r_end; r0 += U) {
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const int64_t rn = r0 + U + k;
            g[k] = (ok && rn < r_end) ? __ldg(col + rn * w) : 0u;
        }
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const int64_t r = r0 + k < r_end ? r0 + k : r_begin;  // f is 0 past the end
#pragma unroll
            for (int p = 0; p < M; ++p) {
                const bb4 wv = wgt[int64_t(p) * n + r];  // the same address across the warp
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[p][j] += uint64_t(f[k]) * wv.c[j];
            }
            if ((k & 3) == 3)
#pragma unroll
                for (int p = 0; p < M; ++p)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[p][j] = fold64(acc[p][j]);
        }
#pragma unroll
        for (int k = 0; k < U; ++k) f[k] = g[k];
    }
    if (ok) {
        const int64_t pi = int64_t(blockIdx.x) * rsplit + rs;
#pragma unroll
        for (int p = 0; p < M; ++p) {
            bb4 v;
#pragma unroll
            for (int j = 0; j < 4; ++j) v.c[j] = reduce64(acc[p][j]);
            part[(pi * M + p) * w + c] = v;
        }
    }
}

// out[p][c] = van_p * sum_b part[b][p][c]   (van in Montgomery form); one CTA per output
__global__ void __launch_bounds__(OPEN_THREADS)
k_open_finish(const bb4* __restrict__ part, int nb, int m, int w, const bb4* __restrict__ van_m,
              bb4* __restrict__ out) {
    __shared__ bb4 red[OPEN_THREADS / 32];
    const int i = blockIdx.x;  // p * w + c
    bb4 s = bb4_zero();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s = bb4_add(s, part[int64_t(b) * m * w + i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int e = 0; e < 4; ++e) s.c[e] = bb::add(s.c[e], __shfl_xor_sync(0xffffffffu, s.c[e], off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        bb4 t = red[0];
        for (int k = 1; k < OPEN_THREADS / 32; ++k) t = bb4_add(t, red[k]);
        out[i] = bb4_mul_cm(t, van_m[i / w]);
    }
}

// q[at(k)] += sum_p (C_p - D_p[k]) inv[p][r] for the CTA's 256 rows: groups of
// 8 lanes take 4 rows at a time (a 32-byte row segment per lane group each
// step, a row's loads issued before its products), reduce their partial dot
// products with 3 shuffles, and one lane of the group adds the row's term.
template <int M>
__global__ void __launch_bounds__(OPEN_THREADS)
k_pcs_reduce(const uint32_t* __restrict__ lde, int log_n, int w, int bitrev_rows,
             const bb4* __restrict__ inv, const bb4* __restrict__ alpha_m, const bb4* __restrict__ cp, int q_bitrev,
             bb4* __restrict__ q) {
    constexpr int U = 16;  // loads per lane issued together (columns sub + 8k)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bb4* A = reinterpret_cast<bb4*>(smem_raw);  // M * w alpha powers, canonical
    for (int i = threadIdx.x; i < M * w; i += blockDim.x) A[i] = alpha_m[i];
    __syncthreads();
    const int64_t n = int64_t(1) << log_n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = lane >> 3, sub = lane & 7;
    const int64_t base = int64_t(blockIdx.x) * OPEN_THREADS + int64_t(warp) * 32;
    if (base >= n) return;
    const int rows = int(n - base < 32 ? n - base : 32);
    for (int j0 = 0; j0 < rows; j0 += 4) {  // uniform across the warp
        const int j = j0 + grp;
        const bool live = j < rows;
        const int64_t r = base + (live ? j : 0);
        const uint32_t* row = lde + r * w;
        uint64_t t[M][4];
#pragma unroll
        for (int p = 0; p < M; ++p)
#pragma unroll
            for (int e = 0; e < 4; ++e) t[p][e] = 0;
        for (int cb = 0; cb < w; cb += 8 * U) {
            uint32_t f[U];
#pragma unroll
            for (int k = 0; k < U; ++k) {
                const int c = cb + sub + 8 * k;
                f[k] = (live && c < w) ? __ldg(row + c) : 0u;
            }
#pragma unroll
            for (int k = 0; k < U; ++k) {
                const int c = cb + sub + 8 * k;
                const int cc = c < w ? c : 0;  // f is 0 past the row's end
#pragma unroll
                for (int p = 0; p < M; ++p) {
                    const bb4 av = A[p * w + cc];
#pragma unroll
                    for (int e = 0; e < 4; ++e) t[p][e] += uint64_t(f[k]) * av.c[e];
                }
                if ((k & 3) == 3)
#pragma unroll
                    for (int p = 0; p < M; ++p)
#pragma unroll
                        for (int e = 0; e < 4; ++e) t[p][e] = fold64(t[p][e]);
            }
        }
        bb4 d[M];
#pragma unroll
        for (int p = 0; p < M; ++p)
#pragma unroll
            for (int e = 0; e < 4; ++e) d[p].c[e] = reduce64(t[p][e]);
        bb4 acc = bb4_zero();
#pragma unroll
        for (int p = 0; p < M; ++p) {
#pragma unroll
            for (int off = 4; off > 0; off >>= 1)
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    d[p].c[e] = bb::add(d[p].c[e], __shfl_xor_sync(0xffffffffu, d[p].c[e], off));
            acc = bb4_add(acc, bb4_mul_cm(bb4_sub(cp[p], d[p]), inv[int64_t(p) * n + r]));
        }
        if (live && sub == 0) {
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

// cinv = 1 / (n g^(n-1)) (interpolation.hpp compute_diff_invs)
static uint32_t open_cinv(uint64_t n, uint32_t shift) {
    return bb::h_inv(bb::h_mul(uint32_t(n % bb::P), bb::h_pow(shift, n - 1)));
}

// inverses (and weights) of every row into pool buffers inv / wgt (n * m bb4 each)
static void open_weights(p3g_ctx* ctx, int log_n, int bitrev_rows, int m, const bb4* dz, uint32_t shift, bb4* inv,
                         bb4* wgt, cudaStream_t st) {
    const int64_t n = int64_t(1) << log_n;
    const int64_t threads = (n + OPEN_BATCH - 1) / OPEN_BATCH;
    k_open_weights<<<unsigned(ceil_div(threads, OPEN_THREADS)), OPEN_THREADS, 0, st>>>(
        log_n, bitrev_rows, m, dz, shift, open_cinv(uint64_t(n), shift), ctx->bb_roots(), inv, wgt);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

struct PoolBufs {  // pool allocations released in stream order, also on errors
    p3g_ctx* ctx;
    cudaStream_t st;
    std::vector<void*> v;
    void* take(size_t bytes) {
        v.push_back(ctx->alloc(bytes, st));
        return v.back();
    }
    ~PoolBufs() {
        for (void* p : v) ctx->release(p, st);
    }
};

void pcs_open_values(p3g_ctx* ctx, const uint32_t* lde, int log_n, int w, int bitrev_rows, uint32_t shift,
                     const uint32_t* h_points, int m, uint32_t* h_out, cudaStream_t st) {
    check_open_args(lde, uint32_t(log_n), uint32_t(w), shift, h_points, uint32_t(m));
    const uint64_t n = uint64_t(1) << log_n;
    std::vector<bb4> host(2 * size_t(m));  // points, then vanishing factors z^n - g^n (Montgomery)
    for (int p = 0; p < m; ++p) {
        host[p] = {{h_points[4 * p], h_points[4 * p + 1], h_points[4 * p + 2], h_points[4 * p + 3]}};
        bb4 v = h_pow4(host[p], n);
        v.c[0] = bb::sub(v.c[0], bb::h_pow(shift, n));
        host[m + p] = bb4_to_mont(v);
    }
    const int groups = ceil_div(w, 32);
    const int cgs = groups < 8 ? groups : 8;  // column groups per CTA
    int rsplit = 8 / cgs;                     // row splits per CTA
    while (rsplit & (rsplit - 1)) --rsplit;   // a power of two divides the slab
    const int nbx = int((n + OPEN_SLAB - 1) / OPEN_SLAB);
    const int nparts = nbx * rsplit;
    PoolBufs b{ctx, st, {}};
    bb4* dz = static_cast<bb4*>(b.take(sizeof(bb4) * host.size()));
    bb4* inv = static_cast<bb4*>(b.take(sizeof(bb4) * n * m));
    bb4* wgt = static_cast<bb4*>(b.take(sizeof(bb4) * n * m));
    bb4* part = static_cast<bb4*>(b.take(sizeof(bb4) * size_t(nparts) * m * w));
    bb4* dout = static_cast<bb4*>(b.take(sizeof(bb4) * size_t(m) * w));
    P3G_CUDA(cudaMemcpyAsync(dz, host.data(), sizeof(bb4) * host.size(), cudaMemcpyHostToDevice, st));
    open_weights(ctx, log_n, bitrev_rows, m, dz, shift, inv, wgt, st);
    dim3 grid(unsigned(nbx), unsigned(ceil_div(groups, cgs)));
    switch (m) {
#define C_(M) case M: k_open_partial<M><<<grid, OPEN_THREADS, 0, st>>>(lde, log_n, w, cgs, rsplit, wgt, part); break;
        C_(1) C_(2) C_(3) C_(4)
#undef C_
    }
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
    k_open_finish<<<unsigned(m * w), OPEN_THREADS, 0, st>>>(part, nparts, m, w, dz + m, dout);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
    P3G_CUDA(cudaMemcpyAsync(h_out, dout, sizeof(bb4) * size_t(m) * w, cudaMemcpyDeviceToHost, st));
    P3G_CUDA(cudaStreamSynchronize(st));
}

void pcs_reduce(p3g_ctx* ctx, const uint32_t* lde, int log_n, int w, int bitrev_rows, uint32_t shift,
                const uint32_t* h_points, int m, const uint32_t* h_opened, const uint32_t* h_alpha, uint64_t alpha_pow,
                int q_bitrev, uint32_t* q, cudaStream_t st) {
    check_open_args(lde, uint32_t(log_n), uint32_t(w), shift, h_points, uint32_t(m));
    P3G_REQUIRE(h_opened && h_alpha && q, "pcs_reduce: null argument");
    const size_t mw = size_t(m) * w;
    P3G_REQUIRE(mw * sizeof(bb4) <= 160 * 1024, "pcs_reduce: points x width above 10240");
    const uint64_t n = uint64_t(1) << log_n;
    const bb4 alpha = {{h_alpha[0], h_alpha[1], h_alpha[2], h_alpha[3]}};
    std::vector<bb4> host(2 * size_t(m) + mw);  // points, C_p, alpha powers
    bb4 a = h_pow4(alpha, alpha_pow);
    for (int p = 0; p < m; ++p) {
        host[p] = {{h_points[4 * p], h_points[4 * p + 1], h_points[4 * p + 2], h_points[4 * p + 3]}};
        bb4 cpv = {{0u, 0u, 0u, 0u}};
        for (int c = 0; c < w; ++c) {
            const uint32_t* o = h_opened + 4 * (size_t(p) * w + c);
            cpv = bb4_add(cpv, h_mul4(a, bb4{{o[0], o[1], o[2], o[3]}}));
            host[2 * m + size_t(p) * w + c] = a;
            a = h_mul4(a, alpha);
        }
        host[m + p] = cpv;
    }
    PoolBufs b{ctx, st, {}};
    bb4* dev = static_cast<bb4*>(b.take(sizeof(bb4) * host.size()));
    bb4* inv = static_cast<bb4*>(b.take(sizeof(bb4) * n * m));
    P3G_CUDA(cudaMemcpyAsync(dev, host.data(), sizeof(bb4) * host.size(), cudaMemcpyHostToDevice, st));
    open_weights(ctx, log_n, bitrev_rows, m, dev, shift, inv, nullptr, st);
    const size_t smem = sizeof(bb4) * mw;
    const unsigned blocks = unsigned(ceil_div(int64_t(n), OPEN_THREADS));
    switch (m) {
#define C_(M)                                                                                                   \
    case M:                                                                                                     \
        P3G_CUDA(cudaFuncSetAttribute(k_pcs_reduce<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))); \
        k_pcs_reduce<M><<<blocks, OPEN_THREADS, smem, st>>>(lde, log_n, w, bitrev_rows, inv, dev + 2 * m, dev + m, \
                                                            q_bitrev, reinterpret_cast<bb4*>(q));               \
        break;
        C_(1) C_(2) C_(3) C_(4)
#undef C_
    }
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}

}  // namespace p3g
