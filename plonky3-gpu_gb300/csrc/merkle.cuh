// merkle.cuh -- Poseidon2 Merkle kernels (templates; instantiated per round
// schedule in merkle_s*.cu so that the unrolled permutations compile in
// parallel translation units).
//
// Every kernel has exactly one call site of the unrolled permutation: the
// sponge loop fills one rate chunk per iteration, and a compression with an
// injected row hash runs its two permutations as two iterations of one loop.
#pragma once
#include <algorithm>
#include <type_traits>

#include "internal.hpp"
#include "poseidon2.cuh"

namespace p3g {

constexpr int MAXG = 64;  // matrices per equal-height group (kernel-parameter space)

template <class T>
struct Group {
    int n = 0;
    int vec = 0;  // single matrix, width % 4 == 0, 16-byte aligned rows (BabyBear)
    const T* ptr[MAXG];
    uint32_t w[MAXG];
};

// Sponge over the concatenated row r of the group (overwrite absorb,
// padding_free_sponge.hpp:63-87); leaves the state (internal form) in s.
// s0, when given, is the state (internal form) after an earlier part of the
// row whose length was a multiple of RATE: the sponge resumes from it.
template <class H, int D, int RF, int RP>
__device__ __forceinline__ void hash_group(const Group<typename H::T>& g, uint64_t r,
                                           const typename H::Params& p, typename H::T* s,
                                           const typename H::T* s0) {
    using T = typename H::T;
#pragma unroll
    for (int i = 0; i < H::W; ++i) s[i] = s0 ? s0[i] : T(0);
    int m = 0;
    uint32_t c = 0;
#pragma unroll 1
    for (;;) {
        int filled = 0;
        if (g.n == 1) {
            const uint32_t w = g.w[0];
            const T* row = g.ptr[0] + r * w;
            bool done = false;
            if constexpr (std::is_same<T, uint32_t>::value) {
                if (g.vec && c + 8 <= w) {
                    const uint4* rv = reinterpret_cast<const uint4*>(row + c);
                    uint4 a = __ldg(rv), b = __ldg(rv + 1);
                    s[0] = H::absorb(a.x); s[1] = H::absorb(a.y); s[2] = H::absorb(a.z); s[3] = H::absorb(a.w);
                    s[4] = H::absorb(b.x); s[5] = H::absorb(b.y); s[6] = H::absorb(b.z); s[7] = H::absorb(b.w);
                    filled = 8;
                    done = true;
                }
            }
            if (!done) {
#pragma unroll
                for (int i = 0; i < H::RATE; ++i)
                    if (c + i < w) s[i] = H::absorb(__ldg(row + c + i));
                filled = c < w ? int(min(uint32_t(H::RATE), w - c)) : 0;
            }
            c += filled;
        } else {
            // A chunk inside one matrix's row takes RATE loads from one
            // pointer (most chunks); one that spans matrices goes element by
            // element below.  With every element on that general path the
            // 64-trace batched commit's step took 6% longer (83.5 against
            // 78.5 ms on one GB300).  The row pointer is recomputed per chunk
            // from shared memory: keeping it (and the width) in registers
            // across the permutation measured 5% slower.
            while (m < g.n && c >= g.w[m]) {
                ++m;
                c = 0;
            }
            if (m < g.n && c + H::RATE <= g.w[m]) {
                const T* q = g.ptr[m] + r * g.w[m] + c;
#pragma unroll
                for (int i = 0; i < H::RATE; ++i) s[i] = H::absorb(__ldg(q + i));
                c += H::RATE;
                filled = H::RATE;
            }
#pragma unroll
            for (int i = 0; i < H::RATE; ++i) {
                if (filled == i) {
                    while (m < g.n && c >= g.w[m]) {
                        ++m;
                        c = 0;
                    }
                    if (m < g.n) {
                        s[i] = H::absorb(__ldg(g.ptr[m] + r * g.w[m] + c));
                        ++c;
                        filled = i + 1;
                    }
                }
            }
        }
        if (filled == 0) break;
        H::template perm<D, RF, RP>(s, p);
        if (filled < H::RATE) break;
    }
}

// ---------------------------------------------------------------- row hashing
// All equal-height groups of a tree (the tallest group's leaves and every
// injected group's row hashes) are hashed by one persistent kernel: work
// units of HASH_ROWS rows are handed out through an atomic counter, units of
// the most expensive groups first, so small groups never leave SMs idle.
// rows (= threads) per work unit (settable at build time, -DP3G_HASH_ROWS=,
// to compare unit sizes)
#ifndef P3G_HASH_ROWS
#define P3G_HASH_ROWS 256
#endif
constexpr int HASH_ROWS = P3G_HASH_ROWS;

template <class T>
struct HashEntry {
    const T* ptr;
    uint32_t width;
    uint32_t pad;
};
template <class T>
struct HashGroup {
    uint64_t rows;
    uint64_t unit0;  // first work unit of the group
    T* out;          // rows x DIG digests
    uint32_t ent0;   // entries [ent0, ent0 + nent)
    uint32_t nent;
    uint32_t vec;    // single matrix, width % 4 == 0, 16-byte aligned
    uint32_t pad;
    // A group hashed in parts (staged build): the sponge states (rows x W,
    // internal form) the part resumes from, and, for every part but the
    // last, the states it leaves instead of digests.  Both null otherwise.
    const T* state_in;
    T* state_out;
};
// Device descriptor block: [counter (8 bytes, zeroed per launch) | groups | entries];
// a launch takes a run of at most MAXG consecutive groups.
constexpr size_t HASH_DESC_HEADER = 256;

template <class H, int D, int RF, int RP>
__global__ void __launch_bounds__(HASH_ROWS) k_hash_groups(typename H::Params p, const HashGroup<typename H::T>* groups,
                                                           int ngroups, const HashEntry<typename H::T>* ents,
                                                           uint64_t total_units, unsigned long long* counter) {
    using T = typename H::T;
    __shared__ HashGroup<T> sg[MAXG];
    __shared__ Group<T> cur;
    __shared__ unsigned long long unit;
    __shared__ int cur_g;
    for (int i = threadIdx.x; i < ngroups; i += blockDim.x) sg[i] = groups[i];
    if (threadIdx.x == 0) cur_g = -1;
    __syncthreads();
#pragma unroll 1
    for (;;) {
        if (threadIdx.x == 0) unit = atomicAdd(counter, 1ull);
        __syncthreads();
        const uint64_t u = unit;
        if (u >= total_units) return;
        int g = 0;
        while (g + 1 < ngroups && sg[g + 1].unit0 <= u) ++g;
        if (g != cur_g) {  // stage the group's matrix list in shared memory
            __syncthreads();
            const uint32_t n = sg[g].nent;
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                cur.ptr[i] = ents[sg[g].ent0 + i].ptr;
                cur.w[i] = ents[sg[g].ent0 + i].width;
            }
            if (threadIdx.x == 0) {
                cur.n = int(n);
                cur.vec = int(sg[g].vec);
                cur_g = g;
            }
            __syncthreads();
        }
        const uint64_t r = (u - sg[g].unit0) * HASH_ROWS + threadIdx.x;
        if (r < sg[g].rows) {
            T s[H::W];
            const T* s0 = sg[g].state_in ? sg[g].state_in + r * H::W : nullptr;
            hash_group<H, D, RF, RP>(cur, r, p, s, s0);
            if (T* so = sg[g].state_out) {
#pragma unroll
                for (int i = 0; i < H::W; ++i) so[r * H::W + i] = s[i];
            } else {
                T* o = sg[g].out + r * H::DIG;
#pragma unroll
                for (int i = 0; i < H::DIG; ++i) o[i] = H::squeeze(s[i]);
            }
        }
        __syncthreads();  // `unit` and `cur` are rewritten next iteration
    }
}

// parent[j] = compress(child[2j], child[2j+1] or the zero digest); with inj,
// parent[j] = compress(parent[j], inj[j]) (merkle_tree.hpp:149-176,
// fri_merkle_tree_mmcs.hpp:77-92).
template <class H, int D, int RF, int RP>
__device__ __forceinline__ void compress_node(const typename H::Params& p, const typename H::T* __restrict__ child,
                                              uint64_t nchild, typename H::T* __restrict__ parent, uint64_t j,
                                              const typename H::T* __restrict__ inj) {
    using T = typename H::T;
    T s[H::W];
    const int iters = inj ? 2 : 1;
#pragma unroll 1
    for (int it = 0; it < iters; ++it) {
        if (it == 0) {
#pragma unroll
            for (int i = 0; i < H::W; ++i) s[i] = 0;
#pragma unroll
            for (int i = 0; i < H::DIG; ++i) s[i] = H::absorb(child[2 * j * H::DIG + i]);
            if (2 * j + 1 < nchild) {
#pragma unroll
                for (int i = 0; i < H::DIG; ++i) s[H::DIG + i] = H::absorb(child[(2 * j + 1) * H::DIG + i]);
            }
        } else {
#pragma unroll
            for (int i = 0; i < H::DIG; ++i) s[H::DIG + i] = H::absorb(inj[j * H::DIG + i]);
#pragma unroll
            for (int i = 2 * H::DIG; i < H::W; ++i) s[i] = 0;
        }
        H::template perm<D, RF, RP>(s, p);
    }
#pragma unroll
    for (int i = 0; i < H::DIG; ++i) parent[j * H::DIG + i] = H::squeeze(s[i]);
}

template <class H, int D, int RF, int RP>
__global__ void __launch_bounds__(128) k_compress_level(typename H::Params p, const typename H::T* __restrict__ child,
                                                        uint64_t nchild, typename H::T* __restrict__ parent,
                                                        uint64_t nparent, const typename H::T* __restrict__ inj) {
    uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= nparent) return;
    compress_node<H, D, RF, RP>(p, child, nchild, parent, j, inj);
}

// The top levels of a tree, each of at most TAIL_NODES parents, in one CTA,
// one level after the other: the compressions of k_compress_level without a
// launch per level (small trees and the tops of large ones are latency-bound).
constexpr int TAIL_NODES = 256;
constexpr int TAIL_MAX_LEVELS = 40;
template <class T>
struct TailLevels {
    int n;
    struct Level {
        const T* child;
        T* parent;
        const T* inj;
        uint32_t nchild, nparent;
    } lev[TAIL_MAX_LEVELS];
};

template <class H, int D, int RF, int RP>
__global__ void __launch_bounds__(TAIL_NODES) k_compress_tail(typename H::Params p, TailLevels<typename H::T> t) {
#pragma unroll 1
    for (int l = 0; l < t.n; ++l) {
        const auto& lv = t.lev[l];
        if (threadIdx.x < lv.nparent) compress_node<H, D, RF, RP>(p, lv.child, lv.nchild, lv.parent, threadIdx.x, lv.inj);
        __syncthreads();  // the next level reads this one's digests
    }
}

// BabyBear: compressions with one 16-lane group per node (p2_bb16_coop), for
// levels too small to fill the GPU with one thread per node.  With one level
// the grid covers its nodes; with several (the top of a tree) one CTA of
// COOP_THREADS runs them in order.
constexpr int COOP_THREADS = 1024;
constexpr uint64_t COOP_TAIL_NODES = COOP_THREADS / 16;  // nodes of one pass of the CTA
constexpr uint64_t COOP_MAX_NODES = 8192;                // larger levels: one thread per node

template <int D, int RF, int RP>
__global__ void __launch_bounds__(COOP_THREADS) k_compress_coop(P2BB16 p, TailLevels<uint32_t> t) {
    const int i = threadIdx.x & 15;
    const CoopConsts cc = coop_consts(p, i);
    const uint64_t g = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 4;
    const uint64_t ng = (uint64_t(gridDim.x) * blockDim.x) >> 4;
#pragma unroll 1
    for (int l = 0; l < t.n; ++l) {
        const auto& lv = t.lev[l];
#pragma unroll 1
        for (uint64_t base = 0; base < lv.nparent; base += ng) {  // uniform trip count: every lane shuffles
            if (base + (g & ~uint64_t(1)) >= lv.nparent) break;  // both groups of this warp idle from here on
            const uint64_t j = base + g;
            const bool on = j < lv.nparent;
            uint32_t x = 0;
            if (on) {
                if (i < 8) x = lv.child[2 * j * 8 + i];
                else if (2 * j + 1 < lv.nchild) x = lv.child[(2 * j + 1) * 8 + i - 8];
            }
            x = p2_bb16_coop<D, RF, RP>(HBB::absorb(x), p, cc, i);
            if (lv.inj) {  // compress(node, injected row digest)
                if (i >= 8) x = HBB::absorb(on ? lv.inj[j * 8 + i - 8] : 0u);
                x = p2_bb16_coop<D, RF, RP>(x, p, cc, i);
            }
            if (on && i < 8) lv.parent[j * 8 + i] = HBB::squeeze(x);
        }
        if (t.n > 1) __syncthreads();  // one CTA: the next level reads this one
    }
}

template <class H, int D, int RF, int RP>
__global__ void __launch_bounds__(128) k_permute(typename H::Params p, typename H::T* states, uint64_t n) {
    using T = typename H::T;
    uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n) return;
    T s[H::W];
#pragma unroll
    for (int i = 0; i < H::W; ++i) s[i] = H::absorb(states[j * H::W + i]);
    H::template perm<D, RF, RP>(s, p);
#pragma unroll
    for (int i = 0; i < H::W; ++i) states[j * H::W + i] = H::squeeze(s[i]);
}

// Proof-of-work search, DuplexChallenger::grind (duplex_challenger.hpp:234-251).
// The challenger's sponge state and pending inputs are fixed; a candidate
// witness c is observed as the two elements F(c mod 2^32) and F(c >> 32)
// (observe_witness, :57-61) and one element is sampled: state word RATE - 1
// after the next duplexing.  With RATE - 1 inputs pending, the low half fills
// the buffer and duplexes first, so such a candidate costs two permutations
// (one call site, run twice).  Thread t tries base + t, base + t + T, ... in
// increasing order and stops once the smallest hit so far is at or below its
// next candidate, so *found ends as the smallest hit in [base, base + count).
template <class T, int W>
struct GrindArgs {
    T state[W];  // sponge state with the pending inputs written over its first words, internal form
    uint32_t n_input;
    uint64_t mask;
};

template <class H, int D, int RF, int RP>
__global__ void __launch_bounds__(128) k_grind(typename H::Params p, const GrindArgs<typename H::T, H::W>* args,
                                               uint64_t base, uint64_t count, unsigned long long* found) {
    using T = typename H::T;
    __shared__ GrindArgs<T, H::W> a;  // from device memory: written by the host or by a transcript kernel
    if (threadIdx.x == 0) a = *args;
    __syncthreads();
    const int k = int(a.n_input);
    const int passes = k + 1 == H::RATE ? 2 : 1;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t off = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; off < count; off += stride) {
        const uint64_t c = base + off;
        if (*reinterpret_cast<volatile unsigned long long*>(found) <= c) break;
        const T lo = H::absorb(H::from_u32(uint32_t(c)));
        const T hi = H::absorb(H::from_u32(uint32_t(c >> 32)));
        T s[H::W];
#pragma unroll
        for (int i = 0; i < H::W; ++i) s[i] = a.state[i];
#pragma unroll
        for (int i = 0; i < H::RATE; ++i) {
            if (i == k) s[i] = lo;
            if (i == k + 1) s[i] = hi;
        }
#pragma unroll 1
        for (int pass = 0; pass < passes; ++pass) {
            if (pass == 1) s[0] = hi;
            H::template perm<D, RF, RP, false>(s, p);
        }
        if ((uint64_t(H::squeeze(s[H::RATE - 1])) & a.mask) == 0) atomicMin(found, c);
    }
}

// Calls fn.template operator()<D, RF, RP>() for a supported round schedule.
template <class Fn>
void dispatch_bb(const p3g_ctx* ctx, const Fn& fn) {
    if (!ctx->has_p2bb) throw Error(P3G_ESTATE, "Poseidon2 constants for BabyBear are not set");
    const int d = ctx->bb_d, rf = ctx->bb_rf, rp = ctx->bb_rp;
    if (rf == 8 && d == 7 && rp == 13) return fn.template operator()<7, 8, 13>();
    if (rf == 8 && d == 7 && rp == 22) return fn.template operator()<7, 8, 22>();
    if (rf == 8 && d == 5 && rp == 14) return fn.template operator()<5, 8, 14>();
    throw Error(P3G_EUNSUPPORTED, "BabyBear Poseidon2 schedule not built (supported: x^7 8+13, x^7 8+22, x^5 8+14)");
}
template <class Fn>
void dispatch_gl(const p3g_ctx* ctx, const Fn& fn) {
    if (!ctx->has_p2gl) throw Error(P3G_ESTATE, "Poseidon2 constants for Goldilocks are not set");
    const int d = ctx->gl_d, rf = ctx->gl_rf, rp = ctx->gl_rp;
    if (rf == 8 && d == 7 && rp == 22) return fn.template operator()<7, 8, 22>();
    throw Error(P3G_EUNSUPPORTED, "Goldilocks Poseidon2 schedule not built (supported: x^7 8+22)");
}

// Host launchers, explicitly instantiated once per schedule.
template <class H, int D, int RF, int RP>
struct Launch {
    using T = typename H::T;
    // persistent hashing of ngroups groups (work counter zeroed first)
    static void hash_groups(const typename H::Params& p, unsigned long long* counter, const HashGroup<T>* groups,
                            int ngroups, const HashEntry<T>* ents, uint64_t total_units, int sm_count,
                            cudaStream_t st);
    static void level(const typename H::Params& p, const T* child, uint64_t nchild, T* parent, uint64_t nparent,
                      const T* inj, cudaStream_t st);
    static void tail(const typename H::Params& p, const TailLevels<T>& t, cudaStream_t st);
    // BabyBear only: k_compress_coop on `blocks` CTAs (1 when t has several levels)
    static void coop(const typename H::Params& p, const TailLevels<T>& t, unsigned blocks, cudaStream_t st);
    static void permute(const typename H::Params& p, T* states, uint64_t n, cudaStream_t st);
    static void grind(const typename H::Params& p, const GrindArgs<T, H::W>* d_args, uint64_t base, uint64_t count,
                      unsigned long long* found, int sm_count, cudaStream_t st);
};

#ifdef P3G_MERKLE_INSTANTIATE
template <class H, int D, int RF, int RP>
void Launch<H, D, RF, RP>::hash_groups(const typename H::Params& p, unsigned long long* counter,
                                       const HashGroup<T>* groups, int ngroups, const HashEntry<T>* ents,
                                       uint64_t total_units, int sm_count, cudaStream_t st) {
    if (total_units == 0) return;
    // resident CTAs per SM (same for every device of one architecture); a
    // function-local static is initialised once even when several host
    // threads get here together
    static const int occ = [] {
        int o = 0;
        P3G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_hash_groups<H, D, RF, RP>, HASH_ROWS, 0));
        return o > 0 ? o : 1;
    }();
    const int grid = occ * sm_count;
    P3G_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
    const int blocks = int(std::min<uint64_t>(uint64_t(grid), total_units));
    k_hash_groups<H, D, RF, RP><<<blocks, HASH_ROWS, 0, st>>>(p, groups, ngroups, ents, total_units, counter);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class H, int D, int RF, int RP>
void Launch<H, D, RF, RP>::level(const typename H::Params& p, const T* child, uint64_t nchild, T* parent,
                                 uint64_t nparent, const T* inj, cudaStream_t st) {
    k_compress_level<H, D, RF, RP><<<unsigned((nparent + 127) / 128), 128, 0, st>>>(p, child, nchild, parent,
                                                                                     nparent, inj);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class H, int D, int RF, int RP>
void Launch<H, D, RF, RP>::grind(const typename H::Params& p, const GrindArgs<T, H::W>* d_args, uint64_t base,
                                 uint64_t count, unsigned long long* found, int sm_count, cudaStream_t st) {
    if (count == 0) return;
    static const int occ = [] {
        int o = 0;
        P3G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_grind<H, D, RF, RP>, 128, 0));
        return o > 0 ? o : 1;
    }();
    const uint64_t blocks = std::min<uint64_t>(uint64_t(occ) * sm_count, (count + 127) / 128);
    k_grind<H, D, RF, RP><<<unsigned(blocks), 128, 0, st>>>(p, d_args, base, count, found);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class H, int D, int RF, int RP>
void Launch<H, D, RF, RP>::tail(const typename H::Params& p, const TailLevels<T>& t, cudaStream_t st) {
    if (t.n == 0) return;
    k_compress_tail<H, D, RF, RP><<<1, TAIL_NODES, 0, st>>>(p, t);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
template <class H, int D, int RF, int RP>
void Launch<H, D, RF, RP>::coop(const typename H::Params& p, const TailLevels<T>& t, unsigned blocks, cudaStream_t st) {
    if constexpr (std::is_same<H, HBB>::value) {
        if (t.n == 0) return;
        k_compress_coop<D, RF, RP><<<blocks, COOP_THREADS, 0, st>>>(p, t);
        P3G_LAUNCHED();
        P3G_CUDA(cudaGetLastError());
    } else {
        throw Error(P3G_EUNSUPPORTED, "cooperative compression is BabyBear only");
    }
}
template <class H, int D, int RF, int RP>
void Launch<H, D, RF, RP>::permute(const typename H::Params& p, T* states, uint64_t n, cudaStream_t st) {
    if (n == 0) return;
    k_permute<H, D, RF, RP><<<unsigned((n + 127) / 128), 128, 0, st>>>(p, states, n);
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
}
#endif

}  // namespace p3g
