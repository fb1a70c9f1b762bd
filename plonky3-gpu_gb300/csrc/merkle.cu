// merkle.cu -- Poseidon2 MerkleTreeMmcs commit on the GPU.
//
// Mixed-height tree, as the reference's build_merkle_tree
// (merkle_tree.hpp:84-185): matrices are stable-sorted by height (desc);
// leaf i = PaddingFreeSponge over the concatenation of row i of every tallest
// matrix (padding_free_sponge.hpp:63-113, overwrite absorb, a partial last
// chunk is permuted, empty input gives the zero digest); each level
// compresses pairs with TruncatedPermutation (truncated_permutation.hpp:61-76)
// and, where some matrices have the level's height, replaces node i by
// compress(node i, hash(row i of those matrices)); the tree stops at
// 2^cap_height nodes.
//
// One persistent kernel (k_hash_groups) hashes the rows of every height group
// -- the leaves and the rows injected at higher levels -- taking 256-row work
// units from an atomic queue, each row read straight from HBM by one thread
// with the Poseidon2 state in registers (no host-side concatenation); one
// kernel per level then compresses pairs and folds in that level's injected
// digests.  tree_prepare lays out the digest layers and uploads the work
// descriptors once, tree_enqueue only launches, so a plan can capture the
// launches in a graph and replay them.  All digest layers stay resident on the
// device for openings.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <type_traits>

#include "merkle.cuh"

namespace p3g {

extern template struct Launch<HBB, 7, 8, 13>;
extern template struct Launch<HBB, 7, 8, 22>;
extern template struct Launch<HBB, 5, 8, 14>;
extern template struct Launch<HGL, 7, 8, 22>;

// Opening: query q gathers row index/(max_h/h_i) of each matrix and the
// sibling digest of every layer below the top (merkle_tree_mmcs.hpp:120-152).
struct OpenMat {
    const void* ptr;
    uint64_t height;
    uint32_t width;
    uint32_t row_off;  // element offset in the query's row block
};
template <class T>
__global__ void k_open(const OpenMat* mats, int nmats, uint64_t max_h, const uint64_t* idx, const T* digests,
                       const uint64_t* layer_off, const uint64_t* layer_size, int nproof, int dig, int flat,
                       T* rows_out, uint32_t row_elems, T* proof_out) {
    const int q = blockIdx.x;
    const uint64_t index = idx[q];
    for (int m = 0; m < nmats; ++m) {
        const OpenMat om = mats[m];
        const uint64_t row = flat ? index : index / (max_h / om.height);
        const T* src = static_cast<const T*>(om.ptr) + row * om.width;
        for (uint32_t c = threadIdx.x; c < om.width; c += blockDim.x)
            rows_out[uint64_t(q) * row_elems + om.row_off + c] = src[c];
    }
    for (int l = threadIdx.x; l < nproof; l += blockDim.x) {
        const uint64_t sib = (index >> l) ^ 1;
        for (int e = 0; e < dig; ++e) {
            T v = 0;
            if (sib < layer_size[l]) v = digests[(layer_off[l] + sib) * dig + e];
            proof_out[(uint64_t(q) * nproof + l) * dig + e] = v;
        }
    }
}

template <class H>
struct HashFn {
    const typename H::Params* p;
    unsigned long long* counter;
    const HashGroup<typename H::T>* groups;
    int ngroups;
    const HashEntry<typename H::T>* ents;
    uint64_t units;
    int sm_count;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const {
        Launch<H, D, RF, RP>::hash_groups(*p, counter, groups, ngroups, ents, units, sm_count, st);
    }
};
template <class H>
struct LevelFn {
    const typename H::Params* p;
    const typename H::T* child;
    uint64_t nchild;
    typename H::T* parent;
    uint64_t npar;
    const typename H::T* inj;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const { Launch<H, D, RF, RP>::level(*p, child, nchild, parent, npar, inj, st); }
};
template <class H>
struct TailFn {
    const typename H::Params* p;
    const TailLevels<typename H::T>* t;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const { Launch<H, D, RF, RP>::tail(*p, *t, st); }
};
template <class H>
struct CoopFn {
    const typename H::Params* p;
    const TailLevels<typename H::T>* t;
    unsigned blocks;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const { Launch<H, D, RF, RP>::coop(*p, *t, blocks, st); }
};
template <class H>
struct PermFn {
    const typename H::Params* p;
    typename H::T* s;
    uint64_t n;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const { Launch<H, D, RF, RP>::permute(*p, s, n, st); }
};

// ------------------------------------------------------------------ tree build
template <class H>
static void prepare(p3g_ctx* ctx, p3g_tree* tree, unsigned cap_height, bool flat, cudaStream_t st,
                    bool sync_upload, bool staged) {
    using T = typename H::T;
    const auto& mats = tree->mats;
    const size_t n = mats.size();
    tree->digest = H::DIG;
    tree->flat = flat;
    std::vector<size_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return mats[a].height > mats[b].height; });
    const uint64_t max_h = mats[order[0]].height;
    // layer geometry (merkle_tree.hpp:145-179; flat: fri_merkle_tree_mmcs.hpp:77-92)
    tree->layer_size.assign(1, max_h);
    tree->layer_off.assign(1, 0);
    uint64_t total = max_h, sz = max_h;
    const uint64_t cap = uint64_t(1) << cap_height;
    while (flat ? sz > 1 : sz > cap) {
        sz = flat ? (sz + 1) / 2 : sz / 2;
        tree->layer_off.push_back(total);
        tree->layer_size.push_back(sz);
        total += sz;
    }
    if (!tree->d_digests) tree->d_digests = ctx->alloc(sizeof(T) * H::DIG * total, st);
    T* dig = static_cast<T*>(tree->d_digests);
    // equal-height groups: the tallest makes the leaves; each shorter group is
    // injected at the level whose size equals its height
    struct G {
        std::vector<size_t> idx;
        uint64_t rows;
        T* out;
    };
    std::vector<G> groups;
    size_t next = 0;
    auto collect = [&](uint64_t h) {
        std::vector<size_t> g;
        while (next < n && mats[order[next]].height == h) g.push_back(order[next++]);
        return g;
    };
    tree->inj.assign(tree->layer_size.size(), nullptr);
    groups.push_back({collect(max_h), max_h, dig});
    if (!flat) {
        for (size_t l = 1; l < tree->layer_size.size(); ++l) {
            auto gi = collect(tree->layer_size[l]);
            if (gi.empty()) continue;
            if (!tree->inj[l]) tree->inj[l] = ctx->alloc(sizeof(T) * H::DIG * tree->layer_size[l], st);
            groups.push_back({gi, tree->layer_size[l], static_cast<T*>(tree->inj[l])});
        }
    }
    // Jobs: one per group, or (staged) one per part of a group's row.  A part
    // ends where the row so far is a multiple of RATE long and the next matrix
    // has columns, so the sponge resumes there from the saved state; a part
    // can run once its last matrix (in commit order) is written.
    struct Job {
        std::vector<size_t> idx;
        uint64_t rows;
        T* out;
        uint64_t cost;  // permutations per row
        size_t ready;
        const T* sin;
        T* sout;
    };
    std::vector<Job> jobs;
    for (auto& g : groups) {
        std::vector<std::vector<size_t>> parts(1);
        uint64_t len = 0;
        for (size_t i : g.idx) {
            if (staged && len > 0 && len % H::RATE == 0 && mats[i].width > 0) parts.emplace_back();
            parts.back().push_back(i);
            len += mats[i].width;
        }
        T* bufs[2] = {nullptr, nullptr};  // states between parts, alternating
        for (size_t k = 0; k + 1 < parts.size() && k < 2; ++k) {
            bufs[k] = static_cast<T*>(ctx->alloc(sizeof(T) * H::W * g.rows, st));
            tree->stage_bufs.push_back(bufs[k]);
        }
        for (size_t k = 0; k < parts.size(); ++k) {
            Job jb{parts[k], g.rows, g.out, 0, staged ? *std::max_element(parts[k].begin(), parts[k].end()) : n - 1,
                   k > 0 ? bufs[(k - 1) % 2] : nullptr, k + 1 < parts.size() ? bufs[k % 2] : nullptr};
            uint64_t w = 0;
            for (size_t i : parts[k]) w += mats[i].width;
            jb.cost = (w + H::RATE - 1) / H::RATE;
            if (jb.idx.size() > size_t(MAXG)) throw Error(P3G_EUNSUPPORTED, "more than 64 matrices of one height");
            jobs.push_back(std::move(jb));
        }
    }
    // stages in commit order; within a stage the most expensive rows first,
    // so the queue drains with cheap units
    std::stable_sort(jobs.begin(), jobs.end(), [](const Job& a, const Job& b) {
        return a.ready != b.ready ? a.ready < b.ready : a.cost > b.cost;
    });
    std::vector<HashGroup<T>> hg;
    std::vector<HashEntry<T>> he;
    tree->stages.clear();
    tree->stages_done = 0;
    for (const auto& jb : jobs) {
        if (tree->stages.empty() || tree->stages.back().ready != jb.ready)
            tree->stages.push_back({jb.ready, uint32_t(hg.size()), 0, 0});
        auto& stg = tree->stages.back();
        if (stg.njobs == uint32_t(MAXG)) throw Error(P3G_EUNSUPPORTED, "more than 64 distinct matrix heights");
        HashGroup<T> d{};
        d.rows = jb.rows;
        d.unit0 = stg.units;
        d.out = jb.out;
        d.ent0 = uint32_t(he.size());
        d.nent = uint32_t(jb.idx.size());
        d.vec = 0;
        d.state_in = jb.sin;
        d.state_out = jb.sout;
        for (size_t i : jb.idx) he.push_back({static_cast<const T*>(mats[i].d_data), mats[i].width, 0});
        if (jb.idx.size() == 1 && sizeof(T) == 4 && mats[jb.idx[0]].width % 4 == 0 &&
            reinterpret_cast<uintptr_t>(mats[jb.idx[0]].d_data) % 16 == 0)
            d.vec = 1;
        hg.push_back(d);
        stg.njobs += 1;
        stg.units += (jb.rows + HASH_ROWS - 1) / HASH_ROWS;
    }
    tree->desc_ents_off = HASH_DESC_HEADER + (sizeof(HashGroup<T>) * hg.size() + 255) / 256 * 256;
    const size_t bytes = tree->desc_ents_off + sizeof(HashEntry<T>) * std::max<size_t>(he.size(), 1);
    std::vector<char> host(bytes, 0);
    std::memcpy(host.data() + HASH_DESC_HEADER, hg.data(), sizeof(HashGroup<T>) * hg.size());
    std::memcpy(host.data() + tree->desc_ents_off, he.data(), sizeof(HashEntry<T>) * he.size());
    if (!tree->d_desc) tree->d_desc = ctx->alloc(bytes, st);
    if (sync_upload) {
        P3G_CUDA(cudaStreamSynchronize(st));
        P3G_CUDA(cudaMemcpy(tree->d_desc, host.data(), bytes, cudaMemcpyHostToDevice));
    } else {
        // pageable source: the copy is staged before cudaMemcpyAsync returns
        P3G_CUDA(cudaMemcpyAsync(tree->d_desc, host.data(), bytes, cudaMemcpyHostToDevice, st));
    }
}

// Launches the row-hash stages [stages_done, end) whose matrices are all
// written (ready < n_ready).
template <class H>
static void hash_stages(p3g_ctx* ctx, p3g_tree* tree, const typename H::Params& p, size_t n_ready, cudaStream_t st) {
    using T = typename H::T;
    char* base = static_cast<char*>(tree->d_desc);
    auto* counter = reinterpret_cast<unsigned long long*>(base);
    auto* groups = reinterpret_cast<const HashGroup<T>*>(base + HASH_DESC_HEADER);
    auto* ents = reinterpret_cast<const HashEntry<T>*>(base + tree->desc_ents_off);
    for (; tree->stages_done < tree->stages.size() && tree->stages[tree->stages_done].ready < n_ready;
         ++tree->stages_done) {
        const auto& stg = tree->stages[tree->stages_done];
        HashFn<H> fn{&p, counter, groups + stg.job0, int(stg.njobs), ents, stg.units, ctx->sm_count, st};
        if constexpr (std::is_same<H, HBB>::value) dispatch_bb(ctx, fn);
        else dispatch_gl(ctx, fn);
    }
}

// Levels of many nodes: one launch each, one thread per node.  The small
// levels are latency-bound: BabyBear runs them with one 16-lane group per
// node (a launch per level up to COOP_MAX_NODES nodes, then one CTA for every
// level of at most COOP_TAIL_NODES), Goldilocks with one CTA for every level
// of at most TAIL_NODES.  A tree's tail_max / coop_max override the two
// thresholds (the batched commit's autotuner sets them).
template <class H>
static void levels(p3g_ctx* ctx, p3g_tree* tree, const typename H::Params& p, cudaStream_t st) {
    using T = typename H::T;
    constexpr bool BB = std::is_same<H, HBB>::value;
    T* dig = static_cast<T*>(tree->d_digests);
    const size_t nl = tree->layer_size.size();
    // the Goldilocks tail kernel covers at most TAIL_NODES nodes per level
    const uint64_t tail_max = tree->tail_max ? (BB ? tree->tail_max : std::min<uint64_t>(tree->tail_max, TAIL_NODES))
                                             : (BB ? COOP_TAIL_NODES : uint64_t(TAIL_NODES));
    const uint64_t coop_max = tree->coop_max ? tree->coop_max : COOP_MAX_NODES;
    size_t first_tail = nl;
    while (first_tail > 1 && tree->layer_size[first_tail - 1] <= tail_max &&
           nl - (first_tail - 1) <= size_t(TAIL_MAX_LEVELS))
        --first_tail;
    auto run = [&](const auto& fn) {
        if constexpr (BB) dispatch_bb(ctx, fn);
        else dispatch_gl(ctx, fn);
    };
    auto level = [&](size_t l) -> typename TailLevels<T>::Level {
        return {dig + tree->layer_off[l - 1] * H::DIG, dig + tree->layer_off[l] * H::DIG,
                static_cast<const T*>(tree->inj[l]), uint32_t(tree->layer_size[l - 1]), uint32_t(tree->layer_size[l])};
    };
    for (size_t l = 1; l < first_tail; ++l) {
        const uint64_t np = tree->layer_size[l];
        if (BB && np <= coop_max) {
            TailLevels<T> t{};
            t.lev[t.n++] = level(l);
            run(CoopFn<H>{&p, &t, unsigned((np * 16 + COOP_THREADS - 1) / COOP_THREADS), st});
        } else {
            run(LevelFn<H>{&p, dig + tree->layer_off[l - 1] * H::DIG, tree->layer_size[l - 1],
                           dig + tree->layer_off[l] * H::DIG, np, static_cast<const T*>(tree->inj[l]), st});
        }
    }
    if (first_tail < nl) {
        TailLevels<T> t{};
        for (size_t l = first_tail; l < nl; ++l) t.lev[t.n++] = level(l);
        if constexpr (BB) run(CoopFn<H>{&p, &t, 1u, st});
        else run(TailFn<H>{&p, &t, st});
    }
}

template <class H>
static void enqueue(p3g_ctx* ctx, p3g_tree* tree, const typename H::Params& p, cudaStream_t st) {
    tree->stages_done = 0;
    hash_stages<H>(ctx, tree, p, ~size_t(0), st);
    levels<H>(ctx, tree, p, st);
}

static void validate_tree(const p3g_tree* tree, bool flat) {
    P3G_REQUIRE(!tree->mats.empty(), "mmcs_commit: need at least one matrix");
    for (const auto& m : tree->mats) {
        if (!flat)
            P3G_REQUIRE(m.height > 0 && (m.height & (m.height - 1)) == 0,
                        "mmcs_commit: matrix height must be a power of two");
        P3G_REQUIRE(m.width == 0 || m.d_data != nullptr, "mmcs_commit: null matrix data");
    }
}

void tree_prepare(p3g_ctx* ctx, p3g_tree* tree, unsigned cap_height, bool flat, cudaStream_t st, bool sync_upload,
                  bool staged) {
    validate_tree(tree, flat);
    P3G_REQUIRE(cap_height < 63, "mmcs_commit: cap_height too large");
    if (tree->field == P3G_BABYBEAR) {
        if (!ctx->has_p2bb) throw Error(P3G_ESTATE, "Poseidon2 constants for BabyBear are not set");
        prepare<HBB>(ctx, tree, cap_height, flat, st, sync_upload, staged);
    } else {
        if (!ctx->has_p2gl) throw Error(P3G_ESTATE, "Poseidon2 constants for Goldilocks are not set");
        prepare<HGL>(ctx, tree, cap_height, flat, st, sync_upload, staged);
    }
}

static void release_stage_bufs(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st) {
    for (void* p : tree->stage_bufs) ctx->release(p, st);
    tree->stage_bufs.clear();
}

void tree_enqueue(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st) {
    if (tree->field == P3G_BABYBEAR) enqueue<HBB>(ctx, tree, ctx->p2bb, st);
    else enqueue<HGL>(ctx, tree, ctx->p2gl, st);
}

void tree_hash_ready(p3g_ctx* ctx, p3g_tree* tree, size_t n_ready, cudaStream_t st) {
    if (tree->field == P3G_BABYBEAR) hash_stages<HBB>(ctx, tree, ctx->p2bb, n_ready, st);
    else hash_stages<HGL>(ctx, tree, ctx->p2gl, n_ready, st);
}

void tree_finish(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st) {
    if (tree->field == P3G_BABYBEAR) {
        hash_stages<HBB>(ctx, tree, ctx->p2bb, ~size_t(0), st);
        levels<HBB>(ctx, tree, ctx->p2bb, st);
    } else {
        hash_stages<HGL>(ctx, tree, ctx->p2gl, ~size_t(0), st);
        levels<HGL>(ctx, tree, ctx->p2gl, st);
    }
    release_stage_bufs(ctx, tree, st);  // stream-ordered: after the last part that reads them
}

void tree_release(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st) {
    if (tree->d_digests) ctx->release(tree->d_digests, st);
    if (tree->d_desc) ctx->release(tree->d_desc, st);
    for (void* p : tree->inj) ctx->release(p, st);
    for (void* p : tree->owned) ctx->release(p, st);
    release_stage_bufs(ctx, tree, st);
    tree->d_digests = tree->d_desc = nullptr;
    tree->inj.clear();
    tree->owned.clear();
}

void mmcs_build(p3g_ctx* ctx, p3g_tree* tree, unsigned cap_height, cudaStream_t st) {
    tree_prepare(ctx, tree, cap_height, false, st, false);
    tree_enqueue(ctx, tree, st);
}

void flat_build(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st) {
    P3G_REQUIRE(tree->mats.size() == 1, "commit_matrix: one matrix");
    P3G_REQUIRE(tree->mats[0].height > 0 && tree->mats[0].width > 0, "commit_matrix: bad dimensions");
    tree_prepare(ctx, tree, 0, true, st, false);
    tree_enqueue(ctx, tree, st);
}

void permute_states(p3g_ctx* ctx, int field, void* d_states, size_t n, cudaStream_t st) {
    if (field == P3G_BABYBEAR)
        dispatch_bb(ctx, PermFn<HBB>{&ctx->p2bb, static_cast<uint32_t*>(d_states), n, st});
    else
        dispatch_gl(ctx, PermFn<HGL>{&ctx->p2gl, static_cast<uint64_t*>(d_states), n, st});
}

template <class H>
struct GrindFn {
    const typename H::Params* p;
    const GrindArgs<typename H::T, H::W>* a;  // device
    uint64_t base, count;
    unsigned long long* found;
    int sm_count;
    cudaStream_t st;
    template <int D, int RF, int RP>
    void operator()() const { Launch<H, D, RF, RP>::grind(*p, a, base, count, found, sm_count, st); }
};

template <class H>
static bool grind_impl(p3g_ctx* ctx, const typename H::Params* params, const typename H::T* h_state,
                       const typename H::T* h_input, uint32_t n_input, uint32_t bits, uint64_t limit,
                       uint64_t* witness, cudaStream_t st) {
    using T = typename H::T;
    GrindArgs<T, H::W> a{};
    for (int i = 0; i < H::W; ++i) a.state[i] = H::absorb(i < int(n_input) ? h_input[i] : h_state[i]);
    a.n_input = n_input;
    a.mask = bits == 64 ? ~uint64_t(0) : (uint64_t(1) << bits) - 1;
    // device block: [found (8 bytes) | arguments]
    char* blk = static_cast<char*>(ctx->alloc(256 + sizeof a, st));
    struct Release {
        p3g_ctx* c;
        void* p;
        cudaStream_t s;
        ~Release() { c->release(p, s); }
    } rel{ctx, blk, st};
    auto* found = reinterpret_cast<unsigned long long*>(blk);
    auto* d_args = reinterpret_cast<GrindArgs<T, H::W>*>(blk + 256);
    P3G_CUDA(cudaMemsetAsync(found, 0xFF, sizeof(unsigned long long), st));
    // pageable source: staged before the call returns
    P3G_CUDA(cudaMemcpyAsync(d_args, &a, sizeof a, cudaMemcpyHostToDevice, st));
    // Launches of at most 2^30 candidates (well under a second each); the
    // first is sized so that it holds a hit with probability 1 - e^-16.
    uint64_t chunk = uint64_t(1) << std::min(30u, std::max(20u, bits + 4));
    unsigned long long hit = ~0ull;
    for (uint64_t base = 0; base < limit; ) {
        const uint64_t count = std::min(chunk, limit - base);
        GrindFn<H> fn{params, d_args, base, count, found, ctx->sm_count, st};
        if constexpr (std::is_same<H, HBB>::value) dispatch_bb(ctx, fn);
        else dispatch_gl(ctx, fn);
        P3G_CUDA(cudaMemcpyAsync(&hit, found, sizeof hit, cudaMemcpyDeviceToHost, st));
        P3G_CUDA(cudaStreamSynchronize(st));
        if (hit != ~0ull) {
            *witness = hit;
            return true;
        }
        base += count;
        chunk = std::min(chunk * 2, uint64_t(1) << 30);
    }
    return false;
}

bool grind(p3g_ctx* ctx, int field, const void* h_state, const void* h_input, uint32_t n_input, uint32_t bits,
           uint64_t limit, uint64_t* witness, cudaStream_t st) {
    if (bits == 0) {  // every sample passes a zero-bit mask: the first candidate
        *witness = 0;
        return limit > 0;
    }
    if (field == P3G_BABYBEAR)
        return grind_impl<HBB>(ctx, &ctx->p2bb, static_cast<const uint32_t*>(h_state),
                               static_cast<const uint32_t*>(h_input), n_input, bits, limit, witness, st);
    return grind_impl<HGL>(ctx, &ctx->p2gl, static_cast<const uint64_t*>(h_state),
                           static_cast<const uint64_t*>(h_input), n_input, bits, limit, witness, st);
}

// Device descriptors of an opening: matrices and layer tables, uploaded from
// pageable memory (staged before the call returns).
static char* open_desc(p3g_ctx* ctx, const p3g_tree* tree, cudaStream_t st, uint32_t* row_elems, size_t* o_loff,
                       size_t* o_lsz) {
    std::vector<OpenMat> om(tree->mats.size());
    uint32_t re = 0;
    for (size_t i = 0; i < om.size(); ++i) {
        om[i] = {tree->mats[i].d_data, tree->mats[i].height, tree->mats[i].width, re};
        re += tree->mats[i].width;
    }
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) / 256 * 256; return o; };
    const size_t o_mats = take(sizeof(OpenMat) * om.size());
    *o_loff = take(8 * tree->layer_off.size());
    *o_lsz = take(8 * tree->layer_size.size());
    char* buf = static_cast<char*>(ctx->alloc(off, st));
    P3G_CUDA(cudaMemcpyAsync(buf + o_mats, om.data(), sizeof(OpenMat) * om.size(), cudaMemcpyHostToDevice, st));
    P3G_CUDA(cudaMemcpyAsync(buf + *o_loff, tree->layer_off.data(), 8 * tree->layer_off.size(), cudaMemcpyHostToDevice, st));
    P3G_CUDA(cudaMemcpyAsync(buf + *o_lsz, tree->layer_size.data(), 8 * tree->layer_size.size(), cudaMemcpyHostToDevice, st));
    *row_elems = re;
    return buf;
}

void open_batch_dev(p3g_ctx* ctx, const p3g_tree* tree, const uint64_t* d_idx, size_t nq, void* d_rows,
                    void* d_proof, cudaStream_t st) {
    if (nq == 0) return;
    const uint64_t max_h = tree->layer_size[0];
    const int nproof = int(tree->layer_size.size()) - 1;
    uint32_t row_elems = 0;
    size_t o_loff = 0, o_lsz = 0;
    char* buf = open_desc(ctx, tree, st, &row_elems, &o_loff, &o_lsz);
    const auto* mats = reinterpret_cast<const OpenMat*>(buf);
    const auto* loff = reinterpret_cast<const uint64_t*>(buf + o_loff);
    const auto* lsz = reinterpret_cast<const uint64_t*>(buf + o_lsz);
    if (tree->field == P3G_BABYBEAR)
        k_open<uint32_t><<<unsigned(nq), 128, 0, st>>>(mats, int(tree->mats.size()), max_h, d_idx,
                                                       static_cast<const uint32_t*>(tree->d_digests), loff, lsz, nproof,
                                                       int(tree->digest), tree->flat ? 1 : 0,
                                                       static_cast<uint32_t*>(d_rows), row_elems,
                                                       static_cast<uint32_t*>(d_proof));
    else
        k_open<uint64_t><<<unsigned(nq), 128, 0, st>>>(mats, int(tree->mats.size()), max_h, d_idx,
                                                       static_cast<const uint64_t*>(tree->d_digests), loff, lsz, nproof,
                                                       int(tree->digest), tree->flat ? 1 : 0,
                                                       static_cast<uint64_t*>(d_rows), row_elems,
                                                       static_cast<uint64_t*>(d_proof));
    P3G_LAUNCHED();
    P3G_CUDA(cudaGetLastError());
    ctx->release(buf, st);
}

void open_batch(p3g_ctx* ctx, const p3g_tree* tree, const uint64_t* h_idx, size_t nq, void* h_rows,
                void* h_proof, cudaStream_t st) {
    if (nq == 0) return;
    const size_t esz = tree->field == P3G_BABYBEAR ? 4 : 8;
    const uint64_t max_h = tree->layer_size[0];
    for (size_t q = 0; q < nq; ++q) P3G_REQUIRE(h_idx[q] < max_h, "open_batch: index out of range");
    uint32_t row_elems = 0;
    for (const auto& m : tree->mats) row_elems += m.width;
    const int nproof = int(tree->layer_size.size()) - 1;
    const size_t rows_bytes = esz * row_elems * nq;
    const size_t proof_bytes = esz * tree->digest * size_t(std::max(nproof, 0)) * nq;
    // one device staging block: indices, rows, proofs
    const size_t o_rows = (8 * nq + 255) / 256 * 256, o_proof = o_rows + (rows_bytes + 255) / 256 * 256;
    char* buf = static_cast<char*>(ctx->alloc(o_proof + std::max<size_t>(proof_bytes, 1), st));
    P3G_CUDA(cudaMemcpyAsync(buf, h_idx, 8 * nq, cudaMemcpyHostToDevice, st));
    open_batch_dev(ctx, tree, reinterpret_cast<const uint64_t*>(buf), nq, buf + o_rows, buf + o_proof, st);
    if (h_rows && rows_bytes) P3G_CUDA(cudaMemcpyAsync(h_rows, buf + o_rows, rows_bytes, cudaMemcpyDeviceToHost, st));
    if (h_proof && proof_bytes) P3G_CUDA(cudaMemcpyAsync(h_proof, buf + o_proof, proof_bytes, cudaMemcpyDeviceToHost, st));
    ctx->release(buf, st);
    P3G_CUDA(cudaStreamSynchronize(st));
}

void grind_bb_dev(p3g_ctx* ctx, const void* d_args, uint64_t count, unsigned long long* found, cudaStream_t st) {
    dispatch_bb(ctx, GrindFn<HBB>{&ctx->p2bb, static_cast<const GrindArgs<uint32_t, 16>*>(d_args), 0, count, found,
                                  ctx->sm_count, st});
}

}  // namespace p3g
