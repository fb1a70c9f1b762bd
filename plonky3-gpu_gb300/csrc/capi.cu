// capi.cu -- the extern "C" boundary of libp3g_gb300 (declared in include/p3g.h).
//
// Converts C++ exceptions into P3G_* status codes and a per-thread message,
// owns contexts (root-of-unity tables, Poseidon2 constants, a stream-ordered
// memory pool) and trees.  No entry point falls back to the CPU.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <new>
#include <string>

#include "internal.hpp"

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};

struct DeviceGuard {
    int prev = -1, want;
    explicit DeviceGuard(int d) : want(d) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != d) P3G_CUDA(cudaSetDevice(d));
    }
    ~DeviceGuard() {
        if (prev >= 0 && prev != want) cudaSetDevice(prev);
    }
};

inline cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }
}  // namespace

#define API_BEGIN try {
#define API_END                                           \
    }                                                     \
    catch (const p3g::Error& e) {                         \
        g_last_error = e.what();                          \
        return e.status;                                  \
    }                                                     \
    catch (const std::bad_alloc&) {                       \
        g_last_error = "host allocation failed";          \
        return P3G_ENOMEM;                                \
    }                                                     \
    catch (const std::exception& e) {                     \
        g_last_error = e.what();                          \
        return P3G_ECUDA;                                 \
    }                                                     \
    return P3G_OK;

namespace p3g {
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace p3g

void* p3g_ctx::alloc(size_t bytes, cudaStream_t st) {
    void* p = nullptr;
    P3G_CUDA(cudaMallocFromPoolAsync(&p, bytes ? bytes : 1, pool, st));
    return p;
}
void p3g_ctx::release(void* p, cudaStream_t st) {
    if (p) P3G_CUDA(cudaFreeAsync(p, st));
}

extern "C" {

int p3g_version(void) { return P3G_VERSION; }

const char* p3g_status_string(int s) {
    switch (s) {
        case P3G_OK: return "ok";
        case P3G_EINVAL: return "invalid argument";
        case P3G_ENOMEM: return "out of device memory";
        case P3G_ECUDA: return "CUDA error";
        case P3G_ETIMEOUT: return "timed out";
        case P3G_EUNSUPPORTED: return "unsupported";
        case P3G_ESTATE: return "missing set-up";
        case P3G_ENOTFOUND: return "not found";
        default: return "unknown status";
    }
}

uint64_t p3g_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

int p3g_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return P3G_EINVAL;
    size_t n = std::min(len - 1, g_last_error.size());
    std::memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
    return P3G_OK;
}

// Frees the context's device tables and pool (null members are skipped).
static void free_ctx_resources(p3g_ctx* ctx) {
    for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
    ctx->events.clear();
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    ctx->copy_stream = nullptr;
    cudaFree(ctx->bb_lo);
    cudaFree(ctx->bb_hi);
    cudaFree(ctx->gl_lo);
    cudaFree(ctx->gl_hi);
    cudaFree(ctx->bb_dft_tw);
    cudaFree(ctx->gl_dft_tw);
    ctx->bb_lo = ctx->bb_hi = nullptr;
    ctx->gl_lo = ctx->gl_hi = nullptr;
    ctx->bb_dft_tw = ctx->gl_dft_tw = nullptr;
    if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
    ctx->pool = nullptr;
}

int p3g_ctx_create(int device, p3g_ctx** out) {
    API_BEGIN
    P3G_REQUIRE(out != nullptr, "ctx_create: null output");
    int n = 0;
    P3G_CUDA(cudaGetDeviceCount(&n));
    P3G_REQUIRE(device >= 0 && device < n, "ctx_create: no such device");
    DeviceGuard g(device);
    auto ctx = std::make_unique<p3g_ctx>();
    ctx->device = device;
    try {
        P3G_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        P3G_CUDA(cudaMemPoolCreate(&ctx->pool, &props));
        uint64_t keep = ~uint64_t(0);
        P3G_CUDA(cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        // two-level root tables g^E = lo[E mod 2^LB] * hi[E >> LB] (const form)
        {
            using RB = p3g::RootTab<p3g::FBB>;
            const uint32_t g27 = p3g::bb::two_adic_generator(27);
            std::vector<uint32_t> lo(size_t(1) << RB::LB), hi(size_t(1) << (27 - RB::LB));
            uint32_t v = 1;
            for (auto& x : lo) { x = p3g::bb::to_mont(v); v = p3g::bb::h_mul(v, g27); }
            const uint32_t step = v;  // g^(2^LB)
            v = 1;
            for (auto& x : hi) { x = p3g::bb::to_mont(v); v = p3g::bb::h_mul(v, step); }
            P3G_CUDA(cudaMalloc(&ctx->bb_lo, lo.size() * 4));
            P3G_CUDA(cudaMalloc(&ctx->bb_hi, hi.size() * 4));
            P3G_CUDA(cudaMemcpy(ctx->bb_lo, lo.data(), lo.size() * 4, cudaMemcpyHostToDevice));
            P3G_CUDA(cudaMemcpy(ctx->bb_hi, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice));
        }
        {
            using RG = p3g::RootTab<p3g::FGL>;
            const uint64_t g32 = p3g::gl::two_adic_generator(32);
            std::vector<uint64_t> lo(size_t(1) << RG::LB), hi(size_t(1) << (32 - RG::LB));
            uint64_t v = 1;
            for (auto& x : lo) { x = v; v = p3g::gl::h_mul(v, g32); }
            const uint64_t step = v;
            v = 1;
            for (auto& x : hi) { x = v; v = p3g::gl::h_mul(v, step); }
            P3G_CUDA(cudaMalloc(&ctx->gl_lo, lo.size() * 8));
            P3G_CUDA(cudaMalloc(&ctx->gl_hi, hi.size() * 8));
            P3G_CUDA(cudaMemcpy(ctx->gl_lo, lo.data(), lo.size() * 8, cudaMemcpyHostToDevice));
            P3G_CUDA(cudaMemcpy(ctx->gl_hi, hi.data(), hi.size() * 8, cudaMemcpyHostToDevice));
        }
        ctx->bb_dft_tw = p3g::make_dft_tw_bb();
        ctx->gl_dft_tw = p3g::make_dft_tw_gl();
    } catch (...) {
        free_ctx_resources(ctx.get());  // whatever was created before the failure
        throw;
    }
    *out = ctx.release();
    API_END
}

int p3g_ctx_destroy(p3g_ctx* ctx) {
    API_BEGIN
    if (!ctx) return P3G_OK;
    {
        DeviceGuard g(ctx->device);
        cudaDeviceSynchronize();
        free_ctx_resources(ctx);
    }
    delete ctx;
    API_END
}

int p3g_stream_synchronize(p3g_ctx* ctx, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx, "null context");
    DeviceGuard g(ctx->device);
    P3G_CUDA(cudaStreamSynchronize(S(stream)));
    API_END
}

int p3g_ctx_memory(p3g_ctx* ctx, uint64_t* reserved, uint64_t* used, uint64_t* reserved_high, uint64_t* used_high) {
    API_BEGIN
    P3G_REQUIRE(ctx, "null context");
    DeviceGuard g(ctx->device);
    const struct {
        uint64_t* out;
        cudaMemPoolAttr attr;
    } q[] = {{reserved, cudaMemPoolAttrReservedMemCurrent},
             {used, cudaMemPoolAttrUsedMemCurrent},
             {reserved_high, cudaMemPoolAttrReservedMemHigh},
             {used_high, cudaMemPoolAttrUsedMemHigh}};
    for (const auto& e : q)
        if (e.out) {
            unsigned long long v = 0;  // the attribute is a cuuint64_t (64-bit unsigned)
            P3G_CUDA(cudaMemPoolGetAttribute(ctx->pool, e.attr, &v));
            *e.out = uint64_t(v);
        }
    API_END
}

int p3g_malloc(p3g_ctx* ctx, size_t bytes, void** d_ptr, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && d_ptr, "malloc: null argument");
    DeviceGuard g(ctx->device);
    *d_ptr = ctx->alloc(bytes, S(stream));
    API_END
}

int p3g_free(p3g_ctx* ctx, void* d_ptr, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx, "free: null context");
    DeviceGuard g(ctx->device);
    ctx->release(d_ptr, S(stream));
    API_END
}

int p3g_memcpy_h2d(p3g_ctx* ctx, void* d_dst, const void* h_src, size_t bytes, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && (bytes == 0 || (d_dst && h_src)), "memcpy_h2d: null argument");
    DeviceGuard g(ctx->device);
    if (bytes) P3G_CUDA(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, S(stream)));
    API_END
}

int p3g_memcpy_d2h(p3g_ctx* ctx, void* h_dst, const void* d_src, size_t bytes, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && (bytes == 0 || (h_dst && d_src)), "memcpy_d2h: null argument");
    DeviceGuard g(ctx->device);
    if (bytes) P3G_CUDA(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, S(stream)));
    P3G_CUDA(cudaStreamSynchronize(S(stream)));
    API_END
}

int p3g_set_poseidon2(p3g_ctx* ctx, int field, uint32_t width, uint32_t rounds_f, uint32_t rounds_p,
                      uint32_t sbox_degree, const void* h_initial, const void* h_terminal, const void* h_internal) {
    API_BEGIN
    P3G_REQUIRE(ctx && h_initial && h_terminal && (h_internal || rounds_p == 0), "set_poseidon2: null argument");
    P3G_REQUIRE(rounds_f % 2 == 0 && rounds_f <= 8, "set_poseidon2: rounds_f must be even and <= 8");
    P3G_REQUIRE(rounds_p <= 32, "set_poseidon2: rounds_p must be <= 32");
    P3G_REQUIRE(sbox_degree == 3 || sbox_degree == 5 || sbox_degree == 7, "set_poseidon2: degree must be 3, 5 or 7");
    const uint32_t half = rounds_f / 2;
    if (field == P3G_BABYBEAR) {
        P3G_REQUIRE(width == 16, "set_poseidon2: BabyBear width must be 16");
        const uint32_t* ini = static_cast<const uint32_t*>(h_initial);
        const uint32_t* ter = static_cast<const uint32_t*>(h_terminal);
        const uint32_t* inr = static_cast<const uint32_t*>(h_internal);
        p3g::P2BB16 p{};
        for (uint32_t r = 0; r < half; ++r)
            for (uint32_t i = 0; i < 16; ++i) {
                P3G_REQUIRE(ini[r * 16 + i] < p3g::bb::P && ter[r * 16 + i] < p3g::bb::P,
                            "set_poseidon2: constants must be canonical");
                p.initial[r][i] = p3g::bb::to_mont(ini[r * 16 + i]);
                p.terminal[r][i] = p3g::bb::to_mont(ter[r * 16 + i]);
            }
        for (uint32_t r = 0; r < rounds_p; ++r) {
            P3G_REQUIRE(inr[r] < p3g::bb::P, "set_poseidon2: constants must be canonical");
            p.internal[r] = p3g::bb::to_mont(inr[r]);
        }
        for (uint32_t i = 0; i < 16; ++i) p.diag[i] = p3g::bb::to_mont(uint32_t((1ull << i) % p3g::bb::P));
        ctx->p2bb = p;
        ctx->bb_rf = int(rounds_f);
        ctx->bb_rp = int(rounds_p);
        ctx->bb_d = int(sbox_degree);
        ctx->has_p2bb = true;
    } else if (field == P3G_GOLDILOCKS) {
        P3G_REQUIRE(width == 8, "set_poseidon2: Goldilocks width must be 8");
        const uint64_t* ini = static_cast<const uint64_t*>(h_initial);
        const uint64_t* ter = static_cast<const uint64_t*>(h_terminal);
        const uint64_t* inr = static_cast<const uint64_t*>(h_internal);
        p3g::P2GL8 p{};
        for (uint32_t r = 0; r < half; ++r)
            for (uint32_t i = 0; i < 8; ++i) {
                P3G_REQUIRE(ini[r * 8 + i] < p3g::gl::P && ter[r * 8 + i] < p3g::gl::P,
                            "set_poseidon2: constants must be canonical");
                p.initial[r][i] = ini[r * 8 + i];
                p.terminal[r][i] = ter[r * 8 + i];
            }
        for (uint32_t r = 0; r < rounds_p; ++r) {
            P3G_REQUIRE(inr[r] < p3g::gl::P, "set_poseidon2: constants must be canonical");
            p.internal[r] = inr[r];
        }
        ctx->p2gl = p;
        ctx->gl_rf = int(rounds_f);
        ctx->gl_rp = int(rounds_p);
        ctx->gl_d = int(sbox_degree);
        ctx->has_p2gl = true;
    } else {
        P3G_REQUIRE(false, "set_poseidon2: unknown field");
    }
    API_END
}

int p3g_poseidon2_permute(p3g_ctx* ctx, int field, void* d_states, size_t n, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && (n == 0 || d_states), "poseidon2_permute: null argument");
    P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "poseidon2_permute: unknown field");
    DeviceGuard g(ctx->device);
    p3g::permute_states(ctx, field, d_states, n, S(stream));
    API_END
}

int p3g_coset_lde(p3g_ctx* ctx, int field, const void* d_in, uint32_t log_h, uint32_t width, uint32_t log_blowup,
                  uint64_t shift, int bitrev_out, void* d_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && (width == 0 || (d_in && d_out)), "coset_lde: null argument");
    P3G_REQUIRE(width <= (1u << 24), "coset_lde: width too large");
    DeviceGuard g(ctx->device);
    if (field == P3G_BABYBEAR) {
        P3G_REQUIRE(shift < p3g::bb::P, "coset_lde: shift must be canonical");
        p3g::lde_bb(ctx, static_cast<const uint32_t*>(d_in), int(log_h), int(width), int(log_blowup),
                    uint32_t(shift), bitrev_out, static_cast<uint32_t*>(d_out), S(stream));
    } else if (field == P3G_GOLDILOCKS) {
        P3G_REQUIRE(shift < p3g::gl::P, "coset_lde: shift must be canonical");
        p3g::lde_gl(ctx, static_cast<const uint64_t*>(d_in), int(log_h), int(width), int(log_blowup), shift,
                    bitrev_out, static_cast<uint64_t*>(d_out), S(stream));
    } else {
        P3G_REQUIRE(false, "coset_lde: unknown field");
    }
    API_END
}

int p3g_dft(p3g_ctx* ctx, int field, int kind, const void* d_in, uint32_t log_h, uint32_t width, uint64_t shift,
            int bitrev_out, void* d_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && (width == 0 || (d_in && d_out)), "dft: null argument");
    P3G_REQUIRE(width <= (1u << 24), "dft: width too large");
    P3G_REQUIRE(kind >= P3G_DFT && kind <= P3G_COSET_IDFT, "dft: unknown kind");
    P3G_REQUIRE(width == 0 || d_in != d_out, "dft: in and out must not overlap");
    DeviceGuard g(ctx->device);
    if (field == P3G_BABYBEAR) {
        P3G_REQUIRE(shift < p3g::bb::P, "dft: shift must be canonical");
        p3g::dft_bb(ctx, kind, static_cast<const uint32_t*>(d_in), int(log_h), int(width), uint32_t(shift),
                    bitrev_out, static_cast<uint32_t*>(d_out), S(stream));
    } else if (field == P3G_GOLDILOCKS) {
        P3G_REQUIRE(shift < p3g::gl::P, "dft: shift must be canonical");
        p3g::dft_gl(ctx, kind, static_cast<const uint64_t*>(d_in), int(log_h), int(width), shift, bitrev_out,
                    static_cast<uint64_t*>(d_out), S(stream));
    } else {
        P3G_REQUIRE(false, "dft: unknown field");
    }
    API_END
}

static void copy_cap(const p3g_tree* t, void* h_out, cudaStream_t st) {
    if (!h_out) return;
    const size_t esz = t->field == P3G_BABYBEAR ? 4 : 8;
    const size_t last = t->layer_size.size() - 1;
    const char* src = static_cast<const char*>(t->d_digests) + t->layer_off[last] * t->digest * esz;
    P3G_CUDA(cudaMemcpyAsync(h_out, src, t->layer_size[last] * t->digest * esz, cudaMemcpyDeviceToHost, st));
    P3G_CUDA(cudaStreamSynchronize(st));
}

static void free_tree(p3g_ctx* ctx, p3g_tree* t, cudaStream_t st) {
    if (!t) return;
    p3g::tree_release(ctx, t, st);
    delete t;
}

int p3g_mmcs_commit(p3g_ctx* ctx, int field, const p3g_matrix* mats, size_t n_mats, uint32_t cap_height,
                    p3g_tree** tree_out, void* h_cap_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && mats && n_mats > 0 && tree_out, "mmcs_commit: null argument");
    P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "mmcs_commit: unknown field");
    DeviceGuard g(ctx->device);
    auto t = std::make_unique<p3g_tree>();
    t->field = field;
    t->mats.assign(mats, mats + n_mats);
    try {
        p3g::mmcs_build(ctx, t.get(), cap_height, S(stream));
        copy_cap(t.get(), h_cap_out, S(stream));
    } catch (...) {
        p3g::tree_release(ctx, t.get(), S(stream));
        throw;
    }
    *tree_out = t.release();
    API_END
}

int p3g_commit_matrix(p3g_ctx* ctx, int field, const void* d_flat, uint64_t height, uint32_t width,
                      p3g_tree** tree_out, void* h_root_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && d_flat && tree_out, "commit_matrix: null argument");
    P3G_REQUIRE(width > 0 && height > 0, "commit_matrix: bad dimensions");
    P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "commit_matrix: unknown field");
    DeviceGuard g(ctx->device);
    auto t = std::make_unique<p3g_tree>();
    t->field = field;
    t->mats.push_back(p3g_matrix{d_flat, height, width, 0});
    try {
        p3g::flat_build(ctx, t.get(), S(stream));
        copy_cap(t.get(), h_root_out, S(stream));
    } catch (...) {
        p3g::tree_release(ctx, t.get(), S(stream));
        throw;
    }
    *tree_out = t.release();
    API_END
}

int p3g_tree_info(const p3g_tree* tree, uint32_t* n_layers, uint64_t* h_layer_sizes, uint32_t* digest_elems) {
    API_BEGIN
    P3G_REQUIRE(tree, "tree_info: null tree");
    if (n_layers) *n_layers = uint32_t(tree->layer_size.size());
    if (h_layer_sizes)
        for (size_t i = 0; i < tree->layer_size.size() && i < 64; ++i) h_layer_sizes[i] = tree->layer_size[i];
    if (digest_elems) *digest_elems = tree->digest;
    API_END
}

int p3g_tree_layer_ptr(const p3g_tree* tree, uint32_t layer, const void** d_ptr) {
    API_BEGIN
    P3G_REQUIRE(tree && d_ptr && layer < tree->layer_size.size(), "tree_layer_ptr: bad argument");
    const size_t esz = tree->field == P3G_BABYBEAR ? 4 : 8;
    *d_ptr = static_cast<const char*>(tree->d_digests) + tree->layer_off[layer] * tree->digest * esz;
    API_END
}

int p3g_tree_leaf_ptr(const p3g_tree* tree, uint32_t i, const void** d_ptr) {
    API_BEGIN
    P3G_REQUIRE(tree && d_ptr && i < tree->mats.size(), "tree_leaf_ptr: bad argument");
    *d_ptr = tree->mats[i].d_data;
    API_END
}

int p3g_mmcs_open_batch(p3g_ctx* ctx, const p3g_tree* tree, const uint64_t* h_indices, size_t n_queries,
                        void* h_rows, void* h_proof, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && tree && (n_queries == 0 || h_indices), "open_batch: null argument");
    DeviceGuard g(ctx->device);
    p3g::open_batch(ctx, tree, h_indices, n_queries, h_rows, h_proof, S(stream));
    API_END
}

int p3g_tree_free(p3g_ctx* ctx, p3g_tree* tree, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx, "tree_free: null context");
    P3G_REQUIRE(!tree || !tree->in_plan, "tree_free: the tree belongs to a plan (p3g_plan_destroy frees it)");
    DeviceGuard g(ctx->device);
    free_tree(ctx, tree, S(stream));
    API_END
}

int p3g_commit_traces(p3g_ctx* ctx, int field, const p3g_trace* traces, size_t n_traces, uint32_t cap_height,
                      p3g_tree** tree_out, void* h_cap_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && traces && n_traces > 0 && tree_out, "commit_traces: null argument");
    P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "commit_traces: unknown field");
    DeviceGuard g(ctx->device);
    cudaStream_t st = S(stream);
    auto t = std::make_unique<p3g_tree>();
    t->field = field;
    const size_t esz = field == P3G_BABYBEAR ? 4 : 8;
    // traces of one shape run as one batch (one launch per LDE pass)
    std::vector<p3g::LdeGroup> groups;
    try {
        std::vector<const void*> in(n_traces);
        for (size_t i = 0; i < n_traces; ++i) {
            const p3g_trace& tr = traces[i];
            P3G_REQUIRE(tr.width == 0 || tr.d_trace, "commit_traces: null trace");
            P3G_REQUIRE(tr.shift < (field == P3G_BABYBEAR ? uint64_t(p3g::bb::P) : p3g::gl::P),
                        "commit_traces: shift must be canonical");
            P3G_REQUIRE(tr.log_h + tr.log_blowup <= (field == P3G_BABYBEAR ? 27u : 32u),
                        "commit_traces: log_h + log_blowup exceeds two-adicity");
            if (tr.log_h > 26) throw p3g::Error(P3G_EUNSUPPORTED, "commit_traces: log_h > 26 is not supported");
            P3G_REQUIRE(tr.shift % (field == P3G_BABYBEAR ? uint64_t(p3g::bb::P) : p3g::gl::P) != 0,
                        "commit_traces: shift must be non-zero");
            const uint64_t H = uint64_t(1) << (tr.log_h + tr.log_blowup);
            void* lde = ctx->alloc(esz * H * tr.width, st);
            t->owned.push_back(lde);
            t->mats.push_back(p3g_matrix{lde, H, tr.width, 0});
            in[i] = tr.d_trace;
        }
        groups = p3g::lde_groups(traces, n_traces);
        for (auto& gr : groups) {
            p3g::lde_group_prepare(ctx, field, gr, traces, st);
            p3g::lde_group_run(ctx, field, gr, traces, in.data(), t->owned.data(), st);
            p3g::lde_group_release(ctx, gr, st);
        }
        p3g::mmcs_build(ctx, t.get(), cap_height, st);
        copy_cap(t.get(), h_cap_out, st);
    } catch (...) {
        for (auto& gr : groups) p3g::lde_group_release(ctx, gr, st);
        p3g::tree_release(ctx, t.get(), st);
        throw;
    }
    *tree_out = t.release();
    API_END
}

int p3g_commit_traces_host(p3g_ctx* ctx, int field, const p3g_trace* traces, size_t n_traces, uint32_t cap_height,
                           p3g_tree** tree_out, void* h_cap_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && traces && n_traces > 0 && tree_out, "commit_traces_host: null argument");
    P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "commit_traces_host: unknown field");
    DeviceGuard g(ctx->device);
    cudaStream_t st = S(stream);
    const size_t esz = field == P3G_BABYBEAR ? 4 : 8;
    for (size_t i = 0; i < n_traces; ++i) {
        const p3g_trace& tr = traces[i];
        P3G_REQUIRE(tr.width == 0 || tr.d_trace, "commit_traces_host: null trace");
        P3G_REQUIRE(tr.shift < (field == P3G_BABYBEAR ? uint64_t(p3g::bb::P) : p3g::gl::P),
                    "commit_traces_host: shift must be canonical");
        if (tr.log_h > 26) throw p3g::Error(P3G_EUNSUPPORTED, "commit_traces_host: log_h > 26 is not supported");
    }
    // Column chunks.  512-byte chunk rows keep the strided copies at the
    // contiguous copy's bandwidth (narrower rows lose 15% at 256 bytes, half
    // at 128).  A large first trace starts with chunks of 1/4, 1/4 and 1/2 of
    // that, so that hashing starts after a short copy; every chunk width is a
    // multiple of the sponge rate, so each chunk's row hashes run as soon as
    // its LDE is written, resuming the sponge of the chunks before it.
    const uint32_t cw_max = uint32_t(512 / esz);
    struct Chunk {
        size_t trace;
        uint32_t c0, cw;
    };
    std::vector<Chunk> chunks;
    for (size_t i = 0; i < n_traces; ++i) {
        const p3g_trace& tr = traces[i];
        uint32_t c0 = 0;
        if (tr.width == 0) chunks.push_back({i, 0, 0});
        if (i == 0 && tr.log_h >= 14)
            for (uint32_t w : {cw_max / 4, cw_max / 4, cw_max / 2})
                if (c0 < tr.width) {
                    chunks.push_back({i, c0, std::min(w, tr.width - c0)});
                    c0 += chunks.back().cw;
                }
        for (; c0 < tr.width; c0 += cw_max) chunks.push_back({i, c0, std::min(cw_max, tr.width - c0)});
    }
    auto t = std::make_unique<p3g_tree>();
    t->field = field;
    // The context's copy stream and events, created once and reused: event 0
    // orders the copies after the caller's work, event 1 + k marks chunk k's copy.
    if (!ctx->copy_stream) P3G_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    while (ctx->events.size() < chunks.size() + 1) {
        cudaEvent_t e;
        P3G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->events.push_back(e);
    }
    cudaStream_t cs = ctx->copy_stream;
    cudaEvent_t start = ctx->events[0];
    // Device copies of the chunks, allocated on `st` before anything else is
    // queued (the pool then reuses them call after call on the same stream),
    // filled on the copy stream, handed back on `st` after each chunk's LDE.
    std::vector<void*> staged_in(chunks.size(), nullptr);
    try {
        for (const Chunk& c : chunks) {  // the tree's leaf matrices: every chunk's LDE, in order
            const uint64_t H = uint64_t(1) << (traces[c.trace].log_h + traces[c.trace].log_blowup);
            void* lde = ctx->alloc(std::max<size_t>(esz * H * c.cw, esz), st);
            t->owned.push_back(lde);
            t->mats.push_back(p3g_matrix{lde, H, c.cw, 0});
        }
        p3g::tree_prepare(ctx, t.get(), cap_height, false, st, false, /*staged=*/true);
        for (size_t k = 0; k < chunks.size(); ++k)
            if (chunks[k].cw > 0)
                staged_in[k] = ctx->alloc(esz * (uint64_t(1) << traces[chunks[k].trace].log_h) * chunks[k].cw, st);
        P3G_CUDA(cudaEventRecord(start, st));
        P3G_CUDA(cudaStreamWaitEvent(cs, start, 0));
        for (size_t k = 0; k < chunks.size(); ++k) {
            const Chunk& c = chunks[k];
            const p3g_trace& tr = traces[c.trace];
            if (c.cw > 0) {
                const uint64_t h = uint64_t(1) << tr.log_h;
                // copy stream: this chunk's columns into a contiguous h x cw buffer
                void* dev = staged_in[k];
                P3G_CUDA(cudaMemcpy2DAsync(dev, esz * c.cw, static_cast<const char*>(tr.d_trace) + esz * c.c0,
                                           esz * tr.width, esz * c.cw, h, cudaMemcpyHostToDevice, cs));
                cudaEvent_t ev = ctx->events[1 + k];
                P3G_CUDA(cudaEventRecord(ev, cs));
                // compute stream: the chunk's LDE as soon as its copy lands
                P3G_CUDA(cudaStreamWaitEvent(st, ev, 0));
                void* lde = t->owned[k];
                if (field == P3G_BABYBEAR)
                    p3g::lde_bb(ctx, static_cast<const uint32_t*>(dev), int(tr.log_h), int(c.cw), int(tr.log_blowup),
                                uint32_t(tr.shift), 1, static_cast<uint32_t*>(lde), st);
                else
                    p3g::lde_gl(ctx, static_cast<const uint64_t*>(dev), int(tr.log_h), int(c.cw), int(tr.log_blowup),
                                tr.shift, 1, static_cast<uint64_t*>(lde), st);
                ctx->release(dev, st);
                staged_in[k] = nullptr;
            }
            p3g::tree_hash_ready(ctx, t.get(), k + 1, st);  // the row parts this chunk completes
        }
        p3g::tree_finish(ctx, t.get(), st);
        copy_cap(t.get(), h_cap_out, st);
    } catch (...) {
        cudaStreamSynchronize(cs);
        for (void* p : staged_in)
            if (p) ctx->release(p, st);
        p3g::tree_release(ctx, t.get(), st);
        throw;
    }
    *tree_out = t.release();
    API_END
}

int p3g_bb4_axpy(p3g_ctx* ctx, void* d_y, const void* d_x, uint64_t n, const uint32_t h_a[4], void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && (n == 0 || (d_y && d_x)) && h_a, "bb4_axpy: null argument");
    DeviceGuard g(ctx->device);
    p3g::bb4_axpy(ctx, static_cast<uint32_t*>(d_y), static_cast<const uint32_t*>(d_x), n, h_a, S(stream));
    API_END
}

int p3g_grind(p3g_ctx* ctx, int field, const void* h_sponge_state, const void* h_input, uint32_t n_input,
              uint32_t bits, uint64_t max_witness, uint64_t* witness_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && h_sponge_state && witness_out && (n_input == 0 || h_input), "grind: null argument");
    P3G_REQUIRE(field == P3G_BABYBEAR || field == P3G_GOLDILOCKS, "grind: unknown field");
    const uint32_t width = field == P3G_BABYBEAR ? 16 : 8, rate = width / 2;
    P3G_REQUIRE(n_input < rate, "grind: more pending inputs than the challenger holds (n_input < RATE)");
    P3G_REQUIRE(bits < (field == P3G_BABYBEAR ? 31u : 64u), "grind: bits must be below the field's FIELD_BITS");
    if (field == P3G_BABYBEAR) {
        const auto* st = static_cast<const uint32_t*>(h_sponge_state);
        const auto* in = static_cast<const uint32_t*>(h_input);
        for (uint32_t i = 0; i < width; ++i) P3G_REQUIRE(st[i] < p3g::bb::P, "grind: sponge state not canonical");
        for (uint32_t i = 0; i < n_input; ++i) P3G_REQUIRE(in[i] < p3g::bb::P, "grind: input not canonical");
    }
    DeviceGuard g(ctx->device);
    const uint64_t limit = max_witness ? max_witness : ~uint64_t(0);
    if (!p3g::grind(ctx, field, h_sponge_state, h_input, n_input, bits, limit, witness_out, S(stream)))
        throw p3g::Error(P3G_ENOTFOUND, "grind: no witness below max_witness");
    API_END
}

int p3g_fri_rounds(const uint32_t* log_heights, uint32_t n_inputs, const p3g_fri_params* params, uint32_t* n_rounds,
                   uint32_t* log_arities) {
    API_BEGIN
    P3G_REQUIRE(log_heights && params && n_rounds, "fri_rounds: null argument");
    p3g::fri_rounds(log_heights, n_inputs, *params, n_rounds, log_arities);
    API_END
}

int p3g_fri_prove(p3g_ctx* ctx, const void* const* d_inputs, const uint32_t* log_heights, uint32_t n_inputs,
                  const p3g_fri_params* params, p3g_challenger* challenger, uint32_t* h_commits,
                  uint64_t* h_commit_witnesses, uint32_t* h_final_poly, uint64_t* h_query_witness,
                  uint64_t* h_query_indices, uint32_t* h_rows, uint32_t* h_paths, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && d_inputs && log_heights && params && challenger, "fri_prove: null argument");
    DeviceGuard g(ctx->device);
    p3g::fri_prove(ctx, d_inputs, log_heights, n_inputs, *params, challenger, h_commits, h_commit_witnesses,
                   h_final_poly, h_query_witness, h_query_indices, h_rows, h_paths, S(stream));
    API_END
}

int p3g_pcs_open_values(p3g_ctx* ctx, const void* d_lde, uint32_t log_n, uint32_t width, int bitrev_rows,
                        uint32_t shift, const uint32_t* h_points, uint32_t n_points, uint32_t* h_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && d_lde && h_points && h_out, "pcs_open_values: null argument");
    DeviceGuard g(ctx->device);
    p3g::pcs_open_values(ctx, static_cast<const uint32_t*>(d_lde), int(log_n), int(width), bitrev_rows, shift,
                         h_points, int(n_points), h_out, S(stream));
    API_END
}

int p3g_pcs_reduce(p3g_ctx* ctx, const void* d_lde, uint32_t log_n, uint32_t width, int bitrev_rows, uint32_t shift,
                   const uint32_t* h_points, uint32_t n_points, const uint32_t* h_opened, const uint32_t h_alpha[4],
                   uint64_t alpha_pow, int q_bitrev, void* d_q, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && d_lde && h_points && h_opened && h_alpha && d_q, "pcs_reduce: null argument");
    DeviceGuard g(ctx->device);
    p3g::pcs_reduce(ctx, static_cast<const uint32_t*>(d_lde), int(log_n), int(width), bitrev_rows, shift, h_points,
                    int(n_points), h_opened, h_alpha, alpha_pow, q_bitrev, static_cast<uint32_t*>(d_q), S(stream));
    API_END
}

int p3g_fold_matrix_bb4(p3g_ctx* ctx, const void* d_in, uint32_t log_height, uint32_t log_arity,
                        const uint32_t h_beta[4], void* d_out, void* stream) {
    API_BEGIN
    P3G_REQUIRE(ctx && d_in && d_out && h_beta, "fold_matrix: null argument");
    DeviceGuard g(ctx->device);
    p3g::fold_bb4(ctx, static_cast<const uint32_t*>(d_in), int(log_height), int(log_arity), h_beta,
                  static_cast<uint32_t*>(d_out), S(stream));
    API_END
}

}  // extern "C"
