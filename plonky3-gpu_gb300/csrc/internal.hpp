// internal.hpp -- shared host/device declarations of libp3g_gb300 (not public).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "p3g.h"
#include "fields.cuh"

namespace p3g {

// ----------------------------------------------------------------- errors
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// Records the calling thread's last error message (read by p3g_last_error).
void set_last_error(const std::string& msg);

// Counts kernel launches (p3g_kernel_launches); every launch site calls
// P3G_LAUNCHED() right after the <<<>>> launch.
void count_launch();
#define P3G_LAUNCHED() ::p3g::count_launch()

#define P3G_CUDA(x)                                                                           \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) {                                                              \
            throw ::p3g::Error(e_ == cudaErrorMemoryAllocation ? P3G_ENOMEM : P3G_ECUDA,      \
                               std::string(#x) + ": " + cudaGetErrorString(e_));              \
        }                                                                                     \
    } while (0)

#define P3G_REQUIRE(cond, msg)                                  \
    do {                                                        \
        if (!(cond)) throw ::p3g::Error(P3G_EINVAL, (msg));     \
    } while (0)

// ----------------------------------------------------------------- roots
// Two-level table of powers of g = omega_{2^TWO_ADICITY} in const form:
// g^E = lo[E & (2^LB-1)] * hi[E >> LB].
template <class F>
struct RootTab {
    using T = typename F::T;
    static constexpr int LB = F::TWO_ADICITY == 27 ? 14 : 16;
    static constexpr uint64_t MASK = (uint64_t(1) << F::TWO_ADICITY) - 1;
    const T* lo;
    const T* hi;
    // g^E, E taken mod 2^TWO_ADICITY.
    __device__ __forceinline__ T pow(uint64_t e) const {
        e &= MASK;
        return F::cmul(lo[e & ((uint64_t(1) << LB) - 1)], hi[e >> LB]);
    }
    // omega_{2^k}^e (e may exceed 2^k; reduced mod the order)
    __device__ __forceinline__ T omega(int k, uint64_t e) const {
        return pow(e << (F::TWO_ADICITY - k));
    }
    __device__ __forceinline__ T omega_inv(int k, uint64_t e) const {
        return pow((uint64_t(0) - (e << (F::TWO_ADICITY - k))));
    }
};

// ----------------------------------------------------------------- Poseidon2 params
// Constants in the field's const form (BabyBear: Montgomery), passed to
// kernels by value so that they live in the constant bank.
struct P2BB16 {
    uint32_t initial[4][16];
    uint32_t terminal[4][16];
    uint32_t internal[32];
    uint32_t diag[16];  // 2^i in Montgomery form
};
struct P2GL8 {
    uint64_t initial[4][8];
    uint64_t terminal[4][8];
    uint64_t internal[32];
};

}  // namespace p3g

// ----------------------------------------------------------------- context
struct p3g_ctx {
    int device = 0;
    int sm_count = 0;
    cudaMemPool_t pool = nullptr;
    // root tables (device, const form)
    uint32_t* bb_lo = nullptr;
    uint32_t* bb_hi = nullptr;
    uint64_t* gl_lo = nullptr;
    uint64_t* gl_hi = nullptr;
    // prepared in-tile DFT twiddles (lde.cuh: build_dft_tw), device
    void* bb_dft_tw = nullptr;
    void* gl_dft_tw = nullptr;
    // Poseidon2
    bool has_p2bb = false, has_p2gl = false;
    int bb_rf = 0, bb_rp = 0, bb_d = 0;
    int gl_rf = 0, gl_rp = 0, gl_d = 0;
    p3g::P2BB16 p2bb{};
    p3g::P2GL8 p2gl{};

    // host-trace commits: a copy stream and events kept across calls (created on
    // first use; the context is used by one host thread at a time)
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> events;

    p3g::RootTab<p3g::FBB> bb_roots() const { return {bb_lo, bb_hi}; }
    p3g::RootTab<p3g::FGL> gl_roots() const { return {gl_lo, gl_hi}; }
    void* alloc(size_t bytes, cudaStream_t st);
    void release(void* p, cudaStream_t st);
};

struct p3g_tree {
    int field = 0;
    uint32_t digest = 8;
    std::vector<uint64_t> layer_size;
    std::vector<uint64_t> layer_off;  // in digests
    void* d_digests = nullptr;        // all layers, owned
    std::vector<p3g_matrix> mats;     // commit order
    std::vector<void*> owned;         // device buffers owned by the tree (LDEs)
    bool flat = false;                // commit_matrix tree (zero-padded odd layers)
    // prepared build (see tree_prepare): row-hash work descriptors and the
    // injected-row digest buffer of every layer that has one
    void* d_desc = nullptr;
    std::vector<void*> inj;           // per layer, nullptr when nothing is injected
    // Row hashing runs in stages, one launch each: a single stage, or for a
    // staged build one per commit-order matrix that completes some parts
    // (stage k may run once matrices 0..ready are written).
    struct HashStage {
        size_t ready;
        uint32_t job0, njobs;         // descriptor range
        uint64_t units;               // work units of the launch
    };
    std::vector<HashStage> stages;
    size_t stages_done = 0;
    size_t desc_ents_off = 0;         // byte offset of the entries in d_desc
    std::vector<void*> stage_bufs;    // sponge states between parts (staged builds)
    bool in_plan = false;             // owned by a plan; p3g_tree_free refuses it
    // Merkle-layer fusion (0 = the defaults of merkle.cu): levels of at most
    // tail_max nodes at the top of the tree run in one CTA, one after the
    // other; BabyBear levels of at most coop_max nodes use 16 lanes per node.
    uint64_t tail_max = 0, coop_max = 0;
};

namespace p3g {

// ----------------------------------------------------------------- entry points
// (implemented in lde.cu, merkle.cu, fold.cu; called by capi.cu)
void lde_bb(p3g_ctx* ctx, const uint32_t* in, int log_h, int w, int log_b, uint32_t shift,
            int bitrev_out, uint32_t* out, cudaStream_t st);
// TwoAdicFriPcs::open's opened values and reduced opening over a resident LDE (open.cu)
void pcs_open_values(p3g_ctx* ctx, const uint32_t* lde, int log_n, int w, int bitrev_rows, uint32_t shift,
                     const uint32_t* h_points, int m, uint32_t* h_out, cudaStream_t st);
void pcs_reduce(p3g_ctx* ctx, const uint32_t* lde, int log_n, int w, int bitrev_rows, uint32_t shift,
                const uint32_t* h_points, int m, const uint32_t* h_opened, const uint32_t* h_alpha, uint64_t alpha_pow,
                int q_bitrev, uint32_t* q, cudaStream_t st);
// prove_fri with the transcript on the device (fri.cu)
void fri_rounds(const uint32_t* log_heights, uint32_t n_inputs, const p3g_fri_params& prm, uint32_t* n_rounds,
                uint32_t* log_arities);
void fri_prove(p3g_ctx* ctx, const void* const* d_inputs, const uint32_t* log_heights, uint32_t n_inputs,
               const p3g_fri_params& prm, p3g_challenger* chal, uint32_t* h_commits, uint64_t* h_commit_witnesses,
               uint32_t* h_final_poly, uint64_t* h_query_witness, uint64_t* h_query_indices, uint32_t* h_rows,
               uint32_t* h_paths, cudaStream_t st);
// y += a * x over BabyBear^4 (fold.cu)
// (d_a: a in device memory instead, canonical)
void bb4_axpy(p3g_ctx* ctx, uint32_t* y, const uint32_t* x, uint64_t n, const uint32_t* a, cudaStream_t st,
              const uint32_t* d_a = nullptr);
// Batched LDEs (lde.cuh): traces that share (log_h, log_b, shift),
// 1 <= log_h <= 21, with bit-reversed rows, in one launch per pass.  The
// shape's three tables (sizes by lde_group_table_bytes_*, k = 0..2; 0 =
// unused) are filled once by lde_group_tables_*; each trace needs
// lde_group_scr_bytes_* of pass-1 scratch (0: none).
size_t lde_group_table_bytes_bb(int log_h, int log_b, int k);
size_t lde_group_table_bytes_gl(int log_h, int log_b, int k);
size_t lde_group_scr_bytes_bb(int log_h, int w);
size_t lde_group_scr_bytes_gl(int log_h, int w);
void lde_group_tables_bb(p3g_ctx* ctx, int log_h, int log_b, uint64_t shift, void* const* tab, cudaStream_t st);
void lde_group_tables_gl(p3g_ctx* ctx, int log_h, int log_b, uint64_t shift, void* const* tab, cudaStream_t st);
void lde_group_bb(p3g_ctx* ctx, int log_h, int log_b, const void* const* in, void* const* scr, void* const* out,
                  const uint32_t* w, size_t n, void* const* tab, cudaStream_t st);
void lde_group_gl(p3g_ctx* ctx, int log_h, int log_b, const void* const* in, void* const* scr, void* const* out,
                  const uint32_t* w, size_t n, void* const* tab, cudaStream_t st);
// The LDE stage of a batched commit (plan.cu): traces grouped by shape.
// Traces that share (log_h, log_b, shift) with 1 <= log_h <= 21 form one
// group, run as one batch; every other trace (log_h 0 or above 21) is a group
// of its own, run by lde_bb / lde_gl.
struct LdeGroup {
    int log_h = 0, log_b = 0;
    uint64_t shift = 0;
    bool batched = false;
    std::vector<size_t> idx;     // trace indices
    void* tab[3] = {nullptr, nullptr, nullptr};
    std::vector<void*> scr;      // per trace of idx
    uint64_t work = 0;           // LDE elements
};
std::vector<LdeGroup> lde_groups(const p3g_trace* traces, size_t n);
// Allocates a batched group's tables and scratch from the pool and fills the tables.
void lde_group_prepare(p3g_ctx* ctx, int field, LdeGroup& g, const p3g_trace* traces, cudaStream_t st);
// Enqueues the group's LDEs (bit-reversed rows): trace i reads in[i] and writes lde[i].
void lde_group_run(p3g_ctx* ctx, int field, const LdeGroup& g, const p3g_trace* traces, const void* const* in,
                   void* const* lde, cudaStream_t st);
void lde_group_release(p3g_ctx* ctx, LdeGroup& g, cudaStream_t st);
// device copies of the prepared DFT twiddle tables (cudaMalloc'd; the context frees them)
void* make_dft_tw_bb();
void* make_dft_tw_gl();
void lde_gl(p3g_ctx* ctx, const uint64_t* in, int log_h, int w, int log_b, uint64_t shift,
            int bitrev_out, uint64_t* out, cudaStream_t st);
// the coset LDE for 2^21 < h <= 2^26, called by lde_bb / lde_gl (dft_bb.cu, dft_gl.cu)
void lde_big(p3g_ctx* ctx, const uint32_t* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
             uint32_t* out, cudaStream_t st);
void lde_big(p3g_ctx* ctx, const uint64_t* in, int log_h, int w, int log_b, uint64_t shift, int bitrev_out,
             uint64_t* out, cudaStream_t st);
// dft / idft / coset_dft / coset_idft (kind = P3G_DFT_*)
void dft_bb(p3g_ctx* ctx, int kind, const uint32_t* in, int log_h, int w, uint32_t shift, int bitrev_out,
            uint32_t* out, cudaStream_t st);
void dft_gl(p3g_ctx* ctx, int kind, const uint64_t* in, int log_h, int w, uint64_t shift, int bitrev_out,
            uint64_t* out, cudaStream_t st);

void mmcs_build(p3g_ctx* ctx, p3g_tree* tree, unsigned cap_height, cudaStream_t st);
void flat_build(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st);
// Two-phase build: tree_prepare allocates every buffer of the tree and uploads
// its work descriptors (synchronously when `sync_upload`, e.g. before a graph
// capture); tree_enqueue only launches kernels on `st`.
void tree_prepare(p3g_ctx* ctx, p3g_tree* tree, unsigned cap_height, bool flat, cudaStream_t st, bool sync_upload,
                  bool staged = false);
void tree_enqueue(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st);
// Staged build (tree_prepare with staged = true) for callers that write the
// matrices one by one in commit order: after matrices 0..n_ready-1 are
// enqueued on `st`, tree_hash_ready hashes every row part they complete (a
// group's row is cut where its length so far is a multiple of the sponge
// rate, and the sponge state is carried across the cut); tree_finish hashes
// the rest and builds the levels.
void tree_hash_ready(p3g_ctx* ctx, p3g_tree* tree, size_t n_ready, cudaStream_t st);
void tree_finish(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st);
void tree_release(p3g_ctx* ctx, p3g_tree* tree, cudaStream_t st);
void permute_states(p3g_ctx* ctx, int field, void* d_states, size_t n, cudaStream_t st);
// DuplexChallenger::grind: smallest witness below `limit` (false if none)
bool grind(p3g_ctx* ctx, int field, const void* h_state, const void* h_input, uint32_t n_input, uint32_t bits,
           uint64_t limit, uint64_t* witness, cudaStream_t st);
void open_batch(p3g_ctx* ctx, const p3g_tree* tree, const uint64_t* h_idx, size_t nq,
                void* h_rows, void* h_proof, cudaStream_t st);
// open_batch with the indices, rows and proofs in device memory; no
// synchronisation.  Indices must be below the tree's leaf count.
void open_batch_dev(p3g_ctx* ctx, const p3g_tree* tree, const uint64_t* d_idx, size_t nq, void* d_rows,
                    void* d_proof, cudaStream_t st);
// The BabyBear proof-of-work search over [0, count) with its arguments in
// device memory (GrindArgs<uint32_t, 16> in internal form, merkle.cuh);
// *found must hold ~0 before.
void grind_bb_dev(p3g_ctx* ctx, const void* d_args, uint64_t count, unsigned long long* found, cudaStream_t st);

// (d_beta: beta in device memory instead, canonical)
void fold_bb4(p3g_ctx* ctx, const uint32_t* in, int log_height, int log_arity,
              const uint32_t beta[4], uint32_t* out, cudaStream_t st, const uint32_t* d_beta = nullptr);

inline int ceil_div(int64_t a, int64_t b) { return int((a + b - 1) / b); }

}  // namespace p3g
